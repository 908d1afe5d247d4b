"""Product code paths checked on the CPU against the oracle.

The BVH build (bvh_build.cpp) and the per-query traversal (collide_traverse.cuh,
the code the GPU kernel runs, FP32 filters and FP64 rechecks included) are compiled
for the host by tests/native and must reproduce the oracle bit for bit."""
import numpy as np
import pytest

from fcl_gb300 import workloads as W
from oracle import pyoracle as O
from tests import emul


@pytest.mark.parametrize("freq,seed", [(1, 0), (3, 1), (8, 2), (16, 3)])
def test_bvh_build_bit_exact(freq, seed):
    v, t = W.perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed)
    on, ofc = O.Mesh(v, t).nodes()
    en, efc, _ = emul.build(v, t)
    assert np.array_equal(ofc, efc)
    assert np.array_equal(on.view(np.uint64), en.view(np.uint64))


@pytest.mark.parametrize("freq,seed", [(32, 4), (56, 5)])
def test_bvh_build_bit_exact_parallel(freq, seed):
    """Meshes of 20,480 and 62,720 triangles: the upper levels are built as tasks on
    several host threads, with FCL's node ids fixed in advance; the tree is still the
    oracle's bit for bit."""
    v, t = W.perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed)
    on, ofc = O.Mesh(v, t).nodes()
    en, efc, _ = emul.build(v, t)
    assert np.array_equal(ofc, efc)
    assert np.array_equal(on.view(np.uint64), en.view(np.uint64))


def test_bvh_build_bit_exact_reference_meshes(golden):
    for k in ("env", "rob"):
        on, ofc = O.Mesh(golden[k + "_v"], golden[k + "_t"]).nodes()
        en, efc, _ = emul.build(golden[k + "_v"], golden[k + "_t"])
        assert np.array_equal(ofc, efc) and np.array_equal(on.view(np.uint64), en.view(np.uint64))


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("maxc", [1, 100000])
def test_traversal_matches_oracle_c0(prec, maxc):
    w = W.config0(n_poses=300)
    a = O.Mesh(*w.meshes[0]); b = O.Mesh(*w.meshes[1])
    oc, oct_, onbv, onl = O.collide_batch(a, b, w.tf2, num_max_contacts=maxc, nthreads=4)
    ec, ect, enbv, enl, enrc = emul.collide(prec, w.meshes[0], w.meshes[1], w.tf2, maxc)
    assert np.array_equal(oc, ec)
    assert np.array_equal(oct_, ect)          # same contacts in the same DFS order
    assert np.array_equal(onbv, enbv) and np.array_equal(onl, enl)
    if prec == 0:
        assert enrc.sum() == 0
    else:
        assert enrc.sum() <= 0.01 * (enbv.sum() + enl.sum())


@pytest.mark.parametrize("prec", [0, 1])
def test_traversal_matches_oracle_reference_fixture(golden, prec):
    env = (golden["env_v"], golden["env_t"]); rob = (golden["rob_v"], golden["rob_t"])
    a = O.Mesh(*env); b = O.Mesh(*rob)
    tf = golden["tf"]
    oc, oct_, onbv, onl = O.collide_batch(a, b, tf, num_max_contacts=1 << 30)
    ec, ect, enbv, enl, _ = emul.collide(prec, env, rob, tf, 1 << 30)
    assert np.array_equal(oc, ec) and np.array_equal(oct_, ect)
    assert np.array_equal(onbv, enbv) and np.array_equal(onl, enl)


def test_traversal_with_tf1_small_triangles():
    # dense meshes (small triangles relative to coordinates) stress the FP32 bounds
    w = W.config1(scale=0.005, n_pairs=2, tri_hi=60000, seed=5)
    for p in range(2):
        A = w.meshes[w.pairs[p, 0]]; B = w.meshes[w.pairs[p, 1]]
        tf2 = w.tf2[w.pair == p][:60]
        tf1 = W.random_poses(tf2.shape[0], -0.5, 0.5, 99 + p)
        a = O.Mesh(*A); b = O.Mesh(*B)
        oc, oct_, onbv, onl = O.collide_batch(a, b, tf2, tf1=tf1, num_max_contacts=100000, nthreads=4)
        ec, ect, enbv, enl, enrc = emul.collide(1, A, B, tf2, 100000, tf1=tf1)
        assert np.array_equal(oc, ec) and np.array_equal(oct_, ect)
        assert np.array_equal(onbv, enbv) and np.array_equal(onl, enl)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("budget", [3, 64, 1000])
def test_work_splitting_rebuilds_dfs_order(prec, budget):
    """Budgeted items + frontier re-queueing + item-tree assembly give the reference's
    contact list (same pairs, same DFS order) for any budget; statistics are equal
    whenever the num_max_contacts cap is not what stopped the traversal."""
    w = W.config0(n_poses=200, seed=8)
    a = O.Mesh(*w.meshes[0]); b = O.Mesh(*w.meshes[1])
    for maxc in (1, 7, 100000):
        oc, oct_, onbv, onl = O.collide_batch(a, b, w.tf2, num_max_contacts=maxc, nthreads=4)
        c, ct, nbv, nl, _ = emul.collide_split(prec, w.meshes[0], w.meshes[1], w.tf2, maxc, budget)
        assert np.array_equal(c, oc)
        assert np.array_equal(ct, oct_)
        uncapped = oc < maxc
        assert np.array_equal(nbv[uncapped], onbv[uncapped])
        assert np.array_equal(nl[uncapped], onl[uncapped])


def test_shape_pairs_bit_exact_vs_oracle():
    """The device GJK/EPA + closed-form code (shape_pair.cuh) built for the host gives
    the oracle's results bit for bit."""
    w = W.config3(n_pairs=6000, n_shapes=128, seed=21)
    e = emul.shape_batch(w.shapes, w.ia, w.ib, w.tf1, w.tf2)
    o = O.shape_batch(w.shapes, w.ia, w.ib, w.tf1, w.tf2, nthreads=4)
    assert np.array_equal(e["hit"], o["hit"]) and np.array_equal(e["status"], o["status"])
    for k in ("normal", "point", "depth", "dist", "p1", "p2"):
        assert np.array_equal(e[k], o[k]), k


@pytest.mark.parametrize("freq,seed", [(2, 0), (6, 1), (12, 2)])
def test_refit_bit_exact_vs_oracle(freq, seed):
    """BVHModel update + endUpdateModel() bottom-up refit: the device refit math (leaf
    fit over both frames, OBB/RSS sums) built for the host equals the oracle bit for bit,
    over two successive updates."""
    v, t = W.perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed)
    rng = np.random.default_rng(seed + 100)
    v1 = v + rng.normal(0, 0.03, v.shape)
    v2 = v1 @ W.random_poses(1, -0.5, 0.5, seed)[0][:, :3].T + 0.2
    o = O.Mesh(v, t)
    o.update(v1)
    o.update(v2)
    on, ofc = o.nodes()
    en, efc = emul.refit(v, t, [v1, v2])
    assert np.array_equal(ofc, efc)
    assert np.array_equal(on.view(np.uint64), en.view(np.uint64))


def test_replace_then_update_bit_exact_vs_oracle():
    """endReplaceModel() refits each leaf to its new triangle alone (fit3: FCL drops the
    previous frame); a later update uses the replaced vertices as its previous frame."""
    v, t = W.perturbed_ellipsoid(8, (1, 0.7, 0.5), 0.01, 0)
    rng = np.random.default_rng(1)
    f1 = v + rng.normal(0, 0.02, v.shape)
    f2 = f1 + rng.normal(0, 0.02, v.shape)
    f3 = f2 + rng.normal(0, 0.02, v.shape)
    o = O.Mesh(v, t)
    o.replace(f1)
    o.update(f2)
    o.replace(f3)
    on, ofc = o.nodes()
    en, efc = emul.refit(v, t, [f1, f2, f3], [1, 0, 1])
    assert np.array_equal(ofc, efc)
    assert np.array_equal(on.view(np.uint64), en.view(np.uint64))


def _cert_vs_oracle(a, b, tf2):
    oa, ob = O.Mesh(*a), O.Mesh(*b)
    od, oids, opts, _, _ = O.distance_batch(oa, ob, tf2, nearest=True, nthreads=4)
    ed, eids, epts, _, _, nrc = emul.distance_cert(a, b, tf2)
    return od, opts, ed, epts, nrc


@pytest.mark.parametrize("seed", [2, 5])
def test_certified_fp32_distance_equals_oracle_c0(seed):
    """The FP32 distance form (distance_traverse.cuh) run on the host: its distance is
    the smallest FP64 triDistance over all triangle pairs, so it equals FCL's, and the
    witness points are those of a pair at that distance (identical at shared vertices)."""
    w = W.config0(n_poses=200, seed=seed)
    od, opts, ed, epts, nrc = _cert_vs_oracle(w.meshes[0], w.meshes[1], w.tf2)
    assert np.array_equal(ed, od)
    sep = od > 0
    assert np.abs(epts[sep] - opts[sep]).max() <= 1e-12
    assert nrc.mean() < 40  # far fewer FP64 triangle distances than FCL's ~230 per query


def test_certified_fp32_distance_reference_fixture(golden):
    """FCL's env/rob fixture (coordinates up to 3,000) at its own poses and at random ones."""
    a = (golden["env_v"], golden["env_t"]); b = (golden["rob_v"], golden["rob_t"])
    tf = np.concatenate([golden["tf"], W.random_poses(60, -3000, 3000, 7)])
    od, opts, ed, epts, _ = _cert_vs_oracle(a, b, tf)
    assert np.array_equal(ed, od)
    sep = od > 0
    assert np.abs(epts[sep] - opts[sep]).max() <= 1e-12 * np.abs(opts).max()


def test_certified_fp32_distance_separated_pairs():
    w = W.config2(total_poses=900, n_pairs=3, tri_hi=30000, seed=4)
    for p in range(3):
        idx = np.nonzero(w.pair == p)[0][:100]
        a, b = w.meshes[w.pairs[p, 0]], w.meshes[w.pairs[p, 1]]
        od, opts, ed, epts, _ = _cert_vs_oracle(a, b, w.tf2[idx])
        assert np.array_equal(ed, od)
        assert np.abs(epts - opts).max() <= 1e-12


def test_mesh_shape_certified_bounds_hold():
    """The FP32 lower bounds of the warp mesh-shape distance (node: support gap of the
    shape against the node's RSS along two directions; triangle: the FP32 GJK
    certificate's gap) never exceed FCL's FP64 shapeTriangleDistance of the triangles
    below them (by more than m64), for every shape type, near and far poses and
    arbitrary directions -- the property that lets the kernel skip volumes and
    triangles.  Host build of the device functions."""
    import ctypes as C
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 41)
    shapes = W.random_shapes(48, 42)
    rng = np.random.default_rng(43)
    n = 160
    sidx = rng.integers(0, 48, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.2, 0.2, 44)
    tfs = W.random_poses(n, -1.6, 1.6, 45)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    chk, pos = C.c_int64(), C.c_int64()
    # the arrays are kept alive for the call
    arrs = [np.ascontiguousarray(a, dt) for a, dt in
            ((shapes.type, np.int32), (shapes.params, np.float64), (shapes.voff, np.int32), (shapes.vcnt, np.int32),
             (shapes.verts, np.float64), (v, np.float64), (t, np.int32), (sidx, np.int32), (tfm, np.float64),
             (tfs, np.float64), (dirs, np.float32))]
    ty, pa, vo, vc, sv, mv, mt, si, tm, ts, dr = [C.c_void_p(a.ctypes.data) for a in arrs]
    lib = emul.lib()
    lib.emu_ms_bounds.restype = C.c_int64
    bad = lib.emu_ms_bounds(C.c_int(48), ty, pa, vo, vc, sv, mv, C.c_int64(v.shape[0]), mt, C.c_int64(t.shape[0]),
                            C.c_int64(n), si, tm, ts, dr, C.byref(chk), C.byref(pos))
    assert bad == 0
    assert chk.value > 100000 and pos.value > chk.value // 10


def test_prepared_leaf_certificate_equals_per_call_form():
    """LeafCert32 (poses, relative rotations and the shape's supports rounded to FP32 once
    per pair, each triangle's vertices once) decides exactly as certified_disjoint, which
    rounds them on every support call: every (shape, triangle) pair of 60 posed shapes of
    every type against a 720-triangle mesh."""
    import ctypes as C
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 51)
    shapes = W.random_shapes(48, 52)
    rng = np.random.default_rng(53)
    n = 60
    sidx = rng.integers(0, 48, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.2, 0.2, 54)
    tfs = W.random_poses(n, -1.2, 1.2, 55)
    arrs = [np.ascontiguousarray(a, dt) for a, dt in
            ((shapes.type, np.int32), (shapes.params, np.float64), (shapes.voff, np.int32), (shapes.vcnt, np.int32),
             (shapes.verts, np.float64), (v, np.float64), (t, np.int32), (sidx, np.int32), (tfm, np.float64),
             (tfs, np.float64))]
    ty, pa, vo, vc, sv, mv, mt, si, tm, ts = [C.c_void_p(a.ctypes.data) for a in arrs]
    dis = C.c_int64()
    lib = emul.lib()
    lib.emu_leaf_cert.restype = C.c_int64
    diff = lib.emu_leaf_cert(C.c_int(48), ty, pa, vo, vc, sv, mv, C.c_int64(v.shape[0]), mt, C.c_int64(t.shape[0]),
                             C.c_int64(n), si, tm, ts, C.byref(dis))
    assert diff == 0
    assert 0 < dis.value < n * t.shape[0]


def test_intersecting_pair_rule_matches_oracle():
    """The warp mesh-shape distance's rule for a pair with an intersecting triangle --
    FCL's result is the first intersecting triangle in its depth-first order when every
    FP64 bound on that triangle's path is 0 and no triangle before it is at distance 0 --
    agrees with the oracle's traversal on every pair it applies to, and applies to most
    intersecting pairs (the rest run FCL's serial traversal)."""
    import ctypes as C
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 61)
    shapes = W.random_shapes(48, 62)
    rng = np.random.default_rng(63)
    n = 400
    sidx = rng.integers(0, 48, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.2, 0.2, 64)
    tfs = W.random_poses(n, -1.0, 1.0, 65)
    arrs = [np.ascontiguousarray(a, dt) for a, dt in
            ((shapes.type, np.int32), (shapes.params, np.float64), (shapes.voff, np.int32), (shapes.vcnt, np.int32),
             (shapes.verts, np.float64), (v, np.float64), (t, np.int32), (sidx, np.int32), (tfm, np.float64),
             (tfs, np.float64))]
    ty, pa, vo, vc, sv, mv, mt, si, tm, ts = [C.c_void_p(a.ctypes.data) for a in arrs]
    tri = np.empty(n, np.int32)
    dist = np.empty(n)
    emul.lib().emu_ms_contact_rule(C.c_int(48), ty, pa, vo, vc, sv, mv, C.c_int64(v.shape[0]), mt,
                                   C.c_int64(t.shape[0]), C.c_int64(n), si, tm, ts,
                                   C.c_void_p(tri.ctypes.data), C.c_void_p(dist.ctypes.data))
    o = O.mesh_shape_distance(O.Mesh(v, t), O.Geoms(shapes), sidx, tfm, tfs, nthreads=8)
    applies = tri >= 0
    np.testing.assert_array_equal(o["tri"][applies], tri[applies])
    np.testing.assert_array_equal(o["dist"][applies], dist[applies])
    neg = o["dist"] < 0
    assert neg.sum() > 50 and applies[neg].mean() > 0.9


def test_separated_pair_min_and_tie_rule_matches_oracle():
    """The warp mesh-shape distance's rule for a pair without an intersecting triangle --
    the smallest FP64 distance over all triangles, and of the triangles tied at it FCL's
    first (the seed triangle 0, else the side FCL enters first at their deepest common
    node) -- gives the oracle's distance and triangle.  Shapes just outside mesh vertices,
    so that many minima are shared by several triangles."""
    import ctypes as C
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 31)
    shapes = W.random_shapes(64, 32)
    rng = np.random.default_rng(33)
    n = 400
    spheres = np.flatnonzero(shapes.type == W.SPHERE)
    sidx = np.where(rng.uniform(size=n) < 0.6, rng.choice(spheres, size=n),
                    rng.integers(0, 64, size=n)).astype(np.int32)
    k = rng.integers(0, v.shape[0], size=n)
    u = v[k] - v.mean(axis=0)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    reach = np.where(shapes.type[sidx] == W.SPHERE, shapes.params[sidx, 0], 0.6)
    tfs = W.random_poses(n, 0.0, 0.0, 34)
    tfs[:, :, 3] = v[k] + u * (reach + rng.uniform(0.002, 0.3, size=n))[:, None]
    tfm = W.identity_poses(n)
    arrs = [np.ascontiguousarray(a, dt) for a, dt in
            ((shapes.type, np.int32), (shapes.params, np.float64), (shapes.voff, np.int32), (shapes.vcnt, np.int32),
             (shapes.verts, np.float64), (v, np.float64), (t, np.int32), (sidx, np.int32), (tfm, np.float64),
             (tfs, np.float64))]
    ty, pa, vo, vc, sv, mv, mt, si, tm, ts = [C.c_void_p(a.ctypes.data) for a in arrs]
    tri = np.empty(n, np.int32)
    dist = np.empty(n)
    ties = np.empty(n, np.int32)
    emul.lib().emu_ms_min_rule(C.c_int(64), ty, pa, vo, vc, sv, mv, C.c_int64(v.shape[0]), mt,
                               C.c_int64(t.shape[0]), C.c_int64(n), si, tm, ts, C.c_void_p(tri.ctypes.data),
                               C.c_void_p(dist.ctypes.data), C.c_void_p(ties.ctypes.data))
    o = O.mesh_shape_distance(O.Mesh(v, t), O.Geoms(shapes), sidx, tfm, tfs, nthreads=8)
    applies = tri >= 0
    assert applies.mean() > 0.9 and (ties[applies] > 1).sum() > 50
    np.testing.assert_array_equal(o["tri"][applies], tri[applies])
    np.testing.assert_array_equal(o["dist"][applies], dist[applies])
