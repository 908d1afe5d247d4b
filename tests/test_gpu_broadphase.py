"""Device broadphase (LBVH + narrowphase dispatch) against the oracle's dynamic AABB
tree manager with FCL's default callbacks."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _shape_scene(n, nq, seed, box=10.0, n_geoms=256):
    shapes = W.random_shapes(n_geoms, seed)
    rng = np.random.default_rng(seed + 1)
    refs = np.zeros((n, 2), np.int32)
    refs[:, 1] = rng.integers(0, n_geoms, size=n)
    tf = W.random_poses(n, 0.0, box, seed + 2)
    qrefs = np.zeros((nq, 2), np.int32)
    qrefs[:, 1] = rng.integers(0, n_geoms, size=nq)
    qtf = W.random_poses(nq, 0.0, box, seed + 3)
    return shapes, refs, tf, qrefs, qtf


def _check_collide(mgr, S, qrefs, qtf, gid_q, nq_checks=None):
    for M in (1, 100000):
        o = S.collide(gid_q, qtf, max_contacts=M, use_tree=True, nthreads=8)
        # FCL-like early stop and exhaustive evaluation report the same contact totals
        g = mgr.collide_batch(qrefs, qtf, num_max_contacts=M, exhaustive=False)
        np.testing.assert_array_equal(g["num_contacts"], o["num_contacts"])
        g = mgr.collide_batch(qrefs, qtf, num_max_contacts=M, exhaustive=True)
        np.testing.assert_array_equal(g["num_contacts"], o["num_contacts"])
        if M > 1:
            np.testing.assert_array_equal(g["num_objects"], o["num_hits"])
            segs = np.split(o["hits"], np.cumsum(o["num_hits"])[:-1])
            first = np.array([s.min() if s.size else -1 for s in segs])
            np.testing.assert_array_equal(g["first_object"], first)
    return g


def _check_distance(mgr, S, qrefs, qtf, gid_q):
    g = mgr.distance_batch(qrefs, qtf)
    o = S.distance(gid_q, qtf, use_tree=True, nthreads=8)
    np.testing.assert_array_equal(g["min_distance"] <= 0, o["dist"] <= 0)
    sep = o["dist"] > 0
    d, r = g["min_distance"][sep], o["dist"][sep]
    assert np.all(np.abs(d - r) <= np.maximum(REL * np.abs(r), ABS))
    same = g["object"][sep] == o["obj"][sep]
    assert same.mean() > 0.999
    pts_g = g["nearest_points"][sep][same]
    pts_o = o["pts"][sep][same]
    assert np.all(np.abs(pts_g - pts_o) <= REL * np.maximum(np.abs(pts_o), 1.0) + ABS)
    return g, o


def test_broadphase_shapes_match_oracle(gpu_lib):
    shapes, refs, tf, qrefs, qtf = _shape_scene(4000, 3000, 11, box=14.0)
    ss = api.ShapeSet.from_workload(shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(refs, tf)
    G = P.Geoms(shapes)
    S = P.Scene(G, refs[:, 1], tf)
    # CollisionObject::computeAABB, bit for bit
    np.testing.assert_array_equal(mgr.getAABBs(), G.world_aabbs(refs[:, 1], tf))
    g = _check_collide(mgr, S, qrefs, qtf, qrefs[:, 1])
    counts, _ = S.candidates(qrefs[:, 1], qtf)
    assert g["total_candidates"] == counts.sum()
    assert 0.2 < (g["num_contacts"] > 0).mean() < 0.99
    _check_distance(mgr, S, qrefs, qtf, qrefs[:, 1])


def test_broadphase_update_rebuilds(gpu_lib):
    shapes, refs, tf, qrefs, qtf = _shape_scene(1500, 800, 21)
    ss = api.ShapeSet.from_workload(shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(refs, tf)
    tf2 = W.random_poses(1500, 0.0, 10.0, 99)
    mgr.update(tf2)
    G = P.Geoms(shapes)
    S = P.Scene(G, refs[:, 1], tf2)
    np.testing.assert_array_equal(mgr.getAABBs(), G.world_aabbs(refs[:, 1], tf2))
    _check_collide(mgr, S, qrefs, qtf, qrefs[:, 1])
    _check_distance(mgr, S, qrefs, qtf, qrefs[:, 1])


def test_broadphase_meshes_match_oracle(gpu_lib):
    vt = [W.perturbed_ellipsoid(f, r, 0.01, k) for k, (f, r) in
          enumerate([(4, (0.6, 0.4, 0.3)), (6, (0.5, 0.5, 0.5)), (3, (0.8, 0.3, 0.3))])]
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in vt]
    om = [P.Mesh(v, t) for v, t in vt]
    rng = np.random.default_rng(5)
    n, nq = 120, 150
    refs = np.stack([np.ones(n, np.int32), rng.integers(0, 3, size=n).astype(np.int32)], 1)
    tf = W.random_poses(n, 0.0, 5.0, 6)
    qrefs = np.stack([np.ones(nq, np.int32), rng.integers(0, 3, size=nq).astype(np.int32)], 1)
    qtf = W.random_poses(nq, 0.0, 5.0, 7)
    mgr = api.DynamicAABBTreeCollisionManager(None, meshes)
    mgr.registerObjects(refs, tf)
    G = P.Geoms(None, om)
    S = P.Scene(G, refs[:, 1], tf)
    np.testing.assert_array_equal(mgr.getAABBs(), G.world_aabbs(refs[:, 1], tf))
    g = _check_collide(mgr, S, qrefs, qtf, qrefs[:, 1])
    assert (g["num_contacts"] > 0).any()
    _check_distance(mgr, S, qrefs, qtf, qrefs[:, 1])


def test_broadphase_small_and_device_paths(gpu_lib):
    import torch
    shapes, refs, tf, qrefs, qtf = _shape_scene(1, 64, 31, box=1.0)
    ss = api.ShapeSet.from_workload(shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(refs, tf)  # a single object: the root is a leaf
    G = P.Geoms(shapes)
    S = P.Scene(G, refs[:, 1], tf)
    _check_collide(mgr, S, qrefs, qtf, qrefs[:, 1])
    _check_distance(mgr, S, qrefs, qtf, qrefs[:, 1])
    # no queries
    out = mgr.collide_batch(qrefs[:0], qtf[:0])
    assert out["num_contacts"].shape == (0,)
    # the device entry points return what the host ones do
    shapes, refs, tf, qrefs, qtf = _shape_scene(2000, 500, 32)
    ss = api.ShapeSet.from_workload(shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(refs, tf)
    h = mgr.collide_batch(qrefs, qtf, num_max_contacts=100000)
    dq = torch.from_numpy(qrefs).cuda()
    dt = torch.from_numpy(np.ascontiguousarray(qtf)).cuda()
    d = mgr.collide_batch(dq, dt, num_max_contacts=100000)
    torch.cuda.synchronize()
    for k in ("num_contacts", "num_objects", "first_object"):
        np.testing.assert_array_equal(d[k].cpu().numpy(), h[k])
    hd = mgr.distance_batch(qrefs, qtf)
    dd = mgr.distance_batch(dq, dt)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dd["min_distance"].cpu().numpy(), hd["min_distance"])


def test_broadphase_rejects_bad_refs(gpu_lib):
    from fcl_gb300.native import FclGpuError
    shapes, refs, tf, qrefs, qtf = _shape_scene(100, 10, 41)
    ss = api.ShapeSet.from_workload(shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(refs, tf)
    bad = qrefs.copy()
    bad[3] = (0, 10 ** 6)
    with pytest.raises(FclGpuError):
        mgr.collide_batch(bad, qtf)


def _mixed_scene(seed=41, n=500, nq=300, box=7.0):
    """Shapes and meshes in the scene and among the queries (every pair kind)."""
    shapes = W.random_shapes(64, seed)
    vt = [W.perturbed_ellipsoid(f, r, 0.01, seed + 10 + k) for k, (f, r) in
          enumerate([(5, (0.6, 0.4, 0.3)), (7, (0.5, 0.5, 0.5)), (4, (0.8, 0.3, 0.3))])]
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in vt]
    om = [P.Mesh(v, t) for v, t in vt]
    ss = api.ShapeSet.from_workload(shapes)
    rng = np.random.default_rng(seed + 1)

    def refs_of(k):
        kind = (rng.uniform(size=k) < 0.35).astype(np.int32)
        return np.stack([kind, np.where(kind == 1, rng.integers(0, 3, size=k), rng.integers(0, 64, size=k))],
                        1).astype(np.int32)

    refs, qrefs = refs_of(n), refs_of(nq)
    tf = W.random_poses(n, 0.0, box, seed + 2)
    qtf = W.random_poses(nq, 0.0, box, seed + 3)
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(refs, tf)
    G = P.Geoms(shapes, om)
    gid = np.where(refs[:, 0] == 1, 64 + refs[:, 1], refs[:, 1]).astype(np.int32)
    qgid = np.where(qrefs[:, 0] == 1, 64 + qrefs[:, 1], qrefs[:, 1]).astype(np.int32)
    return mgr, P.Scene(G, gid, tf), refs, tf, qrefs, qtf, qgid


@pytest.mark.parametrize("M", [1, 3, 100000])
def test_broadphase_contact_lists_match_oracle(gpu_lib, M):
    """Per query every (object, b1, b2) DefaultCollisionFunction records, objects in
    index order, each pair's contacts in FCL's narrowphase order, capped per pair."""
    mgr, S, refs, tf, qrefs, qtf, qgid = _mixed_scene()
    g = mgr.collide_contacts(qrefs, qtf, num_max_contacts=M)
    c, trip = S.collide_lists(qgid, qtf, max_per_pair=M, nthreads=8)
    np.testing.assert_array_equal(g["counts"], c)
    np.testing.assert_array_equal(g["contacts"], trip)
    kinds = set(map(int, refs[trip[:, 0], 0]))
    assert kinds == {0, 1} and (trip[:, 1] >= 0).any() and (trip[:, 2] >= 0).any()
    # FCL's numContacts() is min(num_max_contacts, the query's list length)
    o = S.collide(qgid, qtf, max_contacts=M, use_tree=True, nthreads=8)
    np.testing.assert_array_equal(np.minimum(g["counts"], M), o["num_contacts"])


def test_broadphase_self_collide_matches_oracle(gpu_lib):
    """manager.collide(cdata, DefaultCollisionFunction): every overlapping pair (o1 < o2)
    once; lists equal the oracle's, and the total is FCL's naive manager numContacts()."""
    mgr, S, refs, tf, qrefs, qtf, qgid = _mixed_scene(seed=43, n=700)
    for M in (1, 100000):
        g = mgr.collide_contacts(None, None, num_max_contacts=M)
        c, trip = S.self_collide_lists(max_per_pair=M)
        np.testing.assert_array_equal(g["counts"], c)
        np.testing.assert_array_equal(g["contacts"], trip)
    assert g["counts"].sum() > 10
    assert S.self_collide_count(1 << 40) == g["counts"].sum()
    assert S.self_collide_count(1) == min(1, int(g["counts"].sum()))
    # the FCL-style entry point appends Contact(o1, o2, b1, b2) up to num_max_contacts
    res = api.CollisionResult()
    n = mgr.collide(None, api.CollisionRequest(num_max_contacts=5), res)
    assert n == min(5, int(g["counts"].sum()))
    o2 = np.repeat(np.arange(mgr.size()), g["counts"])
    assert [(ct.o1, ct.o2, ct.b1, ct.b2) for ct in res.contacts] == \
        [(int(a), int(q), int(b), int(d)) for (a, b, d), q in zip(g["contacts"][:5], o2[:5])]


def test_broadphase_self_distance_matches_oracle(gpu_lib):
    """manager.distance(cdata, DefaultDistanceFunction): the nearest pair of scene objects."""
    for seed, n, box in ((45, 300, 30.0), (47, 300, 60.0)):  # some pair in contact
        mgr, S, *_ = _mixed_scene(seed=seed, n=n, box=box)
        assert S.self_distance()["min_distance"] <= 0 and mgr.self_distance()["min_distance"] <= 0
    # separated scenes: nearest pair mesh-shape, shape-shape, mesh-shape
    for seed, n, box in ((45, 200, 60.0), (47, 200, 80.0), (51, 150, 60.0)):
        mgr, S, *_ = _mixed_scene(seed=seed, n=n, box=box)
        g = mgr.self_distance()
        o = S.self_distance()
        assert o["min_distance"] > 0
        assert abs(g["min_distance"] - o["min_distance"]) <= max(REL * o["min_distance"], ABS)
        assert (g["o1"], g["o2"]) == (o["o1"], o["o2"])
        assert (g["b1"], g["b2"]) == (o["b1"], o["b2"])
        assert np.all(np.abs(g["nearest_points"] - o["nearest_points"]) <= REL * np.maximum(
            np.abs(o["nearest_points"]), 1.0) + ABS)
        r = api.DistanceResult()
        mgr.distance(None, api.DistanceRequest(enable_nearest_points=True), r)
        assert r.min_distance == g["min_distance"] and (r.o1, r.o2) == (g["o1"], g["o2"])


def test_broadphase_manager_against_manager(gpu_lib):
    """collide(other_manager, ...): every object of the other manager against this scene."""
    mgr, S, refs, tf, qrefs, qtf, qgid = _mixed_scene(seed=49)
    other = api.DynamicAABBTreeCollisionManager(mgr.shapes, mgr.meshes)
    other.registerObjects(qrefs, qtf)
    res = api.CollisionResult()
    total = mgr.collide(other, api.CollisionRequest(num_max_contacts=1 << 30), res)
    c, trip = S.collide_lists(qgid, qtf, max_per_pair=1 << 30, nthreads=8)
    assert total == c.sum() > 0
    q = np.repeat(np.arange(qgid.shape[0]), c)
    assert [(ct.o1, ct.o2, ct.b1, ct.b2) for ct in res.contacts] == \
        [(int(a), int(b), int(d), int(e)) for (a, d, e), b in zip(trip, q)]


def test_distance_values_without_witnesses(gpu_lib):
    """Distances asked for without ids or nearest points (the motion server's clearance
    pass): the mesh-shape pairs take their values from one warp per pair; the minimum
    distances and nearest objects equal the full call's."""
    shapes = W.random_shapes(64, 71)
    vt = [W.perturbed_ellipsoid(f, r, 0.01, 72 + k) for k, (f, r) in
          enumerate([(5, (0.6, 0.4, 0.3)), (7, (0.5, 0.5, 0.5)), (4, (0.8, 0.3, 0.3))])]
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in vt]
    ss = api.ShapeSet.from_workload(shapes)
    rng = np.random.default_rng(73)
    n, nq = 800, 600
    kind = (rng.uniform(size=n) < 0.4).astype(np.int32)
    refs = np.stack([kind, np.where(kind == 1, rng.integers(0, 3, size=n), rng.integers(0, 64, size=n))], 1)
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(refs.astype(np.int32), W.random_poses(n, 0.0, 16.0, 74))
    qk = (rng.uniform(size=nq) < 0.5).astype(np.int32)
    qrefs = np.stack([qk, np.where(qk == 1, rng.integers(0, 3, size=nq), rng.integers(0, 64, size=nq))], 1)
    qtf = W.random_poses(nq, 0.0, 16.0, 75)
    full = mgr.distance_batch(qrefs.astype(np.int32), qtf)
    vals = mgr.distance_batch(qrefs.astype(np.int32), qtf, witnesses=False)
    assert np.array_equal(vals["min_distance"], full["min_distance"])
    assert np.array_equal(vals["object"], full["object"])
    assert (full["min_distance"] > 0).sum() > 100
