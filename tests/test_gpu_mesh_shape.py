"""Device BVHModel<OBBRSS> x convex shape (collide and distance) against the FP64
oracle: same traversal (identical statistics), same results."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu


def _setup(seed, n=3000):
    vt = [W.perturbed_ellipsoid(f, r, 0.01, seed + k) for k, (f, r) in
          enumerate([(6, (0.8, 0.6, 0.5)), (10, (0.5, 0.9, 0.4))])]
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in vt]
    om = [P.Mesh(v, t) for v, t in vt]
    shapes = W.random_shapes(64, seed + 5)
    ss = api.ShapeSet.from_workload(shapes)
    G = P.Geoms(shapes)
    rng = np.random.default_rng(seed)
    midx = rng.integers(0, 2, size=n).astype(np.int32)
    sidx = rng.integers(0, 64, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.3, 0.3, seed + 1)
    tfs = W.random_poses(n, -1.3, 1.3, seed + 2)
    return meshes, om, ss, G, midx, sidx, tfm, tfs


@pytest.mark.parametrize("seed", [0, 1])
def test_mesh_shape_collide_matches_oracle(gpu_lib, seed):
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(seed)
    for M in (1, 100000):
        g = api.mesh_shape_batch(meshes, ss, midx, sidx, tfm, tfs, mode="collide", num_max_contacts=M,
                                 statistics=True)
        for k in range(2):
            sel = midx == k
            c, nbv, nleaf = P.mesh_shape_collide(om[k], G, sidx[sel], tfm[sel], tfs[sel], max_contacts=M,
                                                 nthreads=8)
            np.testing.assert_array_equal(g["counts"][sel], c)
            np.testing.assert_array_equal(g["num_bv_tests"][sel], nbv)
            np.testing.assert_array_equal(g["num_leaf_tests"][sel], nleaf)
    assert 0.1 < (g["counts"] > 0).mean() < 0.9


@pytest.mark.parametrize("seed", [0, 1])
def test_mesh_shape_distance_matches_oracle(gpu_lib, seed):
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(seed, n=2000)
    g = api.mesh_shape_batch(meshes, ss, midx, sidx, tfm, tfs, mode="distance", statistics=True)
    for k in range(2):
        sel = midx == k
        o = P.mesh_shape_distance(om[k], G, sidx[sel], tfm[sel], tfs[sel], nthreads=8)
        # same FP64 operations in the same order: identical values, triangles, witnesses
        np.testing.assert_array_equal(g["min_distance"][sel], o["dist"])
        np.testing.assert_array_equal(g["tri"][sel], o["tri"])
        np.testing.assert_array_equal(g["nearest_points"][sel], o["pts"])
        np.testing.assert_array_equal(g["num_bv_tests"][sel], o["nbv"])


def test_broadphase_mixed_scene_matches_oracle(gpu_lib):
    shapes = W.random_shapes(64, 21)
    vt = [W.perturbed_ellipsoid(f, r, 0.01, 30 + k) for k, (f, r) in
          enumerate([(5, (0.6, 0.4, 0.3)), (7, (0.5, 0.5, 0.5)), (4, (0.8, 0.3, 0.3))])]
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in vt]
    om = [P.Mesh(v, t) for v, t in vt]
    ss = api.ShapeSet.from_workload(shapes)
    rng = np.random.default_rng(22)
    n, nq = 600, 400
    kind = (rng.uniform(size=n) < 0.3).astype(np.int32)
    refs = np.stack([kind, np.where(kind == 1, rng.integers(0, 3, size=n), rng.integers(0, 64, size=n))], 1)
    refs = refs.astype(np.int32)
    tf = W.random_poses(n, 0.0, 8.0, 23)
    qk = (rng.uniform(size=nq) < 0.5).astype(np.int32)
    qrefs = np.stack([qk, np.where(qk == 1, rng.integers(0, 3, size=nq), rng.integers(0, 64, size=nq))], 1)
    qrefs = qrefs.astype(np.int32)
    qtf = W.random_poses(nq, 0.0, 8.0, 24)
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(refs, tf)
    G = P.Geoms(shapes, om)
    gid = np.where(refs[:, 0] == 1, 64 + refs[:, 1], refs[:, 1]).astype(np.int32)
    qgid = np.where(qrefs[:, 0] == 1, 64 + qrefs[:, 1], qrefs[:, 1]).astype(np.int32)
    # twice: the second time after moving every object (the scene objects' shape BVs are
    # kept between calls and must be refitted after an update)
    for rep in range(2):
        if rep == 1:
            tf = W.random_poses(n, 0.0, 8.0, 25)
            mgr.update(tf)
        S = P.Scene(G, gid, tf)
        np.testing.assert_array_equal(mgr.getAABBs(), G.world_aabbs(gid, tf))
        for M in (1, 100000):
            o = S.collide(qgid, qtf, max_contacts=M, use_tree=True, nthreads=8)
            for ex in (False, True):
                g = mgr.collide_batch(qrefs, qtf, num_max_contacts=M, exhaustive=ex)
                np.testing.assert_array_equal(g["num_contacts"], o["num_contacts"])
        assert (g["num_contacts"] > 0).any()
        d = mgr.distance_batch(qrefs, qtf)
        o = S.distance(qgid, qtf, use_tree=True, nthreads=8)
        np.testing.assert_array_equal(d["min_distance"] <= 0, o["dist"] <= 0)
        sep = o["dist"] > 0
        r = o["dist"][sep]
        assert np.all(np.abs(d["min_distance"][sep] - r) <= np.maximum(1e-6 * np.abs(r), 1e-9))


def test_mesh_shape_distance_ties_and_refit_match_oracle(gpu_lib):
    """Shapes just outside mesh vertices: spheres there are nearest to a vertex shared by
    several triangles, whose FP64 distances tie exactly, and FCL reports the first of
    them in its traversal order.  Then the same poses after a vertex update (refitted
    volumes).  Distance, triangle and witness points equal the oracle's."""
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 31)
    mesh, om = api.BVHModel.from_arrays(v, t), P.Mesh(v, t)
    shapes = W.random_shapes(64, 32)
    ss, G = api.ShapeSet.from_workload(shapes), P.Geoms(shapes)
    rng = np.random.default_rng(33)
    n = 1500
    spheres = np.flatnonzero(shapes.type == W.SPHERE)
    sidx = np.where(rng.uniform(size=n) < 0.7, rng.choice(spheres, size=n),
                    rng.integers(0, 64, size=n)).astype(np.int32)
    k = rng.integers(0, v.shape[0], size=n)
    u = v[k] - v.mean(axis=0)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    reach = np.where(shapes.type[sidx] == W.SPHERE, shapes.params[sidx, 0], 0.6)
    tfs = W.random_poses(n, 0.0, 0.0, 34)
    tfs[:, :, 3] = v[k] + u * (reach + rng.uniform(0.002, 0.3, size=n))[:, None]
    tfm = W.identity_poses(n)
    midx = np.zeros(n, np.int32)
    for step in range(2):
        g = api.mesh_shape_batch([mesh], ss, midx, sidx, tfm, tfs, mode="distance")
        o = P.mesh_shape_distance(om, G, sidx, tfm, tfs, nthreads=8)
        np.testing.assert_array_equal(g["min_distance"], o["dist"])
        np.testing.assert_array_equal(g["tri"], o["tri"])
        np.testing.assert_array_equal(g["nearest_points"], o["pts"])
        assert (o["dist"] > 0).mean() > 0.8
        v1 = v + rng.normal(0, 0.004, v.shape)
        mesh.update_vertices(v1)
        om.update(v1)


@pytest.mark.parametrize("seed", [2])
def test_mesh_shape_split_form_matches_oracle(gpu_lib, seed):
    # without statistics the leaf tests run one per thread; results stay the oracle's
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(seed, n=2500)
    for M in (1, 100000):
        g = api.mesh_shape_batch(meshes, ss, midx, sidx, tfm, tfs, mode="collide", num_max_contacts=M)
        for k in range(2):
            sel = midx == k
            c, _, _ = P.mesh_shape_collide(om[k], G, sidx[sel], tfm[sel], tfs[sel], max_contacts=M, nthreads=8)
            np.testing.assert_array_equal(g["counts"][sel], c)
    g = api.mesh_shape_batch(meshes, ss, midx, sidx, tfm, tfs, mode="distance")
    for k in range(2):
        sel = midx == k
        o = P.mesh_shape_distance(om[k], G, sidx[sel], tfm[sel], tfs[sel], nthreads=8)
        np.testing.assert_array_equal(g["min_distance"][sel], o["dist"])
        np.testing.assert_array_equal(g["tri"][sel], o["tri"])
        np.testing.assert_array_equal(g["nearest_points"][sel], o["pts"])


@pytest.mark.parametrize("seed", [0, 1])
def test_mesh_shape_contact_lists_match_oracle(gpu_lib, seed):
    """Mesh-shape collide with the contact list: the triangles FCL records as
    Contact(mesh, shape, triangle, NONE), in the order its traversal adds them, at caps
    1, 7 and 100,000 (exhaustive)."""
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(seed, n=2000)
    for M in (1, 7, 100000):
        g = api.mesh_shape_contacts_batch(meshes, ss, midx, sidx, tfm, tfs, num_max_contacts=M)
        assert np.array_equal(np.diff(g["offsets"]), g["counts"])
        for k in range(2):
            sel = np.nonzero(midx == k)[0]
            c, tris = P.mesh_shape_contacts(om[k], G, sidx[sel], tfm[sel], tfs[sel], max_contacts=M, nthreads=8)
            np.testing.assert_array_equal(g["counts"][sel], c)
            got = np.concatenate([g["tris"][g["offsets"][q]:g["offsets"][q + 1]] for q in sel])
            np.testing.assert_array_equal(got, tris)
        assert g["counts"].max() > (1 if M > 1 else 0)


def test_mesh_shape_contact_list_capacity(gpu_lib):
    """A tris buffer smaller than the total returns FCLGPU_ERR_CAPACITY with the total,
    counts and offsets set, and leaves the buffer untouched."""
    import ctypes as C
    from fcl_gb300 import native as N
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(3, n=500)
    full = api.mesh_shape_contacts_batch(meshes, ss, midx, sidx, tfm, tfs, num_max_contacts=100000)
    total = int(full["offsets"][-1])
    assert total > 4
    counts = np.zeros(500, np.int32); offsets = np.zeros(501, np.int64); tris = np.full(4, -7, np.int32)
    res = N.MeshShapeContactsResult(counts.ctypes.data, offsets.ctypes.data, tris.ctypes.data, 4, 0)
    hs = (C.c_void_p * 2)(*[m.handle.value for m in meshes])
    m_, s_ = np.ascontiguousarray(midx), np.ascontiguousarray(sidx)
    rc = N.lib().fclgpu_mesh_shape_contacts(hs, 2, ss.handle, 500, m_.ctypes.data, s_.ctypes.data,
                                            np.ascontiguousarray(tfm).ctypes.data,
                                            np.ascontiguousarray(tfs).ctypes.data, 100000, C.byref(res), None)
    assert rc == N.FCLGPU_ERR_CAPACITY and res.total_contacts == total
    assert np.array_equal(counts, full["counts"]) and np.array_equal(offsets, full["offsets"])
    assert (tris == -7).all()


@pytest.mark.parametrize("seed", [0, 1])
def test_mesh_shape_contact_geometry_matches_oracle(gpu_lib, seed):
    """enable_contact: the same triangle list, and per contact the point, normal and depth
    FCL's leaf records (sphereTriangleIntersect for spheres, GJK + EPA otherwise),
    bit-identical to the oracle's FP64 restatement."""
    meshes, om, ss, G, midx, sidx, tfm, tfs = _setup(seed, n=1500)
    for M in (1, 100000):
        plain = api.mesh_shape_contacts_batch(meshes, ss, midx, sidx, tfm, tfs, num_max_contacts=M)
        g = api.mesh_shape_contacts_batch(meshes, ss, midx, sidx, tfm, tfs, num_max_contacts=M, enable_contact=True)
        np.testing.assert_array_equal(g["tris"], plain["tris"])
        np.testing.assert_array_equal(g["offsets"], plain["offsets"])
        pair = np.repeat(np.arange(len(midx)), g["counts"])
        assert len(pair) > 50
        for k in range(2):
            sel = midx[pair] == k
            o = P.mesh_shape_contact_geometry(om[k], G, sidx[pair[sel]], tfm[pair[sel]], tfs[pair[sel]],
                                              g["tris"][sel])
            assert o["ok"].all()
            np.testing.assert_array_equal(g["pos"][sel], o["pos"])
            np.testing.assert_array_equal(g["normal"][sel], o["normal"])
            np.testing.assert_array_equal(g["penetration_depth"][sel], o["depth"])
        assert np.all(g["penetration_depth"] <= 0)
        assert np.allclose(np.linalg.norm(g["normal"], axis=1), 1.0)
