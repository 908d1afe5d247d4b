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
