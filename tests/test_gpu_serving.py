"""The motion-checking request loop: per-request results against the oracle's broadphase
managers, and the same result alone as in a mix of concurrent requests."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _expected(S, robot, poses):
    """First colliding waypoint and clearance from per-query oracle results."""
    K, L = poses.shape[:2]
    qg = np.tile(robot.link_refs[:, 1], K).astype(np.int32)
    tf = poses.reshape(K * L, 12)
    c = S.collide(qg, tf, max_contacts=1, use_tree=True, nthreads=8)
    d = S.distance(qg, tf, use_tree=True, nthreads=8)
    hit = (c["num_contacts"].reshape(K, L) > 0).any(1)
    first = int(np.argmax(hit)) if hit.any() else -1
    dist = d["dist"].reshape(K, L)
    k, i = np.unravel_index(np.argmin(dist), dist.shape)  # first minimum in (waypoint, link) order
    return first, float(dist[k, i]), int(k), int(i)


def test_serving_matches_oracle_alone_and_in_mix(gpu_lib):
    w = W.scene4(n_objects=3000, seed=4, box=12.0, n_shape_geoms=256, mesh_fraction=0.0, mesh_links=False)
    ss = api.ShapeSet.from_workload(w.shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(w.refs, w.tf)
    reqs = W.motion_requests(w, 10, seed=6, k_lo=10, k_hi=60)
    srv = api.MotionServer(mgr, w.robot, max_waypoints_per_step=64)
    G = P.Geoms(w.shapes)
    S = P.Scene(G, w.refs[:, 1], w.tf)
    # link poses: the loop's forward kinematics agrees with the numpy definition
    poses = [srv.link_poses(r.base, r.q) for r in reqs]
    for r, p in zip(reqs, poses):
        np.testing.assert_allclose(p, W.robot_fk(w.robot, r.base, r.q), rtol=0, atol=1e-12)
    exp = [_expected(S, w.robot, p) for p in poses]
    # all requests in flight together (chunks of different requests share steps)
    ids = [srv.submit(r.base, r.q) for r in reqs]
    mix = [srv.wait(i) for i in ids]
    assert srv.stats()["steps"] < sum(r.q.shape[0] for r in reqs) / 8
    for (first, clr, k, i), got in zip(exp, mix):
        assert got["first_colliding_waypoint"] == first
        if clr > 0:
            assert abs(got["min_clearance"] - clr) <= max(REL * abs(clr), ABS)
            assert (got["clearance_waypoint"], got["clearance_link"]) == (k, i)
        else:
            assert got["min_clearance"] <= 0
    assert any(e[0] >= 0 for e in exp) and any(e[0] < 0 for e in exp)
    # each request alone returns what it returned in the mix
    for r, m in zip(reqs[:4], mix[:4]):
        alone = srv.wait(srv.submit(r.base, r.q))
        for key in ("first_colliding_waypoint", "min_clearance", "clearance_waypoint", "clearance_link",
                    "clearance_object"):
            assert alone[key] == m[key], key
    srv.close()


def test_serving_with_mesh_links_and_mesh_objects(gpu_lib):
    # the full request shape: capsule and 2,000-triangle mesh links against a scene of
    # primitives and perturbed icospheres (mesh-mesh, mesh-shape and shape-shape pairs)
    w = W.scene4(n_objects=800, seed=8, box=8.0, n_shape_geoms=128, n_mesh_geoms=6, mesh_fraction=0.25,
                 tri_lo=500, tri_hi=1500)
    ss = api.ShapeSet.from_workload(w.shapes)
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(w.refs, w.tf)
    reqs = W.motion_requests(w, 5, seed=9, k_lo=10, k_hi=25)
    srv = api.MotionServer(mgr, w.robot, max_waypoints_per_step=32)
    om = [P.Mesh(v, t) for v, t in w.meshes]
    G = P.Geoms(w.shapes, om)
    ns = w.shapes.n
    gid = np.where(w.refs[:, 0] == 1, ns + w.refs[:, 1], w.refs[:, 1]).astype(np.int32)
    S = P.Scene(G, gid, w.tf)
    link_gid = np.where(w.robot.link_refs[:, 0] == 1, ns + w.robot.link_refs[:, 1], w.robot.link_refs[:, 1])

    class _R:  # link refs as registry ids for _expected
        link_refs = np.stack([np.zeros_like(link_gid), link_gid], 1)

    exp = [_expected(S, _R, srv.link_poses(r.base, r.q)) for r in reqs]
    ids = [srv.submit(r.base, r.q) for r in reqs]
    got = [srv.wait(i) for i in ids]
    for (first, clr, k, i), g in zip(exp, got):
        assert g["first_colliding_waypoint"] == first
        if clr > 0:
            assert abs(g["min_clearance"] - clr) <= max(REL * abs(clr), ABS)
        else:
            assert g["min_clearance"] <= 0
    srv.close()


def test_destroy_releases_blocked_waiters(gpu_lib):
    """Threads blocked in wait() on unfinished requests return when the server is
    destroyed (FCLGPU_ERR_NOT_INITIALIZED, or the result if the request finished
    first); destroy returns only after they have left the call."""
    import threading
    from fcl_gb300 import native as N
    w = W.scene4(n_objects=2000, seed=5, box=12.0, n_shape_geoms=128, mesh_fraction=0.0, mesh_links=False)
    ss = api.ShapeSet.from_workload(w.shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(w.refs, w.tf)
    reqs = W.motion_requests(w, 6, seed=7, k_lo=200, k_hi=400)
    srv = api.MotionServer(mgr, w.robot, max_waypoints_per_step=8)
    ids = [srv.submit(r.base, r.q) for r in reqs]
    outcome = {}

    def waiter(i):
        try:
            outcome[i] = srv.wait(i)
        except N.FclGpuError as e:
            outcome[i] = e.code

    th = [threading.Thread(target=waiter, args=(i,), daemon=True) for i in ids]
    for t in th:
        t.start()
    import time
    time.sleep(0.5)  # every waiter is inside wait() before destroy begins (the documented contract)
    srv.close()
    for t in th:
        t.join(timeout=60)
    assert not any(t.is_alive() for t in th)
    assert set(outcome) == set(ids)
    assert all(isinstance(v, dict) or v == N.FCLGPU_ERR_NOT_INITIALIZED for v in outcome.values())


def test_memory_budget_limits_step_size_not_results(gpu_lib):
    """Admission under a small free-memory budget: every step takes only the few
    waypoints the budget allows, and each request still returns what it returns
    without the budget."""
    w = W.scene4(n_objects=1500, seed=12, box=10.0, n_shape_geoms=128, mesh_fraction=0.0, mesh_links=False)
    ss = api.ShapeSet.from_workload(w.shapes)
    mgr = api.DynamicAABBTreeCollisionManager(ss)
    mgr.registerObjects(w.refs, w.tf)
    reqs = W.motion_requests(w, 4, seed=13, k_lo=10, k_hi=30)
    free = api.MotionServer(mgr, w.robot, max_waypoints_per_step=256)
    want = [free.wait(free.submit(r.base, r.q)) for r in reqs]
    free.close()
    tight = api.MotionServer(mgr, w.robot, max_waypoints_per_step=256, memory_budget_bytes=100_000)
    got = [tight.wait(tight.submit(r.base, r.q)) for r in reqs]
    st = tight.stats()
    tight.close()
    assert 1 <= st["max_step_waypoints"] <= 4
    for a, b in zip(want, got):
        for k in ("first_colliding_waypoint", "min_clearance", "clearance_waypoint", "clearance_link",
                  "clearance_object"):
            assert a[k] == b[k], k
