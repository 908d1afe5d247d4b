"""The broadphase oracle: CollisionObject world AABBs, the dynamic AABB tree manager
with FCL's default callbacks, and the naive manager it must agree with (the
reference's own broadphase tests compare every manager's contact count with the naive
manager's: test_fcl_broadphase_collision_2.cpp:185-340, test_fcl_broadphase_distance.cpp)."""
import numpy as np
import pytest

from fcl_gb300 import workloads as W
from oracle import pyoracle as P


def _scene(n, seed, box=6.0, n_geoms=64):
    shapes = W.random_shapes(n_geoms, seed)
    rng = np.random.default_rng(seed + 1)
    gid = rng.integers(0, n_geoms, size=n).astype(np.int32)
    tf = W.random_poses(n, 0.0, box, seed + 2)
    return shapes, gid, tf


def test_world_aabb_follows_compute_aabb():
    # box 1 x 2 x 3, sphere r 0.5, capsule r 0.2 lz 1, cylinder r 0.3 lz 2
    types = np.array([W.BOX, W.SPHERE, W.CAPSULE, W.CYLINDER], np.int32)
    params = np.array([[1, 2, 3], [0.5, 0, 0], [0.2, 1.0, 0], [0.3, 2.0, 0]], np.float64)
    S = W.ShapeSet(types, params, np.zeros(4, np.int32), np.zeros(4, np.int32), np.zeros((0, 3)))
    G = P.Geoms(S)
    loc = G.local()
    # aabb_local, aabb_center, aabb_radius per shape (box-inl.h:80-88, sphere-inl.h:62-69,
    # capsule-inl.h:64-72, cylinder-inl.h:64-72)
    np.testing.assert_array_equal(loc[0, :6], [-0.5, -1, -1.5, 0.5, 1, 1.5])
    assert loc[0, 9] == np.sqrt(0.25 + 1 + 2.25)
    assert loc[1, 9] == 0.5
    np.testing.assert_array_equal(loc[2, 3:6], [0.2, 0.2, 0.7])
    np.testing.assert_array_equal(loc[3, 3:6], [0.3, 0.3, 1.0])
    # identity rotation: translated local box; otherwise a cube of half-size aabb_radius
    tf = np.zeros((2, 3, 4))
    tf[0, :, :3] = np.eye(3)
    tf[0, :, 3] = (1, 2, 3)
    tf[1] = W.random_poses(1, 0, 1, 3)[0]
    ab = G.world_aabbs(np.array([0, 0], np.int32), tf)
    np.testing.assert_array_equal(ab[0], [0.5, 1, 1.5, 1.5, 3, 4.5])
    r = loc[0, 9]
    c = tf[1, :, 3]
    np.testing.assert_allclose(ab[1], np.concatenate([c - r, c + r]), rtol=0, atol=1e-15)
    # a rotation within Eigen's isIdentity precision (1e-12) still counts as identity
    tf2 = tf[:1].copy()
    tf2[0, 0, 1] = 5e-13
    np.testing.assert_array_equal(G.world_aabbs(np.array([0], np.int32), tf2)[0], ab[0])


@pytest.mark.parametrize("seed", [0, 1])
def test_tree_manager_matches_naive_manager_shapes(seed):
    shapes, gid, tf = _scene(400, seed)
    G = P.Geoms(shapes)
    S = P.Scene(G, gid, tf)
    assert S.num_tree_nodes() == 2 * 400 - 1
    rng = np.random.default_rng(seed + 10)
    qg = rng.integers(0, shapes.n, size=150).astype(np.int32)
    qtf = W.random_poses(150, 0.0, 6.0, seed + 11)
    for M in (1, 100000):
        a = S.collide(qg, qtf, max_contacts=M, use_tree=True)
        b = S.collide(qg, qtf, max_contacts=M, use_tree=False)
        np.testing.assert_array_equal(a["num_contacts"], b["num_contacts"])
        if M > 1:
            np.testing.assert_array_equal(a["num_hits"], b["num_hits"])
            oa = np.split(a["hits"], np.cumsum(a["num_hits"])[:-1])
            ob = np.split(b["hits"], np.cumsum(b["num_hits"])[:-1])
            for x, y in zip(oa, ob):
                np.testing.assert_array_equal(np.sort(x), np.sort(y))
    assert (a["num_contacts"] > 0).mean() > 0.1  # the scene is dense enough to test something
    da = S.distance(qg, qtf, use_tree=True)
    db = S.distance(qg, qtf, use_tree=False)
    sep = db["dist"] > 0
    np.testing.assert_array_equal(da["dist"] <= 0, db["dist"] <= 0)
    np.testing.assert_array_equal(da["dist"][sep], db["dist"][sep])
    np.testing.assert_array_equal(da["obj"][sep], db["obj"][sep])
    assert sep.any() and (~sep).any()


def test_tree_manager_matches_naive_manager_meshes():
    meshes = [P.Mesh(*W.perturbed_ellipsoid(3, (0.6, 0.4, 0.3), 0.01, k)) for k in range(3)]
    G = P.Geoms(None, meshes)
    n = 40
    rng = np.random.default_rng(7)
    gid = rng.integers(0, 3, size=n).astype(np.int32)
    tf = W.random_poses(n, 0.0, 3.0, 8)
    S = P.Scene(G, gid, tf)
    qg = rng.integers(0, 3, size=20).astype(np.int32)
    qtf = W.random_poses(20, 0.0, 3.0, 9)
    for M in (1, 100000):
        a = S.collide(qg, qtf, max_contacts=M, use_tree=True)
        b = S.collide(qg, qtf, max_contacts=M, use_tree=False)
        np.testing.assert_array_equal(a["num_contacts"], b["num_contacts"])
    assert (a["num_contacts"] > 0).any()
    da = S.distance(qg, qtf, use_tree=True)
    db = S.distance(qg, qtf, use_tree=False)
    sep = db["dist"] > 0
    np.testing.assert_array_equal(da["dist"] <= 0, db["dist"] <= 0)
    np.testing.assert_array_equal(da["dist"][sep], db["dist"][sep])


def test_candidates_are_exact_aabb_overlaps():
    shapes, gid, tf = _scene(300, 3)
    G = P.Geoms(shapes)
    S = P.Scene(G, gid, tf)
    qg = np.arange(50, dtype=np.int32)
    qtf = W.random_poses(50, 0.0, 6.0, 4)
    counts, ids = S.candidates(qg, qtf)
    A = G.world_aabbs(gid, tf)
    Q = G.world_aabbs(qg, qtf)
    seg = np.split(ids, np.cumsum(counts)[:-1])
    for q in range(50):
        ov = ~((A[:, :3] > Q[q, 3:]).any(1) | (A[:, 3:] < Q[q, :3]).any(1))
        np.testing.assert_array_equal(np.nonzero(ov)[0], seg[q])


def test_tree_manager_matches_naive_manager_mixed():
    shapes = W.random_shapes(32, 12)
    meshes = [P.Mesh(*W.perturbed_ellipsoid(4, (0.6, 0.4, 0.3), 0.01, k)) for k in range(2)]
    G = P.Geoms(shapes, meshes)
    rng = np.random.default_rng(13)
    n = 120
    gid = np.where(rng.uniform(size=n) < 0.3, 32 + rng.integers(0, 2, size=n), rng.integers(0, 32, size=n))
    gid = gid.astype(np.int32)
    tf = W.random_poses(n, 0.0, 4.0, 14)
    S = P.Scene(G, gid, tf)
    qg = np.where(rng.uniform(size=60) < 0.5, 32 + rng.integers(0, 2, size=60), rng.integers(0, 32, size=60))
    qg = qg.astype(np.int32)
    qtf = W.random_poses(60, 0.0, 4.0, 15)
    for M in (1, 100000):
        a = S.collide(qg, qtf, max_contacts=M, use_tree=True)
        b = S.collide(qg, qtf, max_contacts=M, use_tree=False)
        np.testing.assert_array_equal(a["num_contacts"], b["num_contacts"])
    assert (a["num_contacts"] > 0).any()
    da = S.distance(qg, qtf, use_tree=True)
    db = S.distance(qg, qtf, use_tree=False)
    sep = db["dist"] > 0
    np.testing.assert_array_equal(da["dist"] <= 0, db["dist"] <= 0)
    np.testing.assert_array_equal(da["dist"][sep], db["dist"][sep])


def test_other_manager_names_answer_like_the_tree():
    """FCL's other BroadPhaseCollisionManager implementations are offered under their names
    and answered by the device tree: the results the device manager reports are
    order-independent, so the tree and the brute-force manager agree (checked above on
    the oracle); the classes keep the manager interface."""
    from fcl_gb300 import api
    for name in ("NaiveCollisionManager", "SaPCollisionManager", "SSaPCollisionManager",
                 "IntervalTreeCollisionManager", "DynamicAABBTreeCollisionManager_Array"):
        cls = getattr(api, name)
        assert issubclass(cls, api.DynamicAABBTreeCollisionManager)
        for m in ("registerObjects", "setup", "update", "collide_batch", "distance_batch", "size"):
            assert callable(getattr(cls, m))


def test_contact_lists_hold_fcl_callback_contacts():
    """The list definition (each overlapping object in index order, a fresh result per
    pair) against FCL's manager with DefaultCollisionFunction: with a cap above every
    total the per-query totals and the colliding objects are FCL's; with cap M FCL's
    numContacts() is min(M, the list length)."""
    shapes = W.random_shapes(64, 3)
    vt = [W.perturbed_ellipsoid(4, (0.6, 0.4, 0.3), 0.01, 5)]
    G = P.Geoms(shapes, [P.Mesh(*vt[0])])
    rng = np.random.default_rng(4)
    n, nq = 300, 200
    gid = np.where(rng.uniform(size=n) < 0.3, 64, rng.integers(0, 64, size=n)).astype(np.int32)
    qgid = np.where(rng.uniform(size=nq) < 0.3, 64, rng.integers(0, 64, size=nq)).astype(np.int32)
    S = P.Scene(G, gid, W.random_poses(n, 0.0, 6.0, 5))
    qtf = W.random_poses(nq, 0.0, 6.0, 6)
    c, trip = S.collide_lists(qgid, qtf, max_per_pair=1 << 30, nthreads=4)
    o = S.collide(qgid, qtf, max_contacts=1 << 30, use_tree=True, nthreads=4)
    np.testing.assert_array_equal(c, o["num_contacts"])
    segs = np.split(trip[:, 0], np.cumsum(c)[:-1])
    hits = np.split(o["hits"], np.cumsum(o["num_hits"])[:-1])
    assert all(sorted(set(a)) == sorted(h) for a, h in zip(segs, hits))
    for M in (1, 3):
        cm, _ = S.collide_lists(qgid, qtf, max_per_pair=M, nthreads=4)
        om = S.collide(qgid, qtf, max_contacts=M, use_tree=False, nthreads=4)
        np.testing.assert_array_equal(np.minimum(cm, M), om["num_contacts"])
    # the scene against itself: the lists' total is the naive manager's numContacts()
    sc, strip = S.self_collide_lists(max_per_pair=1 << 30)
    assert S.self_collide_count(1 << 40) == sc.sum() > 0
    assert np.all(strip[:, 0] < np.repeat(np.arange(n), sc))
