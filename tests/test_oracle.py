"""The FP64 oracle against the reference's own known answers and invariants."""
import math

import numpy as np
import pytest

from oracle import pyoracle as O
from fcl_gb300 import workloads as W


def _rss(axis, To, l, r):
    return np.concatenate([np.asarray(axis, float).reshape(9), To, l, [r]])


def test_rss_distance_known_answers():
    # test/test_fcl_math.cpp:256-290 (test_rss_distance), expected within eps^(7/8)
    eps = np.finfo(np.float64).eps ** (7.0 / 8.0)
    p0 = np.array([[1, 1, 1], [1, 1, -1], [0, 1, -1]], float)
    p1 = np.array([[1, -1, 1], [1, -1, -1], [0, -1, -1]], float)
    assert abs(O.rss_member_distance(O.rss_fit3(p0), O.rss_fit3(p1)) - 2.0) < eps
    a = _rss(np.eye(3), [0, 0, 0.5], [1, 1], 0.5)
    b = _rss(np.eye(3), [-1, -1, 2.5], [1, 1], 0.5)
    assert abs(O.rss_member_distance(a, b) - 1.0) < eps
    b2 = _rss(-np.eye(3), [-1, -1, 2.5], [1, 1], 0.5)
    assert abs(O.rss_member_distance(a, b2) - (math.sqrt(6) - 1.0)) < eps
    b3 = _rss(-np.eye(3), [0, 0, 2.5], [1, 1], 0.5)
    assert abs(O.rss_member_distance(a, b3) - 1.0) < eps


def test_rss_fit3_known_answer():
    # test/test_fcl_math.cpp:201-208: fitting (0,0,0),(1,0,0),(0,1,0)
    r = O.rss_fit3(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float))
    assert abs(r[12] - math.sqrt(2.0)) < 1e-12   # width = l[0]
    assert abs(r[13] - math.sqrt(2.0) / 2) < 1e-12
    assert r[14] == 0.0


def test_obb_overlap_basic():
    I = np.eye(3).reshape(9)
    a = np.concatenate([I, [0, 0, 0], [1, 1, 1]])
    tf = np.zeros((3, 4)); tf[:, :3] = np.eye(3)
    assert O.obb_overlap(tf, a, a)
    tf[0, 3] = 2.0 + 1e-3          # gap > 1e-6 padding (OBB-inl.h:404)
    assert not O.obb_overlap(tf, a, a)
    tf[0, 3] = 2.0 - 1e-3
    assert O.obb_overlap(tf, a, a)


def test_triangle_tests_touching_and_separated():
    P = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], float)
    tf = np.zeros((3, 4)); tf[:, :3] = np.eye(3)
    Q = np.array([[0.2, 0.2, 0.0, 0.2, 0.2, 1.0, 0.3, 0.2, 1.0]], float)   # touches the face
    assert O.tri_intersect_batch(P, Q, tf)[0]
    Q2 = Q.copy(); Q2[0, 2::3] += 1e-3
    assert not O.tri_intersect_batch(P, Q2, tf)[0]
    d, _ = O.tri_distance_batch(P, Q2)
    assert abs(d[0] - 1e-3) < 1e-12


@pytest.mark.parametrize("i", range(10))
def test_reference_fixture_cross_consistency(golden, i):
    """test_fcl_collision.cpp:313-888 / test_fcl_distance.cpp:85-304: on env.obj x
    rob.obj the OBBRSS traversal must report the same contacts as any other BV type.
    The AABB / brute-force equivalent is the set of all intersecting triangle pairs,
    and the distance must equal the minimum over all triangle pairs."""
    env = O.Mesh(golden["env_v"], golden["env_t"])
    rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    tf = golden["tf"][i]
    counts, contacts, _, _ = O.collide_batch(env, rob, tf[None], num_max_contacts=1 << 30)
    brute = O.brute_collide(env, rob, tf)
    assert sorted(map(tuple, contacts)) == sorted(map(tuple, brute))
    d, ids, pts, _, _ = O.distance_batch(env, rob, tf[None], nearest=True)
    assert d[0] == O.brute_distance(env, rob, tf)
    if d[0] > 0:
        assert abs(np.linalg.norm(pts[0, 0] - pts[0, 1]) - d[0]) <= 1e-9 * max(1.0, d[0])


def test_bvh_structure_contains_triangles():
    v, t = W.perturbed_ellipsoid(6, (1.0, 0.7, 0.5), 0.01, 3)
    m = O.Mesh(v, t)
    nodes, fc = m.nodes()
    assert nodes.shape[0] == 2 * t.shape[0] - 1
    leaves = sorted(-(c + 1) for c in fc if c < 0)
    assert leaves == list(range(t.shape[0]))
    # every leaf OBB contains its triangle (up to rounding)
    for k in np.nonzero(fc < 0)[0]:
        A = nodes[k, :9].reshape(3, 3); To = nodes[k, 9:12]; ext = nodes[k, 12:15]
        tri = v[t[-(fc[k] + 1)]]
        loc = (tri - To) @ A
        assert np.all(np.abs(loc) <= ext + 1e-9)


def test_collide_num_max_contacts_semantics():
    w = W.config0(n_poses=200, freq=8)
    a = O.Mesh(*w.meshes[0]); b = O.Mesh(*w.meshes[1])
    c1, ct1, _, _ = O.collide_batch(a, b, w.tf2, num_max_contacts=1)
    call, ctall, _, _ = O.collide_batch(a, b, w.tf2, num_max_contacts=1 << 30)
    assert np.array_equal(c1, np.minimum(call, 1))
    # the first contact found with num_max_contacts=1 is the first of the full DFS list
    off = np.concatenate([[0], np.cumsum(call)])
    off1 = np.concatenate([[0], np.cumsum(c1)])
    for i in np.nonzero(c1)[0]:
        assert tuple(ct1[off1[i]]) == tuple(ctall[off[i]])
    c0, _, _, _ = O.collide_batch(a, b, w.tf2, num_max_contacts=0)
    assert c0.sum() == 0
