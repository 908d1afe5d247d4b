"""Mesh-shape oracle (BVHModel<OBBRSS> x convex shape with GJKSolver_indep): the
reference's shape-triangle known answers, and the BVH traversals against a brute-force
loop over every triangle."""
import numpy as np
import pytest

from fcl_gb300 import workloads as W
from oracle import pyoracle as P


def _tri_mesh(tri):
    return P.Mesh(np.asarray(tri, np.float64), np.array([[0, 1, 2]], np.int32))


def test_sphere_triangle_known_answers():
    # test_fcl_geometric_shapes.cpp:4670-4700 (shapeIntersectionGJK_spheretriangle):
    # sphere r = 10 against two triangles, identity and a shared random transform
    S = W.ShapeSet(np.array([W.SPHERE], np.int32), np.array([[10.0, 0, 0]]), np.zeros(1, np.int32),
                   np.zeros(1, np.int32), np.zeros((0, 3)))
    G = P.Geoms(S)
    tf = W.random_poses(1, -1.0, 1.0, 3)[0]
    eye = W.identity_poses(1)[0]
    for tri in ([[20, 0, 0], [-20, 0, 0], [0, 20, 0]], [[30, 0, 0], [9.9, -20, 0], [9.9, 20, 0]]):
        m = _tri_mesh(tri)
        for t in (eye, tf):
            c, _, _ = P.mesh_shape_collide(m, G, [0], t, t, max_contacts=1)
            assert c[0] == 1
    # a triangle just beyond the sphere's reach
    m = _tri_mesh([[30, 0, 0], [10.1, -20, 0], [10.1, 20, 0]])
    c, _, _ = P.mesh_shape_collide(m, G, [0], eye, eye)
    assert c[0] == 0
    d = P.mesh_shape_distance(m, G, [0], eye, eye)
    assert abs(d["dist"][0] - 0.1) < 1e-12


def test_sphere_triangle_contact_known_answers():
    # test_fcl_geometric_shapes.cpp:4697-4705: sphere r = 10, triangle (30,0,0), (9.9,-20,0),
    # (9.9,20,0): shapeTriangleIntersect's normal is (1,0,0), and R (1,0,0) under a shared
    # transform; the mesh-shape leaf records -normal, the nearest edge point, depth -0.1
    S = W.ShapeSet(np.array([W.SPHERE], np.int32), np.array([[10.0, 0, 0]]), np.zeros(1, np.int32),
                   np.zeros(1, np.int32), np.zeros((0, 3)))
    G = P.Geoms(S)
    m = _tri_mesh([[30, 0, 0], [9.9, -20, 0], [9.9, 20, 0]])
    tf = W.random_poses(1, -1.0, 1.0, 3)[0]
    eye = W.identity_poses(1)[0]
    for t in (eye, tf):
        R = t.reshape(3, 4)[:, :3]
        o = P.mesh_shape_contact_geometry(m, G, [0], t, t, [0])
        assert o["ok"][0] == 1
        np.testing.assert_allclose(o["normal"][0], -R @ np.array([1.0, 0, 0]), atol=1e-9)
        np.testing.assert_allclose(o["depth"][0], -0.1, atol=1e-9)
        np.testing.assert_allclose(o["pos"][0], R @ np.array([9.9, 0, 0]) + t.reshape(3, 4)[:, 3], atol=1e-9)
    # a GJK shape: a box of side 2 resting 0.05 deep in a large triangle; EPA's contact
    B = W.ShapeSet(np.array([W.BOX], np.int32), np.array([[2.0, 2.0, 2.0]]), np.zeros(1, np.int32),
                   np.zeros(1, np.int32), np.zeros((0, 3)))
    Gb = P.Geoms(B)
    mb = _tri_mesh([[-20, -20, 0], [20, -20, 0], [0, 20, 0]])
    tb = eye.copy().reshape(3, 4)
    tb[2, 3] = 0.95
    o = P.mesh_shape_contact_geometry(mb, Gb, [0], eye, tb.reshape(12), [0])
    assert o["ok"][0] == 1
    np.testing.assert_allclose(o["depth"][0], -0.05, atol=1e-9)
    np.testing.assert_allclose(np.abs(o["normal"][0]), [0, 0, 1], atol=1e-9)


@pytest.mark.parametrize("seed", [0, 1])
def test_mesh_shape_traversals_match_brute_force(seed):
    v, t = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, seed)
    m = P.Mesh(v, t)
    shapes = W.random_shapes(48, seed + 5)
    G = P.Geoms(shapes)
    n = 96
    rng = np.random.default_rng(seed)
    sid = rng.integers(0, 48, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.2, 0.2, seed + 1)
    tfs = W.random_poses(n, -1.2, 1.2, seed + 2)
    counts, nbv, nleaf = P.mesh_shape_collide(m, G, sid, tfm, tfs, max_contacts=10 ** 6)
    dist = P.mesh_shape_distance(m, G, sid, tfm, tfs)
    hits = 0
    for q in range(n):
        c, d = P.mesh_shape_brute(m, G, int(sid[q]), tfm[q], tfs[q])
        assert counts[q] == c
        hits += c > 0
        if d > 0:
            assert abs(dist["dist"][q] - d) <= 1e-9 * max(1.0, d)
        else:
            assert dist["dist"][q] <= 0
    assert 0 < hits < n
    # the traversal prunes
    assert nleaf.sum() < n * t.shape[0]
    # boolean collide stops at the first contact
    c1, _, _ = P.mesh_shape_collide(m, G, sid, tfm, tfs, max_contacts=1)
    np.testing.assert_array_equal(c1, np.minimum(counts, 1))


def test_shape_obbrss_contains_bound_vertices():
    shapes = W.random_shapes(24, 9)
    G = P.Geoms(shapes)
    tf = W.random_poses(1, -1, 1, 2)[0]
    for sid in range(24):
        o = P.shape_obbrss(G, sid, tf)
        axis = o[:9].reshape(3, 3)
        np.testing.assert_allclose(axis.T @ axis, np.eye(3), atol=1e-12)
        assert np.all(o[12:15] >= 0)
