"""Convex-pair oracle (GJK/EPA GST_INDEP + closed forms) against reference known answers."""
import numpy as np
import pytest

from oracle import pyoracle as O
from fcl_gb300 import workloads as W


def test_projection_known_answers():
    # test/test_fcl_simple.cpp:173-214: triangle (0,0,1),(0,1,0),(1,0,0) and point p;
    # the origin projection of the translated triangle is the same problem
    v = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0]], float)
    for p, enc, sq, par in [((1, 1, 1), 7, 4 / 3.0, (1 / 3.0, 1 / 3.0, 1 / 3.0)),
                            ((0, 0, 1.5), 1, 0.25, (1, 0, 0)),
                            ((1.5, 0, 0), 4, 0.25, (0, 0, 1))]:
        e, s, prm = O.project_origin(v - np.array(p, float))
        assert e == enc
        assert abs(s - sq) < 1e-12
        assert np.allclose(prm[:3], par, atol=1e-12)
    # line (test_projection_test_line :152-165): a=(0,0,1), b=(0,1,0), p=(0,0,1.5) -> a
    e, s, prm = O.project_origin(np.array([[0, 0, 1], [0, 1, 0]], float) - np.array([0, 0, 1.5]))
    assert e == 1 and abs(s - 0.25) < 1e-12 and np.allclose(prm[:2], (1, 0))


def _one(t, params, tf1, tf2, t2=None, params2=None, verts=None):
    s = W.ShapeSet(np.array([t, t2 if t2 is not None else t], np.int32),
                   np.array([params, params2 if params2 is not None else params], float),
                   np.zeros(2, np.int32), np.zeros(2, np.int32), np.zeros((0, 3)))
    return O.shape_batch(s, [0], [1], tf1[None], tf2[None])


def _tf(t=(0, 0, 0), R=None):
    tf = np.zeros((3, 4)); tf[:, :3] = np.eye(3) if R is None else R; tf[:, 3] = t
    return tf


def test_sphere_sphere_known_answers():
    # test_fcl_geometric_shapes.cpp:3667-3700 (shapeDistance_spheresphere): r=20 and r=10
    for t1, t2, expect in [((0, 0, 0), (0, 40, 0), 10.0), ((0, 0, 0), (30.1, 0, 0), 0.1),
                           ((40, 0, 0), (0, 0, 0), 10.0), ((30.1, 0, 0), (0, 0, 0), 0.1)]:
        r = _one(W.SPHERE, [20, 0, 0], _tf(t1), _tf(t2), t2=W.SPHERE, params2=[10, 0, 0])
        assert not r["hit"][0] and abs(r["dist"][0] - expect) < 0.001
    for t1, t2 in [((0, 0, 0), (29.9, 0, 0)), ((29.9, 0, 0), (0, 0, 0))]:
        r = _one(W.SPHERE, [20, 0, 0], _tf(t1), _tf(t2), t2=W.SPHERE, params2=[10, 0, 0])
        assert r["hit"][0]


def test_box_sphere_distance_known_answer():
    # test_fcl_geometric_shapes.cpp:4945-4980 (shapeDistanceGJK_boxsphere, GJKSolver_indep):
    # Sphere(20) vs Box(5,5,5): overlapping at identity, 0.1 at x=22.6, 17.5 at x=40, and
    # the same under a common rigid transform
    R = W.random_poses(1, -10, 10, 123)[0]
    for X in (_tf(), R):
        def comp(t):
            out = X.copy()
            out[:, 3] = X[:, :3] @ np.array(t, float) + X[:, 3]
            return out
        r = _one(W.SPHERE, [20, 0, 0], X, X, t2=W.BOX, params2=[5, 5, 5])
        assert r["hit"][0]
        r = _one(W.SPHERE, [20, 0, 0], X, comp((22.6, 0, 0)), t2=W.BOX, params2=[5, 5, 5])
        assert not r["hit"][0] and abs(r["dist"][0] - 0.1) < 0.01
        r = _one(W.SPHERE, [20, 0, 0], X, comp((40, 0, 0)), t2=W.BOX, params2=[5, 5, 5])
        assert not r["hit"][0] and abs(r["dist"][0] - 17.5) < 0.001


def test_gjk_box_box_distance():
    # two unit boxes 3 apart along x: GJK distance 2 with witnesses on the faces
    r = _one(W.BOX, [1, 1, 1], _tf(), _tf((3, 0, 0)))
    assert not r["hit"][0] and abs(r["dist"][0] - 2.0) < 1e-9
    assert abs(r["p1"][0][0] - 0.5) < 1e-9 and abs(r["p2"][0][0] - 2.5) < 1e-9


def test_gjk_epa_penetration_boxes_offset():
    # capsule/cylinder/cone pairs overlapping: EPA returns a depth (FCL reports -depth)
    for t in (W.CAPSULE, W.CYLINDER, W.CONE):
        r = _one(t, [0.5, 2.0, 0], _tf(), _tf((0.6, 0, 0)))
        assert r["hit"][0]
        assert r["depth"][0] < 0  # GST_INDEP ContactPoint depth = -epa.depth
        assert abs(r["depth"][0]) < 1.0


def test_random_batch_consistency():
    w = W.config3(n_pairs=3000, n_shapes=64, seed=5)
    r = O.shape_batch(w.shapes, w.ia, w.ib, w.tf1, w.tf2, nthreads=4)
    sep = ~r["hit"]
    ok = r["dist"][sep] >= 0
    assert ok.mean() > 0.99
    # separated pairs: witness distance equals the reported distance
    d = np.linalg.norm(r["p1"][sep][ok] - r["p2"][sep][ok], axis=1)
    assert np.allclose(d, r["dist"][sep][ok], rtol=1e-6, atol=1e-9)


def test_gjk_tolerance_constant():
    # FCL's gjk_default_tolerance = std::pow(eps, 7/8) (math/constants.h:145-167);
    # the oracle and the device code use this literal
    import math
    assert math.pow(np.finfo(np.float64).eps, 7.0 / 8.0) == 2.0097183471152322e-14
