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


def _angle_axis(angle, axis):
    # Eigen::AngleAxis::toRotationMatrix
    a = np.asarray(axis, float)
    s = np.sin(angle) * a
    c = np.cos(angle)
    c1 = (1 - c) * a
    R = np.empty((3, 3))
    t = c1[0] * a[1]; R[0, 1] = t - s[2]; R[1, 0] = t + s[2]
    t = c1[0] * a[2]; R[0, 2] = t + s[1]; R[2, 0] = t - s[1]
    t = c1[1] * a[2]; R[1, 2] = t - s[0]; R[2, 1] = t + s[0]
    for i in range(3):
        R[i, i] = c1[i] * a[i] + c
    return R


_ISO = [np.eye(3), _angle_axis(np.pi, (1, 0, 0)),
        _angle_axis(np.pi / 2, (1, 0, 0)), _angle_axis(3 * np.pi / 2, (1, 0, 0)),
        _angle_axis(np.pi / 2, (0, 1, 0)), _angle_axis(3 * np.pi / 2, (0, 1, 0))]


def _box_box_cases(size1, R1, size2, t2, R2):
    """The twelve collide calls of test_fcl_box_box.cpp:126-150: box 2 (a cube) in its
    six face-up orientations, in (1, 2) and (2, 1) order."""
    for P in _ISO:
        X1 = _tf(R=R1)
        X2 = _tf(t2, R2 @ P)
        yield 1.0, _one(W.BOX, [size1] * 3, X1, X2, t2=W.BOX, params2=[size2] * 3)
        yield -1.0, _one(W.BOX, [size2] * 3, X2, X1, t2=W.BOX, params2=[size1] * 3)


def _is_approx(a, b, tol):
    return np.linalg.norm(a - b) <= tol * min(np.linalg.norm(a), np.linalg.norm(b))


def test_box_box_all_contacts_known_answer():
    # test_fcl_box_box.cpp:227-263 (GST_INDEP, tolerance 1e-12): unit cube turned 45
    # degrees about y resting in a size-3 cube below it
    tol = 1e-12
    for sgn, r in _box_box_cases(1.0, _angle_axis(np.pi / 4, (0, 1, 0)), 3.0, (0, 0, -1.5), np.eye(3)):
        assert r["hit"][0]
        assert abs(r["depth"][0] - np.sqrt(2) / 2) <= tol
        assert _is_approx(r["normal"][0], sgn * np.array([0, 0, -1.0]), tol)
        pos = r["point"][0]
        assert abs(pos[2] + np.sqrt(2) / 4) <= tol and abs(pos[0]) <= tol
        assert -0.5 <= pos[1] <= 0.5


def test_box_box_cull_contacts_known_answer():
    # test_fcl_box_box.cpp:277-318 (GST_INDEP, tolerance 1e-14): two unit cubes, one
    # tilted pi/8 about x, the other turned pi/4 about z at z = -0.75; eight clipped
    # points are culled to four and the deepest is reported
    tol = 1e-14
    tilt = np.pi / 8
    depth = np.sqrt(2) / 2 * np.cos(np.pi / 4 - tilt) - 0.25
    ez = -0.25 - depth / 2
    ey = -np.sqrt(2) / 2 * np.sin(np.pi / 4 - tilt)
    ex = np.sqrt(2) / 2 + ey + np.finfo(float).eps
    for sgn, r in _box_box_cases(1.0, _angle_axis(tilt, (1, 0, 0)), 1.0, (0, 0, -0.75),
                                 _angle_axis(np.pi / 4, (0, 0, 1))):
        assert r["hit"][0]
        assert abs(r["depth"][0] - depth) <= tol
        assert _is_approx(r["normal"][0], sgn * np.array([0, 0, -1.0]), tol)
        pos = r["point"][0]
        assert abs(pos[2] - ez) <= tol and abs(pos[1] - ey) <= tol
        assert -ex <= pos[0] <= ex


_RX90 = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]], float)   # AngleAxis(pi/2, UnitX)


def test_sphere_capsule_known_answers():
    # test_fcl_sphere_capsule.cpp:48-260: Sphere(50) vs Capsule(50, 200); the closed forms
    # sphereCapsuleIntersect / sphereCapsuleDistance are the GST_INDEP dispatch too
    def run(ts, tc, R=None):
        return _one(W.SPHERE, [50, 0, 0], _tf(ts), _tf(tc, R), t2=W.CAPSULE, params2=[50, 200, 0])
    for ts, tc, R in [((0, 0, -50), (0, 0, 200), None), ((0, 0, 50), (0, 0, -200), None),
                      ((0, 0, -50), (150, 0, 0), None), ((0, 0, -50), (150, 0, 0), _RX90)]:
        assert not run(ts, tc, R)["hit"][0]                      # separated_z / _negative / _x / rotated
    r = run((0, 0, -50), (0, 0, 125))                            # penetration_z
    assert r["hit"][0] and r["depth"][0] == 25.0
    assert np.allclose(r["normal"][0], (0, 0, 1)) and np.allclose(r["point"][0], (0, 0, 0))
    r = run((0, 0, 0), (0, 50, 75), _RX90)                       # penetration_z_rotated
    assert r["hit"][0] and abs(r["depth"][0] - 25) < 1e-6
    assert np.allclose(r["normal"][0], (0, 0, 1)) and np.allclose(r["point"][0], (0, 0, 50), atol=1e-6)
    assert run((0, 0, -50), (0, 0, 100))["hit"][0]               # Distance_test_collision
    r = run((0, 0, -50), (0, 0, 175))                            # Distance_test_separated
    assert not r["hit"][0] and r["dist"][0] == 25.0


def _angle_axis_matrix(angle, axis):
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.cos(angle) * np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * np.outer(k, k)


def test_capsule_capsule_separated_known_answer():
    # test_fcl_capsule_capsule.cpp:535-740 (CapsuleCapsuleSegmentTest, NominalSeparatedCase):
    # Capsule(1.5, 2.5) and Capsule(2, 3) (the second turned by pi/2 about y) 0.25 apart
    # along z in a frame T, evaluated in F = X_FT (angle pi/7 about (1,2,3), translation
    # (10.5, 12.75, -2.5)); distance 0.25 and witnesses X_FT (0,0,2.75), X_FT (0,0,3) within
    # eps^(3/4)
    R_FT = _angle_axis_matrix(np.pi / 7, (1, 2, 3))
    t_FT = np.array([10.5, 12.75, -2.5])
    R_TC2 = _angle_axis_matrix(np.pi / 2, (0, 1, 0))
    X1 = _tf(t_FT, R_FT)
    X2 = _tf(R_FT @ np.array([0, 0, 1.25 + 1.5 + 2 + 0.25]) + t_FT, R_FT @ R_TC2)
    r = _one(W.CAPSULE, [1.5, 2.5, 0], X1, X2, t2=W.CAPSULE, params2=[2, 3, 0])
    eps = np.finfo(float).eps ** 0.75
    assert not r["hit"][0] and abs(r["dist"][0] - 0.25) < eps
    assert np.allclose(r["p1"][0], R_FT @ np.array([0, 0, 2.75]) + t_FT, atol=eps, rtol=0)
    assert np.allclose(r["p2"][0], R_FT @ np.array([0, 0, 3.0]) + t_FT, atol=eps, rtol=0)


@pytest.mark.parametrize("r", [0.0, np.finfo(float).eps, 4.5, 9 - 0.0015])
def test_sphere_cylinder_known_answers(r):
    # test_fcl_sphere_cylinder.cpp:100-224 (LargeCylinderSmallSphereTest, GST_INDEP): a
    # sphere of radius 0.0015 sinks half its radius into the top face of Cylinder(9,
    # 0.0025) at radial offsets r and angles theta + pi/7; depth 0.00075, normal -z (+z in
    # the reversed order), contact at (sx, sy, h/2 - depth/2), all within machine epsilon
    eps = np.finfo(float).eps
    r_c, h_c, r_s = 9.0, 0.0025, 0.0015
    depth = r_s * 0.5
    sz = h_c / 2 + r_s - depth
    pz = h_c / 2 - depth / 2
    for theta in (0, np.pi / 2, np.pi, 3 * np.pi / 4):
        a = theta + np.pi / 7
        sx, sy = np.cos(a) * r, np.sin(a) * r
        for order in (0, 1):
            if order == 0:
                res = _one(W.SPHERE, [r_s, 0, 0], _tf((sx, sy, sz)), _tf(), t2=W.CYLINDER, params2=[r_c, h_c, 0])
                nrm = (0, 0, -1)
            else:
                res = _one(W.CYLINDER, [r_c, h_c, 0], _tf(), _tf((sx, sy, sz)), t2=W.SPHERE, params2=[r_s, 0, 0])
                nrm = (0, 0, 1)
            assert res["hit"][0]
            assert abs(res["depth"][0] - depth) <= eps
            assert np.allclose(res["normal"][0], nrm, atol=eps, rtol=0)
            assert np.allclose(res["point"][0], (sx, sy, pz), atol=eps, rtol=0)


def test_sphere_box_known_answers():
    # test_fcl_sphere_box.cpp:91-210 (LargeBoxSmallSphereTest, GST_INDEP): a sphere of
    # radius 0.0015 sinks half its radius into the top face of Box(0.115, 0.01, 0.0025) at
    # a grid of offsets; depth 0.00075, normal -z (+z reversed), contact at (sx, sy,
    # h/2 - depth/2), within machine epsilon
    eps = np.finfo(float).eps
    w, d, h, r = 0.115, 0.01, 0.0025, 0.0015
    depth = r * 0.5
    sz = h / 2 + r - depth
    pz = h / 2 - depth / 2
    hx, hy = w / 2, d / 2
    xs = (-hx + r, -hx * 0.5, -eps, 0.0, eps, hx * 0.5, hx - r)
    ys = (-hy + r, -hy * 0.5, -eps, 0.0, eps, hy * 0.5, hy - r)
    for sx in xs:
        for sy in ys:
            for order in (0, 1):
                if order == 0:
                    res = _one(W.SPHERE, [r, 0, 0], _tf((sx, sy, sz)), _tf(), t2=W.BOX, params2=[w, d, h])
                    nrm = (0, 0, -1)
                else:
                    res = _one(W.BOX, [w, d, h], _tf(), _tf((sx, sy, sz)), t2=W.SPHERE, params2=[r, 0, 0])
                    nrm = (0, 0, 1)
                assert res["hit"][0]
                assert abs(res["depth"][0] - depth) <= eps
                assert np.allclose(res["normal"][0], nrm, atol=eps, rtol=0)
                assert np.allclose(res["point"][0], (sx, sy, pz), atol=eps, rtol=0)


def test_separating_spheres_known_answers():
    # test_fcl_sphere_sphere.cpp:55-178 (TestSeparatingSpheres, GST_INDEP, tolerance 1e-14):
    # every pair of four separated spheres, both orders: distance |cA - cB| - rA - rB and
    # the witnesses on the centre line
    spheres = [(0.5, (0, 0, -1)), (0.6, (1.2, 0, 0)), (0.4, (-0.3, 0, 0)), (0.3, (0, 0, 1))]
    for i in range(4):
        for j in range(4):
            if i == j:
                continue
            (ra, ca), (rb, cb) = spheres[i], spheres[j]
            ca, cb = np.array(ca, float), np.array(cb, float)
            ab = (ca - cb) / np.linalg.norm(ca - cb)
            res = _one(W.SPHERE, [ra, 0, 0], _tf(ca), _tf(cb), t2=W.SPHERE, params2=[rb, 0, 0])
            assert not res["hit"][0]
            assert abs(res["dist"][0] - (np.linalg.norm(ca - cb) - ra - rb)) < 1e-14
            assert np.allclose(res["p1"][0], ca - ab * ra, atol=1e-14, rtol=0)
            assert np.allclose(res["p2"][0], cb + ab * rb, atol=1e-14, rtol=0)


@pytest.mark.parametrize("kind", ["boxbox", "cylindercylinder", "conecone"])
def test_gjk_distance_known_answers(kind):
    # test_fcl_geometric_shapes.cpp:4939-5133 (shapeDistanceGJK_boxbox / _cylindercylinder /
    # _conecone, GJKSolver_indep): overlapping at identity; 0.1 and 5 / 30 apart along an axis;
    # the same under a common rigid transform; tolerance 0.001
    if kind == "boxbox":
        a, b = (W.BOX, [20, 40, 50]), (W.BOX, [10, 10, 10])
        cases = [((15.1, 0, 0), 0.1), ((20, 0, 0), 5.0)]
    elif kind == "cylindercylinder":
        a = b = (W.CYLINDER, [5, 10, 0])
        cases = [((10.1, 0, 0), 0.1), ((40, 0, 0), 30.0)]
    else:
        a = b = (W.CONE, [5, 10, 0])
        cases = [((10.1, 0, 0), 0.1), ((0, 0, 40), 30.0)]
    for X in (_tf(), W.random_poses(1, -10, 10, 321)[0]):
        def comp(t):
            out = X.copy()
            out[:, 3] = X[:, :3] @ np.array(t, float) + X[:, 3]
            return out
        assert _one(a[0], a[1], X, X, t2=b[0], params2=b[1])["hit"][0]
        for t, expect in cases:
            r = _one(a[0], a[1], X, comp(t), t2=b[0], params2=b[1])
            assert not r["hit"][0] and abs(r["dist"][0] - expect) < 0.001


def test_sphere_sphere_intersection_known_answers():
    # test_fcl_geometric_shapes.cpp:544-610 (shapeIntersection_spheresphere; the closed form
    # sphereSphereIntersect serves both solvers): Sphere(20) and Sphere(10) apart by 40 and
    # 30.01 (no contact), touching at 30 (depth 0 at x = 20), overlapping at 29.9 (depth 0.1
    # at x = 20 - 0.1 * 20/30, normal +x, also under a rigid transform) and concentric
    # (normal 0, position 0, depth 30)
    X = W.random_poses(1, -10, 10, 77)[0]

    def at(base, t):
        out = base.copy()
        out[:, 3] = base[:, :3] @ np.array(t, float) + base[:, 3]
        return out
    for base in (_tf(), X):
        for d in (40.0, 30.01):
            assert not _one(W.SPHERE, [20, 0, 0], base, at(base, (d, 0, 0)), t2=W.SPHERE, params2=[10, 0, 0])["hit"][0]
        for d, depth in ((30.0, 0.0), (29.9, 0.1)):
            r = _one(W.SPHERE, [20, 0, 0], base, at(base, (d, 0, 0)), t2=W.SPHERE, params2=[10, 0, 0])
            assert r["hit"][0] and abs(r["depth"][0] - depth) < 1e-12
            assert np.allclose(r["normal"][0], base[:, :3] @ np.array([1.0, 0, 0]), atol=1e-12)
            assert np.allclose(r["point"][0], at(base, (20.0 - depth * 20.0 / 30.0, 0, 0))[:, 3], atol=1e-12)
    r = _one(W.SPHERE, [20, 0, 0], _tf(), _tf(), t2=W.SPHERE, params2=[10, 0, 0])
    assert r["hit"][0] and r["depth"][0] == 30.0
    assert np.array_equal(r["normal"][0], [0, 0, 0]) and np.array_equal(r["point"][0], [0, 0, 0])
