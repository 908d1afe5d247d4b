"""GPU GJK/EPA + closed-form shape pairs against the FP64 oracle (GJKSolver_indep)."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def test_shape_batch_matches_oracle(gpu_lib):
    w = W.config3(n_pairs=20000, n_shapes=256, seed=7)
    ss = api.ShapeSet.from_workload(w.shapes)
    g = api.shape_batch(ss, w.ia, w.ib, w.tf1, w.tf2)
    o = O.shape_batch(w.shapes, w.ia, w.ib, w.tf1, w.tf2, nthreads=8)
    assert np.array_equal(g["hit"], o["hit"])
    assert np.array_equal(g["status"], o["status"])
    # same FP64 arithmetic in the same order: bit-identical results
    for k in ("normal", "point", "depth", "dist", "p1", "p2"):
        assert np.array_equal(g[k], o[k]), k


def test_shape_batch_device_api(gpu_lib):
    import torch
    w = W.config3(n_pairs=5000, n_shapes=64, seed=8)
    ss = api.ShapeSet.from_workload(w.shapes)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    g = api.shape_batch(ss, d(w.ia), d(w.ib), d(w.tf1), d(w.tf2))
    torch.cuda.synchronize()
    o = O.shape_batch(w.shapes, w.ia, w.ib, w.tf1, w.tf2, nthreads=8)
    assert np.array_equal(g["hit"].cpu().numpy().astype(bool), o["hit"])
    assert np.array_equal(g["dist"].cpu().numpy(), o["dist"])


def _kat_cases():
    """The known-answer configurations of FCL's shape tests that the oracle is pinned to
    (test_fcl_sphere_capsule.cpp, test_fcl_capsule_capsule.cpp, test_fcl_sphere_box.cpp,
    test_fcl_sphere_cylinder.cpp, test_fcl_sphere_sphere.cpp), as (type, params) pairs
    and poses."""
    def tf(t=(0, 0, 0), R=None):
        x = np.zeros((3, 4)); x[:, :3] = np.eye(3) if R is None else R; x[:, 3] = t
        return x

    def aa(angle, axis):
        k = np.asarray(axis, float) / np.linalg.norm(axis)
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        return np.cos(angle) * np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * np.outer(k, k)

    rx = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]], float)
    cases = []
    sph, cap = (W.SPHERE, [50, 0, 0]), (W.CAPSULE, [50, 200, 0])
    for ts, tc, R in [((0, 0, -50), (0, 0, 200), None), ((0, 0, 50), (0, 0, -200), None),
                      ((0, 0, -50), (150, 0, 0), None), ((0, 0, -50), (150, 0, 0), rx),
                      ((0, 0, -50), (0, 0, 125), None), ((0, 0, 0), (0, 50, 75), rx),
                      ((0, 0, -50), (0, 0, 100), None), ((0, 0, -50), (0, 0, 175), None)]:
        cases.append((sph, cap, tf(ts), tf(tc, R)))
    R_FT, t_FT = aa(np.pi / 7, (1, 2, 3)), np.array([10.5, 12.75, -2.5])
    cases.append(((W.CAPSULE, [1.5, 2.5, 0]), (W.CAPSULE, [2, 3, 0]), tf(t_FT, R_FT),
                  tf(R_FT @ np.array([0, 0, 5.0]) + t_FT, R_FT @ aa(np.pi / 2, (0, 1, 0)))))
    eps = np.finfo(float).eps
    w, d, h, r = 0.115, 0.01, 0.0025, 0.0015
    for sx in (-w / 2 + r, -w / 4, -eps, 0.0, eps, w / 4, w / 2 - r):
        for sy in (-d / 2 + r, -d / 4, -eps, 0.0, eps, d / 4, d / 2 - r):
            p = tf((sx, sy, h / 2 + r / 2))
            cases.append(((W.SPHERE, [r, 0, 0]), (W.BOX, [w, d, h]), p, tf()))
            cases.append(((W.BOX, [w, d, h]), (W.SPHERE, [r, 0, 0]), tf(), p))
    for rr in (0.0, eps, 4.5, 9 - 0.0015):
        for th in (0, np.pi / 2, np.pi, 3 * np.pi / 4):
            a = th + np.pi / 7
            p = tf((np.cos(a) * rr, np.sin(a) * rr, 0.0025 / 2 + 0.0015 / 2))
            cases.append(((W.SPHERE, [0.0015, 0, 0]), (W.CYLINDER, [9, 0.0025, 0]), p, tf()))
            cases.append(((W.CYLINDER, [9, 0.0025, 0]), (W.SPHERE, [0.0015, 0, 0]), tf(), p))
    spheres = [(0.5, (0, 0, -1)), (0.6, (1.2, 0, 0)), (0.4, (-0.3, 0, 0)), (0.3, (0, 0, 1))]
    for i in range(4):
        for j in range(4):
            if i != j:
                cases.append(((W.SPHERE, [spheres[i][0], 0, 0]), (W.SPHERE, [spheres[j][0], 0, 0]),
                              tf(spheres[i][1]), tf(spheres[j][1])))
    return cases


def test_reference_known_answer_cases_match_oracle(gpu_lib):
    """FCL's shape known-answer configurations through the product: bit for bit the oracle,
    which tests/test_oracle_gjk.py pins to FCL's expected values."""
    cases = _kat_cases()
    n = len(cases)
    types = np.array([c[k][0] for c in cases for k in (0, 1)], np.int32)
    params = np.array([c[k][1] for c in cases for k in (0, 1)], float)
    ia, ib = np.arange(0, 2 * n, 2, dtype=np.int32), np.arange(1, 2 * n, 2, dtype=np.int32)
    tf1 = np.stack([c[2] for c in cases]); tf2 = np.stack([c[3] for c in cases])
    ws = W.ShapeSet(types, params, np.zeros(2 * n, np.int32), np.zeros(2 * n, np.int32), np.zeros((0, 3)))
    ref = O.shape_batch(ws, ia, ib, tf1, tf2)
    got = api.shape_batch(api.ShapeSet(types, params), ia, ib, tf1, tf2)
    for k in ("hit", "normal", "point", "depth", "dist", "p1", "p2"):
        assert np.array_equal(np.asarray(got[k]), np.asarray(ref[k])), k
