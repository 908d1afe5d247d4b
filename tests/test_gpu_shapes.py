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
