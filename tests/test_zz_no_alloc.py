"""The allocation-free distance entry point (fclgpu_distance_batch_noalloc).

Callers that cannot allocate GPU memory at query time -- deadline-bound control
loops, processes whose device memory belongs to another allocator -- use this entry
point; its scratch is a fixed array inside the library.  It must return what the
allocating entry point (fclgpu_distance_batch_device) returns, on consecutive calls
that reuse the shared scratch, including after a larger call with another mesh and
pair table has left its contents there.  This file is collected last so a failure
here does not hide the others.
"""
import ctypes as C

import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import native as N
from fcl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _noalloc(meshes, pairs, tf2, pq, precision):
    import torch
    n = tf2.shape[0]
    dev = tf2.device
    out = dict(d=torch.empty(n, dtype=torch.float64, device=dev), ids=torch.empty((n, 2), dtype=torch.int32, device=dev),
               pts=torch.empty((n, 2, 3), dtype=torch.float64, device=dev))
    hs = (C.c_void_p * len(meshes))(*[m.handle.value for m in meshes])
    pairs = np.ascontiguousarray(pairs, np.int32)
    req = N.DistanceRequest(1, api._prec(precision), 0, 0)
    res = N.DistanceResult(out["d"].data_ptr(), out["ids"].data_ptr(), out["pts"].data_ptr(), None, None, None, None,
                           None)
    s = torch.cuda.current_stream(dev).cuda_stream
    rc = N.lib().fclgpu_distance_batch_noalloc(hs, len(meshes), pairs.ctypes.data, pairs.shape[0], n, pq.data_ptr(),
                                               None, tf2.data_ptr(), C.byref(req), C.byref(res), s)
    N.check(rc, "fclgpu_distance_batch_noalloc")
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _check(got, ref):
    rd = ref["min_distance"].cpu().numpy()
    rp = ref["nearest_points"].cpu().numpy()
    ri = ref["ids"].cpu().numpy()
    assert np.all(np.abs(got["d"] - rd) <= np.maximum(REL * np.abs(rd), ABS))
    assert np.all(np.abs(got["pts"] - rp) <= REL * np.maximum(np.abs(rp), 1.0) + ABS)
    sep = rd > 0  # at distance 0 the reported triangles depend on the visit order
    assert np.array_equal(got["ids"][sep], ri[sep])


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_noalloc_distance_matches_allocating_entry_point(gpu_lib, precision):
    import torch
    w = W.config2(total_poses=1500, n_pairs=4, tri_hi=20000, seed=12)
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]
    tf2 = torch.from_numpy(w.tf2).cuda()
    pq = torch.from_numpy(w.pair).cuda()
    ref = api.distance_batch(meshes, w.pairs, None, tf2, pair_of_query=pq, nearest_points=True, precision=precision)
    # a larger call in between: more meshes, more pairs, and another pair mapping
    wb = W.config2(total_poses=3000, n_pairs=9, tri_hi=8000, seed=31)
    mb = [api.BVHModel.from_arrays(v, t) for v, t in wb.meshes]
    pairs_b = np.ascontiguousarray(wb.pairs[::-1], np.int32)
    pq_b = torch.from_numpy((len(pairs_b) - 1 - wb.pair).astype(np.int32)).cuda()
    tf2_b = torch.from_numpy(wb.tf2).cuda()
    ref_b = api.distance_batch(mb, pairs_b, None, tf2_b, pair_of_query=pq_b, nearest_points=True,
                               precision=precision)
    torch.cuda.synchronize()
    _check(_noalloc(meshes, w.pairs, tf2, pq, precision), ref)
    _check(_noalloc(mb, pairs_b, tf2_b, pq_b, precision), ref_b)
    _check(_noalloc(meshes, w.pairs, tf2, pq, precision), ref)


def test_noalloc_rejects_requests_beyond_its_limits(gpu_lib):
    import torch
    w = W.config0(n_poses=4, freq=2)
    m = api.BVHModel.from_arrays(*w.meshes[0])
    tf2 = torch.from_numpy(w.tf2).cuda()
    hs = (C.c_void_p * 65)(*([m.handle.value] * 65))
    pairs = np.zeros((1, 2), np.int32)
    d = torch.empty(4, dtype=torch.float64, device="cuda")
    req = N.DistanceRequest(0, N.FP32_RECHECK, 0, 0)
    res = N.DistanceResult(d.data_ptr(), None, None, None, None, None, None, None)
    rc = N.lib().fclgpu_distance_batch_noalloc(hs, 65, pairs.ctypes.data, 1, 4, None, None, tf2.data_ptr(),
                                               C.byref(req), C.byref(res), None)
    assert rc == -1  # FCLGPU_ERR_INVALID_ARGUMENT: more than 64 meshes
