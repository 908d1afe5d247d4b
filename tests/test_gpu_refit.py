"""Device refit of a BVHModel<OBBRSS> after vertex updates (beginUpdateModel /
updateVertex / endUpdateModel(), bottom-up) against the FP64 oracle: the refitted
nodes bit for bit, then collide and distance on the refitted models."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import native as N
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _frames(seed, freq=8):
    v, t = W.perturbed_ellipsoid(freq, (1.0, 0.7, 0.5), 0.01, seed)
    rng = np.random.default_rng(seed + 7)
    v1 = v + rng.normal(0, 0.02, v.shape)                      # deformation
    R = W.random_poses(1, -0.3, 0.3, seed)[0]
    v2 = v1 @ R[:, :3].T + R[:, 3] + rng.normal(0, 0.01, v.shape)  # moved and deformed again
    return v, t, v1, v2


@pytest.mark.parametrize("seed", [0, 1])
def test_refit_nodes_bit_exact(gpu_lib, seed):
    v, t, v1, v2 = _frames(seed)
    g = api.BVHModel.from_arrays(v, t)
    o = O.Mesh(v, t)
    # the FCL update protocol on the first frame, the one-call form on the second
    assert g.beginUpdateModel() == 0
    for p in v1:
        g.updateVertex(p)
    assert g.endUpdateModel() == 0
    o.update(v1)
    gn, gfc = g.get_nodes()
    on, ofc = o.nodes()
    assert np.array_equal(gfc, ofc)
    assert np.array_equal(gn.view(np.uint64), on.view(np.uint64))
    g.update_vertices(v2)
    o.update(v2)
    gn, gfc = g.get_nodes()
    on, ofc = o.nodes()
    assert np.array_equal(gn.view(np.uint64), on.view(np.uint64))


def test_refit_from_device_pointer(gpu_lib):
    import torch
    v, t, v1, _ = _frames(3)
    g = api.BVHModel.from_arrays(v, t)
    o = O.Mesh(v, t)
    g.update_vertices(torch.from_numpy(v1).cuda())
    torch.cuda.synchronize()
    o.update(v1)
    assert np.array_equal(g.get_nodes()[0].view(np.uint64), o.nodes()[0].view(np.uint64))


def test_collide_and_distance_on_refitted_models(gpu_lib):
    va, ta, va1, _ = _frames(4, freq=10)
    vb, tb, vb1, _ = _frames(5, freq=6)
    ga, gb = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    oa, ob = O.Mesh(va, ta), O.Mesh(vb, tb)
    ga.update_vertices(va1); oa.update(va1)
    gb.update_vertices(vb1); ob.update(vb1)
    tf = W.random_poses(600, -1.0, 1.0, 9)
    for prec in ("fp32", "fp64"):
        g = api.collide_batch([ga, gb], [[0, 1]], None, tf, num_max_contacts=1000, precision=prec)
        c, ct, _, _ = O.collide_batch(oa, ob, tf, num_max_contacts=1000, nthreads=8)
        assert np.array_equal(g["counts"], c)
        assert np.array_equal(g["contacts"], ct)
    far = W.random_poses(400, 1.8, 3.0, 10)
    d, ids, pts, _, _ = O.distance_batch(oa, ob, far, nearest=True, nthreads=8)
    g64 = api.distance_batch([ga, gb], [[0, 1]], None, far, nearest_points=True, precision="fp64")
    assert np.array_equal(g64["min_distance"], d) and np.array_equal(g64["ids"], ids)
    g32 = api.distance_batch([ga, gb], [[0, 1]], None, far, nearest_points=True, precision="fp32")
    assert np.all(np.abs(g32["min_distance"] - d) <= np.maximum(REL * np.abs(d), ABS))


def test_update_with_wrong_vertex_count(gpu_lib):
    v, t, v1, _ = _frames(6, freq=3)
    g = api.BVHModel.from_arrays(v, t)
    with pytest.raises(N.FclGpuError) as e:
        g.update_vertices(v1[:-1])
    assert e.value.code == N.FCLGPU_ERR_INCORRECT_DATA
    assert g.beginUpdateModel() == 0
    g.updateSubModel(v1[:-1])
    assert g.endUpdateModel() == -7  # BVH_ERR_INCORRECT_DATA, as FCL's endUpdateModel


def test_replace_model_bit_exact(gpu_lib):
    """beginReplaceModel / replaceVertex / endReplaceModel(): leaves refitted to the new
    triangle alone (fit3), then an update on top, against the oracle bit for bit."""
    v, t, v1, v2 = _frames(8)
    g = api.BVHModel.from_arrays(v, t)
    o = O.Mesh(v, t)
    assert g.beginReplaceModel() == 0
    for p in v1:
        g.replaceVertex(p)
    assert g.endReplaceModel() == 0
    o.replace(v1)
    assert np.array_equal(g.get_nodes()[0].view(np.uint64), o.nodes()[0].view(np.uint64))
    g.update_vertices(v2)
    o.update(v2)
    assert np.array_equal(g.get_nodes()[0].view(np.uint64), o.nodes()[0].view(np.uint64))
    # the top-down refit stays off the GPU path; refit = False rebuilds
    # (tests/test_gpu_build.py)
    with pytest.raises(N.FclGpuError) as e:
        assert g.beginReplaceModel() == 0
        g.replaceSubModel(v1)
        g.endReplaceModel(bottomup=False)
    assert e.value.code == N.FCLGPU_ERR_UNSUPPORTED
