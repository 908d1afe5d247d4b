"""Continuous collision of mesh pairs on the GPU (fcl::continuousCollide, naive solver)
against the FP64 oracle: with the translation motion the collision flags, times of contact
and the transforms at the time of contact bit for bit, through the host and device entry
points and the fcl mirror; with the linear and screw motions the flags and times exactly and
the transforms to 1e-12."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import native as N
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _meshes():
    va, ta = W.perturbed_ellipsoid(10, (1, 0.7, 0.5), 0.01, 0)
    vb, tb = W.perturbed_ellipsoid(8, (0.8, 0.56, 0.4), 0.01, 1)
    return (va, ta), (vb, tb)


def _motions(n, seed, both):
    b0 = W.random_poses(n, -2.5, 2.5, seed)
    b1 = b0.copy()
    rng = np.random.default_rng(seed + 1)
    b1[:, :, 3] += rng.normal(0, 1.0, (n, 3))
    if not both:
        return None, None, b0, b1
    a0 = W.random_poses(n, -0.5, 0.5, seed + 3)
    a1 = a0.copy()
    a1[:, :, 3] += rng.normal(0, 1.0, (n, 3))
    return a0, a1, b0, b1


def _same(g, ref):
    hit, toc, c1, c2 = ref
    assert np.array_equal(np.asarray(g["is_collide"]), hit)
    assert np.array_equal(np.asarray(g["time_of_contact"]), toc)
    assert np.array_equal(np.asarray(g["contact_tf1"]).view(np.uint64), c1.view(np.uint64))
    assert np.array_equal(np.asarray(g["contact_tf2"]).view(np.uint64), c2.view(np.uint64))


@pytest.mark.parametrize("both", [False, True])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("iters,toc_err", [(10, 1e-4), (10, 0.25), (0, 1e-4)])
def test_ccd_matches_oracle(gpu_lib, both, prec, iters, toc_err):
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(700, 5, both)
    ref = O.continuous_collide_batch(O.Mesh(va, ta), O.Mesh(vb, tb), b0, b1, a0, a1, num_max_iterations=iters,
                                     toc_err=toc_err, nthreads=8)
    g = api.continuous_collide_batch([A, B], [[0, 1]], a0, a1, b0, b1, num_max_iterations=iters, toc_err=toc_err,
                                     precision=prec)
    _same(g, ref)
    if iters:
        assert 0 < ref[0].sum() < len(b0)


@pytest.mark.parametrize("kind", ["linear", "screw"])
def test_ccd_rotating_motions(gpu_lib, kind):
    """The linear and screw motions call sin/cos/tan/atan2, whose device results differ
    from the host's in the last bits: the sampled transforms agree with the oracle's to
    1e-12, the collision flags and times of contact exactly (no sampled pose of this
    workload lies within rounding of touching)."""
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(700, 31, True)
    b1[:, :, :3] = W.random_poses(700, 0, 0, 32)[:, :, :3]
    ref = O.continuous_collide_batch(O.Mesh(va, ta), O.Mesh(vb, tb), b0, b1, a0, a1, nthreads=8, motion=kind)
    g = api.continuous_collide_batch([A, B], [[0, 1]], a0, a1, b0, b1, motion=kind)
    assert np.array_equal(g["is_collide"], ref[0]) and np.array_equal(g["time_of_contact"], ref[1])
    assert np.allclose(g["contact_tf1"], ref[2], rtol=0, atol=1e-12)
    assert np.allclose(g["contact_tf2"], ref[3], rtol=0, atol=1e-12)
    assert 0 < ref[0].sum() < 700


def test_ccd_device_entry_and_mixed_pairs(gpu_lib):
    import torch
    (va, ta), (vb, tb) = _meshes()
    vc, tc = W.grid_box(4)
    geo = [(va, ta), (vb, tb), (vc, tc)]
    ms = [api.BVHModel.from_arrays(v, t) for v, t in geo]
    os_ = [O.Mesh(v, t) for v, t in geo]
    pairs = np.array([[0, 1], [2, 1], [0, 2]], np.int32)
    a0, a1, b0, b1 = _motions(600, 9, True)
    pq = np.random.default_rng(2).integers(0, 3, 600).astype(np.int32)
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    g = api.continuous_collide_batch(ms, pairs, d(a0), d(a1), d(b0), d(b1), pair_of_query=d(pq))
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy() for k, v in g.items()}
    for p in range(3):
        sel = np.nonzero(pq == p)[0]
        ref = O.continuous_collide_batch(os_[pairs[p, 0]], os_[pairs[p, 1]], b0[sel], b1[sel], a0[sel], a1[sel],
                                         nthreads=8)
        _same({k: v[sel] for k, v in g.items()}, ref)


def test_ccd_rejects_what_fcl_cannot_run_here(gpu_lib):
    (va, ta), (vb, tb) = _meshes()
    ms = [api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)]
    _, _, b0, b1 = _motions(4, 1, False)
    for kw in ({"motion": "spline"}, {"solver": "ray_shooting"}, {"solver": "polynomial_solver"},
               {"motion": "spline", "solver": "conservative_advancement"}):
        with pytest.raises(N.FclGpuError) as e:
            api.continuous_collide_batch(ms, [[0, 1]], None, None, b0, b1, **kw)
        assert e.value.code == N.FCLGPU_ERR_UNSUPPORTED
    with pytest.raises(N.FclGpuError):   # one sample: FCL divides 0 by 0
        api.continuous_collide_batch(ms, [[0, 1]], None, None, b0, b1, num_max_iterations=1)


def test_continuous_collide_mirror(gpu_lib):
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(60, 21, True)
    ref = O.continuous_collide_batch(O.Mesh(va, ta), O.Mesh(vb, tb), b0, b1, a0, a1)
    for q in range(60):
        res = api.ContinuousCollisionResult()
        t = api.continuousCollide(api.CollisionObject(A, a0[q]), a1[q], api.CollisionObject(B, b0[q]), b1[q],
                                  api.ContinuousCollisionRequest(), res)
        assert t == ref[1][q] and res.is_collide == bool(ref[0][q])
        if res.is_collide:
            assert np.array_equal(res.contact_tf1, ref[2][q]) and np.array_equal(res.contact_tf2, ref[3][q])


@pytest.mark.parametrize("both", [False, True])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_conservative_advancement_matches_oracle(gpu_lib, both, prec):
    """Conservative advancement with the translation motion: flags, times of contact,
    transforms at contact and the number of traversals bit for bit against the oracle's
    restatement of FCL's oriented OBBRSS node (the start collide runs in either form)."""
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(400, 41, both)
    ref = O.ca_batch(O.Mesh(va, ta), O.Mesh(vb, tb), b0, b1, a0, a1, nthreads=8)
    g = api.continuous_collide_batch([A, B], [[0, 1]], a0, a1, b0, b1, solver="conservative_advancement",
                                     precision=prec)
    _same(g, ref[:4])
    assert np.array_equal(g["iterations"], ref[4])
    assert 0 < ref[0].sum() < 400 and ref[4].max() >= 3


@pytest.mark.parametrize("kind", ["linear", "screw"])
def test_conservative_advancement_rotating_motions(gpu_lib, kind):
    """With the linear and screw motions (sin/cos/tan/atan2 differ from the host's in the
    last bits) the times of contact agree with the oracle's to 1e-9 and the flags exactly."""
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(300, 43, True)
    b1[:, :, :3] = W.random_poses(300, 0, 0, 44)[:, :, :3]
    ref = O.ca_batch(O.Mesh(va, ta), O.Mesh(vb, tb), b0, b1, a0, a1, motion=kind, nthreads=8)
    g = api.continuous_collide_batch([A, B], [[0, 1]], a0, a1, b0, b1, solver="conservative_advancement",
                                     motion=kind)
    assert np.array_equal(g["is_collide"], ref[0])
    assert np.allclose(g["time_of_contact"], ref[1], rtol=0, atol=1e-9)
    assert np.allclose(g["contact_tf2"], ref[3], rtol=0, atol=1e-9)
    assert 0 < ref[0].sum() < 300


def test_conservative_advancement_mirror_and_contact_distance(gpu_lib):
    """api.continuousCollide with CCDC_CONSERVATIVE_ADVANCEMENT equals the batch; at a
    reported time of contact the meshes are within the last step's reach of touching (the
    oracle's distance at the contact transforms is below 1e-4)."""
    (va, ta), (vb, tb) = _meshes()
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    a0, a1, b0, b1 = _motions(60, 45, True)
    batch = api.continuous_collide_batch([A, B], [[0, 1]], a0, a1, b0, b1, solver="conservative_advancement")
    req = api.ContinuousCollisionRequest(ccd_solver_type="conservative_advancement")
    MA, MB = O.Mesh(va, ta), O.Mesh(vb, tb)
    for q in range(60):
        res = api.ContinuousCollisionResult()
        t = api.continuousCollide(api.CollisionObject(A, a0[q]), a1[q], api.CollisionObject(B, b0[q]), b1[q], req,
                                  res)
        assert t == batch["time_of_contact"][q] and res.is_collide == bool(batch["is_collide"][q])
        if res.is_collide:
            d, _, _, _, _ = O.distance_batch(MA, MB, res.contact_tf2[None], res.contact_tf1[None])
            assert d[0] < 1e-4
    assert batch["is_collide"].sum() > 0
