"""Continuous collision of mesh pairs on the CPU (fcl::continuousCollide, naive solver,
translation / linear / screw motion: continuous_collision-inl.h:134-171,
translation_motion-inl.h, interp_motion-inl.h, screw_motion-inl.h): the
oracle against its definition (the first colliding sample of the discrete collide), the
sample count rule, and the product's motion code (motion.cuh, built for the host)
against the oracle's bit for bit."""
import numpy as np
import pytest

from fcl_gb300 import workloads as W
from oracle import pyoracle as O
from tests import emul as E


def _motions(n, seed, spread=2.5, step=1.0, both=False):
    b0 = W.random_poses(n, -spread, spread, seed)
    b1 = b0.copy()
    rng = np.random.default_rng(seed + 1)
    b1[:, :, 3] += rng.normal(0, step, (n, 3))
    b1[:, :, :3] = W.random_poses(n, 0, 0, seed + 2)[:, :, :3]  # the end rotation is ignored by the motion
    if not both:
        return None, None, b0, b1
    a0 = W.random_poses(n, -0.5, 0.5, seed + 3)
    a1 = a0.copy()
    a1[:, :, 3] += rng.normal(0, step, (n, 3))
    return a0, a1, b0, b1


def _meshes():
    va, ta = W.perturbed_ellipsoid(6, (1, 0.7, 0.5), 0.01, 0)
    vb, tb = W.perturbed_ellipsoid(5, (0.8, 0.56, 0.4), 0.01, 1)
    return O.Mesh(va, ta), O.Mesh(vb, tb)


@pytest.mark.parametrize("kind", ["trans", "linear", "screw"])
@pytest.mark.parametrize("both", [False, True])
@pytest.mark.parametrize("iters,toc_err", [(10, 1e-4), (4, 1e-4), (10, 0.25), (25, 1e-4)])
def test_ccd_is_first_colliding_sample(kind, both, iters, toc_err):
    A, B = _meshes()
    a0, a1, b0, b1 = _motions(150, 7, both=both)
    hit, toc, c1, c2 = O.continuous_collide_batch(A, B, b0, b1, a0, a1, num_max_iterations=iters, toc_err=toc_err,
                                                  nthreads=8, motion=kind)
    n_iter = min(iters, int(np.ceil(1 / toc_err)))
    ts = np.arange(n_iter) / (n_iter - 1)
    n = b0.shape[0]
    ident = np.broadcast_to(W.identity_poses(1), (n, 3, 4))
    first = np.full(n, -1)
    for i, t in enumerate(ts):
        ta = O.motion(ident if a0 is None else a0, ident if a1 is None else a1, np.full(n, t), kind)
        tb = O.motion(b0, b1, np.full(n, t), kind)
        for q in range(n):
            if first[q] < 0:
                c, _, _, _ = O.collide_batch(A, B, tb[q:q + 1], tf1=ta[q:q + 1], num_max_contacts=1)
                if c[0] > 0:
                    first[q] = i
                    assert np.array_equal(c1[q], ta[q]) and np.array_equal(c2[q], tb[q])
    assert np.array_equal(hit, (first >= 0).astype(np.int32))
    assert np.array_equal(toc, np.where(first >= 0, ts[np.maximum(first, 0)], 1.0))
    assert 0 < hit.sum() < n


def test_ccd_without_samples():
    A, B = _meshes()
    _, _, b0, b1 = _motions(20, 3, spread=0.2)
    hit, toc, _, _ = O.continuous_collide_batch(A, B, b0, b1, num_max_iterations=0)
    assert hit.sum() == 0 and np.all(toc == 1.0)


def test_translation_motion_quaternion_round_trip():
    # the motion's rotation is Quaternion(R_beg).toRotationMatrix() at every t: equal to
    # R_beg within rounding, bit-identical across t; the translation is start + range t
    _, _, b0, b1 = _motions(500, 11)
    for t in (0.0, 1 / 3, 1.0):
        f = O.translation_motion(b0, b1, np.full(500, t))
        assert np.allclose(f[:, :, :3], b0[:, :, :3], atol=1e-14)
        assert np.array_equal(f[:, :, 3], b0[:, :, 3] + (b1[:, :, 3] - b0[:, :, 3]) * t)
    f0 = O.translation_motion(b0, b1, np.zeros(500))
    f1 = O.translation_motion(b0, b1, np.ones(500))
    assert np.array_equal(f0[:, :, :3], f1[:, :, :3])


@pytest.mark.parametrize("kind", ["trans", "linear", "screw"])
def test_product_motion_bit_exact(kind):
    _, _, b0, b1 = _motions(2000, 13)
    b1[:200, :, :3] = b0[:200, :, :3]   # no rotation: the screw's translation-only branch
    # rotations with a non-positive trace take the largest-diagonal branch of the
    # matrix -> quaternion conversion
    t = np.random.default_rng(0).uniform(0, 1.2, 2000)
    ref = O.motion(b0, b1, t, kind)
    got = E.motion(b0, b1, t, kind)
    assert np.array_equal(ref.view(np.uint64), got.view(np.uint64))
    tr = b0[:, 0, 0] + b0[:, 1, 1] + b0[:, 2, 2]
    assert (tr <= 0).sum() > 100 and (tr > 0).sum() > 100


@pytest.mark.parametrize("kind", ["linear", "screw"])
def test_rotating_motions_run_from_start_to_end(kind):
    _, _, b0, b1 = _motions(500, 17)
    f0 = O.motion(b0, b1, np.zeros(500), kind)
    f1 = O.motion(b0, b1, np.ones(500), kind)
    assert np.allclose(f0, b0, atol=1e-13) and np.allclose(f1, b1, atol=1e-12)
    # the rotation angle of R(t) R(0)^T grows linearly in t about a fixed axis
    fh = O.motion(b0, b1, np.full(500, 0.5), kind)
    rel = np.einsum("nij,nkj->nik", fh[:, :, :3], b0[:, :, :3])
    relf = np.einsum("nij,nkj->nik", b1[:, :, :3], b0[:, :, :3])
    ang = np.arccos(np.clip((np.trace(rel, axis1=1, axis2=2) - 1) / 2, -1, 1))
    angf = np.arccos(np.clip((np.trace(relf, axis1=1, axis2=2) - 1) / 2, -1, 1))
    assert np.allclose(ang, angf / 2, atol=1e-9)


def test_screw_without_rotation_keeps_fcl_scaling():
    """ScrewMotion with a rotation angle below 1e-10 takes axis = t2 - t1 unnormalised and
    linear_vel = |t2 - t1| (screw_motion-inl.h computeScrewParameter), so the translation
    at t is t1 + (t2 - t1) t |t2 - t1|; the restatement keeps that."""
    b0 = W.random_poses(50, -1, 1, 23)
    b1 = b0.copy()
    b1[:, :, 3] += np.random.default_rng(5).normal(0, 1, (50, 3))
    f = O.motion(b0, b1, np.full(50, 0.5), "screw")
    d = b1[:, :, 3] - b0[:, :, 3]
    assert np.allclose(f[:, :, 3], b0[:, :, 3] + d * (0.5 * np.linalg.norm(d, axis=1))[:, None], atol=1e-12)


def test_conservative_advancement_oracle_properties():
    """The oracle's conservative advancement (FCL's oriented OBBRSS node): a contact it
    reports lies within the last step's reach of touching, its time is within one
    fine-sampling step of the first colliding sample for these smooth translations, and a
    motion that never collides runs to t = 1."""
    va, ta = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 1)
    vb, tb = W.perturbed_ellipsoid(5, (0.5, 0.4, 0.6), 0.01, 2)
    A, B = O.Mesh(va, ta), O.Mesh(vb, tb)
    n = 12
    b0 = W.random_poses(n, -3, 3, 5)
    b1 = b0.copy()
    b1[:, :, 3] = -b1[:, :, 3]  # through the other mesh
    hit, toc, _, c2, it = O.ca_batch(A, B, b0, b1, nthreads=4)
    assert hit.all() and (it >= 2).all()
    d, _, _, _, _ = O.distance_batch(A, B, c2)
    assert (d < 1e-4).all()
    ts = np.linspace(0, 1, 801)
    for q in range(n):
        poses = O.motion(np.repeat(b0[q].reshape(1, 12), ts.size, 0), np.repeat(b1[q].reshape(1, 12), ts.size, 0), ts)
        c, _, _, _ = O.collide_batch(A, B, poses.reshape(-1, 12), num_max_contacts=1)
        first = ts[np.argmax(c > 0)]
        assert abs(toc[q] - first) <= 2.5e-3
    far = b0.copy()
    far[:, :, 3] += 20.0
    far1 = far.copy()
    far1[:, 0, 3] += 1.0
    hit, toc, _, _, _ = O.ca_batch(A, B, far, far1)
    assert not hit.any() and (toc == 1.0).all()
