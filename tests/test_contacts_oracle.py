"""Contact information of mesh-mesh collide (CollisionRequest::enable_contact = true) on
the CPU: the oracle's restatement against hand-derived answers of the reference's
algorithm (intersect-inl.h:800-886), its traversal against the contact-free one, the
num_max_contacts truncation rule (mesh_collision_traversal_node-inl.h:579-600), and the
product's contact code (tri_contact.cuh, built for the host) against the oracle bit for
bit."""
import numpy as np
import pytest

from fcl_gb300 import workloads as W
from oracle import pyoracle as O
from tests import emul as E

P_FLAT = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
Q_SLANT = np.array([[0.2, 0.2, -0.1], [0.3, 0.2, 0.5], [0.2, 0.3, 0.5]])
Q_TWO = np.array([[0.2, 0.2, -0.1], [0.4, 0.2, -0.1], [0.3, 0.3, 0.5]])


def test_tri_contact_known_answers():
    # Q_SLANT pokes 0.1 below P_FLAT's plane with one vertex; P_FLAT reaches 0.41 below
    # Q_SLANT's plane, so the contact is Q's deepest vertex with P's normal.  Q_TWO has
    # two vertices at the same depth: two contacts.  With the roles swapped the
    # shallower side is the first triangle's: its vertex, and the second normal negated.
    cnt, pts, nrm, dep = O.tri_contact_batch(np.stack([P_FLAT, P_FLAT, Q_SLANT]),
                                             np.stack([Q_SLANT, Q_TWO, P_FLAT]))
    assert list(cnt) == [1, 2, 1]
    assert np.allclose(pts[0, 0], [0.2, 0.2, -0.1], atol=1e-15)
    assert np.allclose(pts[1], [[0.2, 0.2, -0.1], [0.4, 0.2, -0.1]], atol=1e-15)
    assert np.allclose(pts[2, 0], [0.2, 0.2, -0.1], atol=1e-15)
    assert np.array_equal(nrm[:2], [[0, 0, 1], [0, 0, 1]])
    assert np.array_equal(nrm[2], [0, 0, -1])
    assert np.allclose(dep, 0.1, atol=1e-15)


def _move(Q, tf):
    """R Q + T with the oracle's summation order ((r0 x + r1 y) + r2 z) + t."""
    R, T = tf[:, :3], tf[:, 3]
    out = np.empty_like(Q)
    for r in range(3):
        out[..., r] = ((R[r, 0] * Q[..., 0] + R[r, 1] * Q[..., 1]) + R[r, 2] * Q[..., 2]) + T[r]
    return out


def _pairs(c, ct):
    off = np.concatenate([[0], np.cumsum(c)])
    return [ct[off[i]:off[i + 1]] for i in range(len(c))]


def _meshes(kind):
    if kind == "ellipsoid":
        va, ta = W.perturbed_ellipsoid(6, (1, 0.7, 0.5), 0.01, 0)
        vb, tb = W.perturbed_ellipsoid(5, (0.8, 0.56, 0.4), 0.01, 1)
        tf = W.random_poses(200, -1.0, 1.0, 3)
    else:
        va, ta = W.grid_box(4)
        vb, tb = W.grid_box(3, (0.3, 0.4, 0.35))
        rng = np.random.default_rng(0)
        tf = W.identity_poses(200)
        tf[:, :, 3] = rng.uniform(-0.8, 0.8, (200, 3))
    return (va, ta), (vb, tb), tf


@pytest.mark.parametrize("kind", ["ellipsoid", "grid_box"])
def test_contact_traversal_visits_the_same_pairs(kind):
    (va, ta), (vb, tb), tf = _meshes(kind)
    A, B = O.Mesh(va, ta), O.Mesh(vb, tb)
    big = 10 ** 7
    c, ct, _, _ = O.collide_batch(A, B, tf, num_max_contacts=big)
    cc, ids, pos, nrm, dep = O.collide_contacts_batch(A, B, tf, num_max_contacts=big)
    two = 0
    for q, (pairs, got) in enumerate(zip(_pairs(c, ct), _pairs(cc, ids))):
        # every intersecting pair, in DFS order, contributes its tri_contact count
        P = va[ta[pairs[:, 0]]]
        Qm = _move(vb[tb[pairs[:, 1]]], tf[q])
        k, _, _, _ = O.tri_contact_batch(P, Qm)
        assert np.array_equal(np.repeat(pairs, k, axis=0), got)
        two += int((k == 2).sum())
    if kind == "grid_box":
        assert two > 100   # parallel faces: many pairs with two contact points
    assert np.all(np.isfinite(pos)) and np.all(np.abs(np.linalg.norm(nrm, axis=1) - 1) < 1e-12)


def test_contact_cap_truncates_a_prefix():
    (va, ta), (vb, tb), tf = _meshes("grid_box")
    A, B = O.Mesh(va, ta), O.Mesh(vb, tb)
    full = O.collide_contacts_batch(A, B, tf, num_max_contacts=10 ** 7)
    foff = np.concatenate([[0], np.cumsum(full[0])])
    for cap in (1, 2, 3, 5, 11):
        got = O.collide_contacts_batch(A, B, tf, num_max_contacts=cap)
        assert np.array_equal(got[0], np.minimum(full[0], cap))
        goff = np.concatenate([[0], np.cumsum(got[0])])
        for q in range(len(tf)):
            for a, b in zip(got[1:], full[1:]):
                assert np.array_equal(a[goff[q]:goff[q + 1]], b[foff[q]:foff[q] + got[0][q]])


def _tri_pairs(seed, n=4000):
    rng = np.random.default_rng(seed)
    P = rng.uniform(-1, 1, (n, 3, 3))
    Qm = P.mean(axis=1, keepdims=True) + rng.uniform(-0.6, 0.6, (n, 3, 3))
    # ties: axis-aligned triangles with two vertices at the same height
    m = n // 4
    P[:m, :, 2] = 0.0
    Qm[:m, 0, 2] = Qm[:m, 1, 2] = rng.uniform(-0.2, 0.0, m)
    # a degenerate (zero-area) triangle: the zero plane
    P[m:m + 10, 2] = P[m:m + 10, 1]
    return P, Qm


@pytest.mark.parametrize("seed", [0, 1])
def test_product_tri_contact_bit_exact(seed):
    P, Qm = _tri_pairs(seed)
    ref = O.tri_contact_batch(P, Qm)
    got = E.tri_contact_batch(P, Qm)
    assert np.array_equal(ref[0], got[0])
    for a, b in zip(ref[1:], got[1:]):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert set(np.unique(ref[0])) >= {1, 2}


@pytest.mark.parametrize("i", [0, 3, 7])
def test_reference_fixture_contact_mode(golden, i):
    """FCL's collision test runs with enable_contact = true and num_max_contacts = INT_MAX
    (test_fcl_collision.cpp:74-75) and compares sorted contact lists across BV types; the
    OBBRSS list here holds every intersecting triangle pair (the brute-force set) once per
    contact point of the pair."""
    env = O.Mesh(golden["env_v"], golden["env_t"])
    rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    tf = golden["tf"][i]
    cnt, ids, pos, nrm, dep = O.collide_contacts_batch(env, rob, tf[None], num_max_contacts=2 ** 31 - 1)
    brute = O.brute_collide(env, rob, tf)
    assert sorted(set(map(tuple, ids))) == sorted(map(tuple, brute))
    P = golden["env_v"][golden["env_t"][ids[:, 0]]]
    Qm = _move(golden["rob_v"][golden["rob_t"][ids[:, 1]]], tf)
    k, _, _, d = O.tri_contact_batch(P, Qm)
    uniq, first, mult = np.unique(ids, axis=0, return_index=True, return_counts=True)
    assert np.array_equal(mult, k[first])
    assert np.array_equal(dep, d) and np.all(dep >= -1e-5)
