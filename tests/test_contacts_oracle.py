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
        Qm = vb[tb[pairs[:, 1]]] @ tf[q, :, :3].T + tf[q, :, 3]
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
