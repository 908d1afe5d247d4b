"""Mesh-mesh collide with CollisionRequest::enable_contact = true on the GPU against the
FP64 oracle: the contact lists (b1, b2 in DFS order), counts under num_max_contacts,
and the contact positions, normals and depths bit for bit, through the host and the
device entry points and the fcl::collide mirror."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import native as N
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _case(kind):
    if kind == "ellipsoid":
        va, ta = W.perturbed_ellipsoid(10, (1, 0.7, 0.5), 0.01, 0)
        vb, tb = W.perturbed_ellipsoid(8, (0.8, 0.56, 0.4), 0.01, 1)
        tf2 = W.random_poses(800, -1.0, 1.0, 3)
        tf1 = W.random_poses(800, -0.5, 0.5, 4)
    else:  # flat faces: many triangle pairs with two contact points
        va, ta = W.grid_box(5)
        vb, tb = W.grid_box(4, (0.3, 0.4, 0.35))
        rng = np.random.default_rng(0)
        tf2 = W.identity_poses(400)
        tf2[:, :, 3] = rng.uniform(-0.8, 0.8, (400, 3))
        tf1 = W.random_poses(400, -0.5, 0.5, 5)
    return (va, ta), (vb, tb), tf1, tf2


def _same(g, ref):
    counts, ids, pos, nrm, dep = ref
    assert np.array_equal(np.asarray(g["counts"]), counts)
    assert g["total_contacts"] == counts.sum()
    assert np.array_equal(np.asarray(g["contacts"]), ids)
    for key, r in (("pos", pos), ("normal", nrm), ("depth", dep)):
        a = np.asarray(g[key])
        assert np.array_equal(a.view(np.uint64), r.view(np.uint64)), key


@pytest.mark.parametrize("kind", ["ellipsoid", "grid_box"])
@pytest.mark.parametrize("cap", [1, 3, 10 ** 6])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_contacts_match_oracle(gpu_lib, kind, cap, prec):
    (va, ta), (vb, tb), tf1, tf2 = _case(kind)
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    ref = O.collide_contacts_batch(O.Mesh(va, ta), O.Mesh(vb, tb), tf2, tf1=tf1, num_max_contacts=cap, nthreads=8)
    g = api.collide_contacts_batch([A, B], [[0, 1]], tf1, tf2, num_max_contacts=cap, precision=prec)
    _same(g, ref)


def test_contacts_device_entry_point(gpu_lib):
    import torch
    (va, ta), (vb, tb), tf1, tf2 = _case("grid_box")
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    ref = O.collide_contacts_batch(O.Mesh(va, ta), O.Mesh(vb, tb), tf2, tf1=tf1, num_max_contacts=5, nthreads=8)
    api._contacts_hint["cap"] = 16   # forces the capacity retry
    g = api.collide_contacts_batch([A, B], [[0, 1]], torch.from_numpy(tf1).cuda(), torch.from_numpy(tf2).cuda(),
                                   num_max_contacts=5)
    torch.cuda.synchronize()
    _same({k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in g.items()}, ref)


def test_contacts_mixed_pairs_and_empty(gpu_lib):
    (va, ta), (vb, tb), _, _ = _case("ellipsoid")
    (vc, tc), _, _, _ = _case("grid_box")
    ms = [api.BVHModel.from_arrays(v, t) for v, t in ((va, ta), (vb, tb), (vc, tc))]
    os_ = [O.Mesh(v, t) for v, t in ((va, ta), (vb, tb), (vc, tc))]
    pairs = np.array([[0, 1], [2, 1], [0, 2]], np.int32)
    tf2 = W.random_poses(600, -1.2, 1.2, 9)
    pq = np.random.default_rng(1).integers(0, 3, 600).astype(np.int32)
    g = api.collide_contacts_batch(ms, pairs, None, tf2, pair_of_query=pq, num_max_contacts=7)
    off = np.asarray(g["offsets"])
    for p in range(3):
        sel = np.nonzero(pq == p)[0]
        ref = O.collide_contacts_batch(os_[pairs[p, 0]], os_[pairs[p, 1]], tf2[sel], num_max_contacts=7, nthreads=8)
        rows = np.concatenate([np.arange(off[q], off[q + 1]) for q in sel]).astype(np.int64)
        _same({"counts": g["counts"][sel], "total_contacts": int(ref[0].sum()), "contacts": g["contacts"][rows],
               "pos": g["pos"][rows], "normal": g["normal"][rows], "depth": g["depth"][rows]}, ref)
    empty = api.collide_contacts_batch(ms, pairs, None, tf2[:0], num_max_contacts=7)
    assert empty["total_contacts"] == 0 and len(empty["counts"]) == 0


def test_fcl_collide_mirror_with_contacts(gpu_lib):
    (va, ta), (vb, tb), tf1, tf2 = _case("grid_box")
    A, B = api.BVHModel.from_arrays(va, ta), api.BVHModel.from_arrays(vb, tb)
    o1, o2 = api.CollisionObject(A, tf1[0]), api.CollisionObject(B, tf2[0])
    req = api.CollisionRequest(num_max_contacts=4, enable_contact=True)
    res = api.CollisionResult()
    n = api.collide(o1, o2, req, res)
    counts, ids, pos, nrm, dep = O.collide_contacts_batch(O.Mesh(va, ta), O.Mesh(vb, tb), tf2[:1], tf1=tf1[:1],
                                                          num_max_contacts=4)
    assert n == counts[0] == res.numContacts()
    for i, c in enumerate(res.contacts):
        assert (c.b1, c.b2) == tuple(ids[i])
        assert np.array_equal(c.pos, pos[i]) and np.array_equal(c.normal, nrm[i])
        assert c.penetration_depth == dep[i]
    with pytest.raises(N.FclGpuError):
        api.collide(o1, o2, api.CollisionRequest(num_max_contacts=4, enable_contact=True, enable_statistics=True),
                    api.CollisionResult())


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_contacts_on_reference_fixture(gpu_lib, golden, prec):
    """FCL's collision test setting (enable_contact = true, num_max_contacts = INT_MAX,
    test_fcl_collision.cpp:74-75) on its env.obj / rob.obj fixture and poses: contact lists
    and geometry equal the oracle's bit for bit."""
    ms = [api.BVHModel.from_arrays(golden["env_v"], golden["env_t"]),
          api.BVHModel.from_arrays(golden["rob_v"], golden["rob_t"])]
    tf = golden["tf"]
    g = api.collide_contacts_batch(ms, [[0, 1]], None, tf, num_max_contacts=2 ** 31 - 1, precision=prec)
    ref = O.collide_contacts_batch(O.Mesh(golden["env_v"], golden["env_t"]),
                                   O.Mesh(golden["rob_v"], golden["rob_t"]), tf, num_max_contacts=2 ** 31 - 1)
    _same(g, ref)
    assert ref[0].sum() > 0
