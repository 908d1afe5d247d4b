"""Front-list collide on the GPU against the oracle's literal restatement (std::list
semantics): the same contacts in the same order, the same new front and the same
statistics, from the roots and propagated to nearby poses, in both precision forms."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

from .test_front_oracle import _perturb

pytestmark = pytest.mark.gpu

BIG = 1 << 30


def _oracle_front(om, pairs, pq, tf2, fronts, maxc):
    outs = []
    for q in range(tf2.shape[0]):
        a, b = om[pairs[pq[q], 0]], om[pairs[pq[q], 1]]
        outs.append(O.collide_front(a, b, tf2[q], front=None if fronts is None else fronts[q],
                                    num_max_contacts=maxc))
    return outs


def _check(g, outs):
    for q, (c, f, nbv, nleaf) in enumerate(outs):
        lo, hi = g["contact_offsets"][q], g["contact_offsets"][q + 1]
        np.testing.assert_array_equal(g["contacts"][lo:hi], c)
        np.testing.assert_array_equal(g["fronts"][q], f)
        assert g["num_bv_tests"][q] == nbv and g["num_leaf_tests"][q] == nleaf


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_front_list_fixture_matches_oracle(gpu_lib, golden, precision):
    env_vt = (golden["env_v"], golden["env_t"])
    rob_vt = (golden["rob_v"], golden["rob_t"])
    meshes = [api.BVHModel.from_arrays(*env_vt), api.BVHModel.from_arrays(*rob_vt)]
    om = [O.Mesh(*env_vt), O.Mesh(*rob_vt)]
    pairs = np.array([[0, 1]], np.int32)
    tf0 = golden["tf"].reshape(-1, 12)
    n = tf0.shape[0]
    pq = np.zeros(n, np.int32)
    g0 = api.collide_front_batch(meshes, pairs, None, tf0, num_max_contacts=BIG, precision=precision,
                                 statistics=True)
    o0 = _oracle_front(om, pairs, pq, tf0, None, BIG)
    _check(g0, o0)
    tf1 = np.stack([_perturb(tf0[i], i).reshape(12) for i in range(n)])
    for maxc in (1, BIG):
        g1 = api.collide_front_batch(meshes, pairs, None, tf1, fronts=g0["fronts"], num_max_contacts=maxc,
                                     precision=precision, statistics=True)
        o1 = _oracle_front(om, pairs, pq, tf1, [o[1] for o in o0], maxc)
        _check(g1, o1)
    assert sum(len(o[0]) for o in o1) > 100


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_front_list_chain_multi_pair(gpu_lib, precision):
    """A chain of three nearby poses per query over several mesh pairs: each call starts
    from the front the previous one returned."""
    w = W.config1(scale=0.002, n_pairs=4, tri_hi=8000, seed=31)
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]
    om = [O.Mesh(v, t) for v, t in w.meshes]
    n = min(w.n, 300)
    pq, tf = w.pair[:n], w.tf2[:n]
    fronts_g = fronts_o = None
    for step in range(3):
        tfs = tf if step == 0 else np.stack([_perturb(tf[i], 7 * step + i, dt=0.02, dr=0.01).reshape(12)
                                             for i in range(n)])
        maxc = BIG if step != 1 else 3
        g = api.collide_front_batch(meshes, w.pairs, None, tfs, fronts=fronts_g, pair_of_query=pq,
                                    num_max_contacts=maxc, precision=precision, statistics=True)
        o = _oracle_front(om, w.pairs, pq, tfs, fronts_o, maxc)
        _check(g, o)
        fronts_g, fronts_o = g["fronts"], [x[1] for x in o]
        tf = tfs
    assert (g["counts"] > 0).any() and (g["counts"] == 0).any()


def test_front_list_mirror(gpu_lib, golden):
    """api.collide_front (collide(node, front_list)): the collision verdict at the new
    pose equals fcl.collide's, as FCL's front-list test checks."""
    env = api.BVHModel.from_arrays(golden["env_v"], golden["env_t"])
    rob = api.BVHModel.from_arrays(golden["rob_v"], golden["rob_t"])
    for i in range(10):
        tf0 = np.array(golden["tf"][i], np.float64).reshape(3, 4)
        tf1 = _perturb(tf0, i)
        fl = api.BVHFrontList()
        r = api.CollisionResult()
        api.collide_front(api.CollisionObject(env, tf0), api.CollisionObject(rob, api.transform()),
                          api.CollisionRequest(num_max_contacts=BIG), r, fl)
        assert fl.size() > 0
        r1, r2 = api.CollisionResult(), api.CollisionResult()
        api.collide_front(api.CollisionObject(env, tf1), api.CollisionObject(rob, api.transform()),
                          api.CollisionRequest(), r1, fl)
        api.collide(api.CollisionObject(env, tf1), api.CollisionObject(rob, api.transform()),
                    api.CollisionRequest(), r2)
        assert r1.isCollision() == r2.isCollision()
