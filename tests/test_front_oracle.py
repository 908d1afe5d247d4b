"""Front-list (temporal coherence) collide in the oracle: FCL's front-list test
(test_fcl_frontlist.cpp:68-196) on its env.obj x rob.obj fixture -- a front built at one
pose, propagated to a nearby pose, must report a collision exactly when the plain
traversal does -- and the stronger set properties the algorithm implies."""
import numpy as np
import pytest

from oracle import pyoracle as O


def _perturb(tf, k, dt=1.0, dr=0.005 * 2 * np.pi):
    """A nearby pose as test::generateRandomTransforms(extents, delta_trans, delta_rot)
    draws it: translation moved by up to dt per axis, rotation by up to dr per Euler
    angle (seeded)."""
    rng = np.random.default_rng(1000 + k)
    a = rng.uniform(-dr, dr, 3)
    cx, cy, cz = np.cos(a)
    sx, sy, sz = np.sin(a)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    out = np.array(tf, np.float64).reshape(3, 4).copy()
    out[:, :3] = out[:, :3] @ (Rx @ Ry @ Rz)
    out[:, 3] += rng.uniform(-dt, dt, 3)
    return out


@pytest.mark.parametrize("i", range(10))
def test_front_list_fixture(golden, i):
    env = O.Mesh(golden["env_v"], golden["env_t"])
    rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    tf0 = golden["tf"][i]
    tf1 = _perturb(tf0, i)
    big = 1 << 30
    # the front of an exhaustive traversal at tf0, as the test builds it
    c0, front, _, _ = O.collide_front(env, rob, tf0, num_max_contacts=big)
    plain0, ct0, _, _ = O.collide_batch(env, rob, tf0[None], num_max_contacts=big)
    assert sorted(map(tuple, c0)) == sorted(map(tuple, ct0))  # no early stop: the full set
    assert front.shape[0] > 0
    # propagated to the nearby pose with the default request (one contact)
    c1, _, _, _ = O.collide_front(env, rob, tf1, front=front, num_max_contacts=1)
    plain1, ct1, _, _ = O.collide_batch(env, rob, tf1[None], num_max_contacts=1)
    assert (len(c1) > 0) == (plain1[0] > 0)
    # exhaustively: the same contact set (a leaf reached from an overlapping front node
    # is tested twice, so pairs may repeat)
    c1x, front1, _, _ = O.collide_front(env, rob, tf1, front=front, num_max_contacts=big)
    _, ct1x, _, _ = O.collide_batch(env, rob, tf1[None], num_max_contacts=big)
    assert set(map(tuple, c1x)) == set(map(tuple, ct1x))
    # propagating again at the same pose keeps the contact set
    c2, _, _, _ = O.collide_front(env, rob, tf1, front=front1, num_max_contacts=big)
    assert set(map(tuple, c2)) == set(map(tuple, ct1x))
