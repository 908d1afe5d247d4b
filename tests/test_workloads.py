import numpy as np

from fcl_gb300 import workloads as W


def test_geodesic_counts():
    for f in (1, 2, 5, 16):
        v, t = W.geodesic_sphere(f)
        assert t.shape[0] == 20 * f * f
        assert v.shape[0] == 10 * f * f + 2
        assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
        # closed 2-manifold: every edge shared by exactly two triangles
        e = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert np.all(cnt == 2)


def test_haar_rotations_orthonormal():
    tf = W.random_poses(1000, -2, 2, 0)
    R = tf[:, :, :3]
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-12)
    assert np.allclose(np.linalg.det(R), 1.0)
    assert tf[:, :, 3].min() >= -2 and tf[:, :, 3].max() <= 2


def test_config_shapes():
    w = W.config0(n_poses=100)
    assert w.meshes[0][1].shape[0] == 5120 and w.meshes[0][0].shape[0] == 2562
    w1 = W.config1(scale=0.01, n_pairs=4, tri_hi=2000)
    assert w1.pairs.shape == (4, 2) and w1.n == w1.tf2.shape[0]
    assert w1.pair.max() == 3
