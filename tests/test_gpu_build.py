"""Device construction of the OBBRSS tree (fclgpu_mesh_create_on_device) against the host
build and the oracle node for node, bit for bit; the rebuilds of endUpdateModel /
endReplaceModel with refit = false against the oracle's restatement."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _same_tree(a, b):
    na, fa = a.get_nodes()
    nb, fb = b.get_nodes()
    assert np.array_equal(fa, fb)
    assert np.array_equal(na.view(np.uint64), nb.view(np.uint64))


def _meshes(golden):
    yield golden["env_v"], golden["env_t"]
    yield golden["rob_v"], golden["rob_t"]
    for f, r in ((1, (1.0, 0.7, 0.5)), (3, (0.5, 0.5, 0.5)), (12, (1.2, 0.4, 0.8))):
        yield W.perturbed_ellipsoid(f, r, 0.01, f)
    yield W.grid_box(5)  # axis-aligned, with zero coordinates (signs of zero in the fit)
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    yield tri, np.array([[0, 1, 2]], np.int32)
    rng = np.random.default_rng(3)
    v = rng.uniform(-1, 1, (300, 3))
    yield v, rng.integers(0, 300, (100, 3)).astype(np.int32)  # a triangle soup


def test_device_build_equals_host_build(gpu_lib, golden):
    for v, t in _meshes(golden):
        h = api.BVHModel.from_arrays(v, t)
        d = api.BVHModel.from_arrays(v, t, build="device")
        _same_tree(h, d)
        assert d.info().max_depth == h.info().max_depth
        on, ofc = O.Mesh(v, t).nodes()
        dn, dfc = d.get_nodes()
        assert np.array_equal(ofc, dfc) and np.array_equal(on.view(np.uint64), dn.view(np.uint64))


def test_device_build_largest_c1_mesh(gpu_lib):
    """The 200k-triangle C1 mesh: node for node, and the same collide results."""
    v, t = W.perturbed_ellipsoid(100, (1.0, 0.7, 0.5), 0.01, 5)
    assert t.shape[0] == 200000
    h = api.BVHModel.from_arrays(v, t)
    d = api.BVHModel.from_arrays(v, t, build="device")
    _same_tree(h, d)
    tf = W.random_poses(500, -1.0, 1.0, 6)
    a = api.collide_batch([h, h], [[0, 1]], None, tf, num_max_contacts=1000, statistics=True)
    b = api.collide_batch([d, d], [[0, 1]], None, tf, num_max_contacts=1000, statistics=True)
    for k in ("counts", "contacts", "num_bv_tests"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("update", [True, False])
def test_rebuild_matches_oracle(gpu_lib, update):
    """endUpdateModel(refit = false): rebuild on the new vertices, then the bottom-up refit
    over both frames; endReplaceModel(refit = false): rebuild alone.  Twice in a row."""
    v, t = W.perturbed_ellipsoid(8, (1.0, 0.6, 0.5), 0.01, 9)
    rng = np.random.default_rng(10)
    om = O.Mesh(v, t)
    m = api.BVHModel.from_arrays(v, t)
    for step in range(2):
        nv = v + rng.normal(0, 0.05, v.shape) + np.array([0.3, 0.0, -0.2]) * (step + 1)
        om.rebuild(nv, update)
        (m.beginUpdateModel if update else m.beginReplaceModel)()
        (m.updateSubModel if update else m.replaceSubModel)(nv)
        rc = (m.endUpdateModel if update else m.endReplaceModel)(refit=False)
        assert rc == 0
        on, ofc = om.nodes()
        dn, dfc = m.get_nodes()
        assert np.array_equal(ofc, dfc)
        assert np.array_equal(on.view(np.uint64), dn.view(np.uint64))
        # queries on the rebuilt tree equal the oracle's
        tf = W.random_poses(200, -0.8, 0.8, 11 + step)
        g = api.collide_batch([m, m], [[0, 1]], None, tf, num_max_contacts=100, statistics=True)
        c, ct, nbv, _ = O.collide_batch(om, om, tf, num_max_contacts=100, nthreads=8)
        assert np.array_equal(g["counts"], c) and np.array_equal(g["contacts"], ct)
        assert np.array_equal(g["num_bv_tests"], nbv)
