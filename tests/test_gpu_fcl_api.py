"""The fcl.collide / fcl.distance mirror on every pair kind it dispatches: mesh x mesh,
shape x shape and mesh x shape (both argument orders), against the oracle, and the
explicit rejection of GST_LIBCCD for pairs that need a GJK solver."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import native as N
from fcl_gb300 import workloads as W
from oracle import pyoracle as P

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _objs(shapes, ss, rng, n, box):
    idx = rng.integers(0, shapes.n, size=n)
    tf = W.random_poses(n, 0.0, box, int(rng.integers(1 << 30)))
    return [api.CollisionObject(api.ShapeRef(ss, int(i)), tf[k]) for k, i in enumerate(idx)], idx, tf


def test_shape_pairs_collide_and_distance(gpu_lib):
    shapes = W.random_shapes(48, 61)
    ss = api.ShapeSet.from_workload(shapes)
    G = P.Geoms(shapes)
    rng = np.random.default_rng(62)
    a, ia, tfa = _objs(shapes, ss, rng, 300, 1.2)
    b, ib, tfb = _objs(shapes, ss, rng, 300, 1.2)
    req = api.CollisionRequest(gjk_solver_type=api.GST_INDEP)
    reqc = api.CollisionRequest(gjk_solver_type=api.GST_INDEP, enable_contact=True)
    dreq = api.DistanceRequest(enable_nearest_points=True, gjk_solver_type=api.GST_INDEP)
    # fcl::collide / fcl::distance run the solver at the request's tolerance (1e-6)
    P.set_gjk_solver_params(1e-6, 1e-6)
    ref = P.shape_batch(shapes, ia, ib, tfa, tfb, nthreads=8)
    hits = 0
    for k in range(300):
        # enable_contact = false: FCL's default callback semantics (one NONE contact)
        S = P.Scene(G, np.array([ia[k]], np.int32), tfa[k])
        want = int(S.collide(np.array([ib[k]], np.int32), tfb[k], max_contacts=1, use_tree=False)["num_contacts"][0])
        r = api.CollisionResult()
        assert api.collide(a[k], b[k], req, r) == want
        if want:
            assert (r.contacts[0].b1, r.contacts[0].b2) == (api.Contact.NONE, api.Contact.NONE)
        # with contact: the deepest contact point, normal and depth of GJKSolver_indep
        rc = api.CollisionResult()
        got = api.collide(a[k], b[k], reqc, rc)
        assert got == int(ref["hit"][k])
        if got:
            hits += 1
            c = rc.contacts[0]
            assert np.array_equal(c.pos, ref["point"][k]) and np.array_equal(c.normal, ref["normal"][k])
            assert c.penetration_depth == ref["depth"][k]
        dr = api.DistanceResult()
        d = api.distance(a[k], b[k], dreq, dr)
        if ref["hit"][k]:
            assert d == -1.0
        else:
            assert d == ref["dist"][k]
            assert np.array_equal(dr.nearest_points, np.stack([ref["p1"][k], ref["p2"][k]]))
    P.set_gjk_solver_params()
    assert 20 < hits < 280
    assert api.get_gjk_solver_params() == api.SOLVER_DEFAULTS  # the mirror restores the parameters


def test_mesh_shape_pairs_both_orders(gpu_lib):
    vt = W.perturbed_ellipsoid(6, (0.8, 0.6, 0.5), 0.01, 63)
    mesh = api.BVHModel.from_arrays(*vt)
    om = P.Mesh(*vt)
    shapes = W.random_shapes(32, 64)
    ss = api.ShapeSet.from_workload(shapes)
    G = P.Geoms(shapes)
    rng = np.random.default_rng(65)
    n = 200
    sid = rng.integers(0, 32, size=n).astype(np.int32)
    tfm = W.random_poses(n, -0.3, 0.3, 66)
    tfs = W.random_poses(n, -1.3, 1.3, 67)
    P.set_gjk_solver_params(1e-6, 1e-6)
    c, tris = P.mesh_shape_contacts(om, G, sid, tfm, tfs, max_contacts=4, nthreads=8)
    off = np.concatenate([[0], np.cumsum(c)])
    dist = P.mesh_shape_distance(om, G, sid, tfm, tfs, nthreads=8)
    P.set_gjk_solver_params()
    req = api.CollisionRequest(num_max_contacts=4, gjk_solver_type=api.GST_INDEP)
    dreq = api.DistanceRequest(enable_nearest_points=True, gjk_solver_type=api.GST_INDEP)
    for k in range(n):
        om_, os_ = api.CollisionObject(mesh, tfm[k]), api.CollisionObject(api.ShapeRef(ss, int(sid[k])), tfs[k])
        for x, y in ((om_, os_), (os_, om_)):
            r = api.CollisionResult()
            assert api.collide(x, y, req, r) == c[k]
            # FCL records the mesh's triangle as b1 whichever argument came first
            assert [ct.b1 for ct in r.contacts] == list(tris[off[k]:off[k + 1]])
            assert all(ct.o1 is mesh and ct.b2 == api.Contact.NONE for ct in r.contacts)
            dr = api.DistanceResult()
            d = api.distance(x, y, dreq, dr)
            assert d == dist["dist"][k]
            if d > 0:
                assert dr.b1 == dist["tri"][k] and np.array_equal(dr.nearest_points, dist["pts"][k])
    assert (c > 0).any() and (c == 0).any()
    # enable_contact: Contact(mesh, shape, tri, NONE, contactp, -normal, penetration)
    reqc = api.CollisionRequest(num_max_contacts=4, enable_contact=True, gjk_solver_type=api.GST_INDEP)
    pair = np.repeat(np.arange(n), c)
    P.set_gjk_solver_params(1e-6, 1e-6)
    geo = P.mesh_shape_contact_geometry(om, G, sid[pair], tfm[pair], tfs[pair], tris)
    P.set_gjk_solver_params()
    assert geo["ok"].all()
    for k in np.nonzero(c)[0][:60]:
        om_, os_ = api.CollisionObject(mesh, tfm[k]), api.CollisionObject(api.ShapeRef(ss, int(sid[k])), tfs[k])
        for x, y in ((om_, os_), (os_, om_)):
            r = api.CollisionResult()
            assert api.collide(x, y, reqc, r) == c[k]
            for j, ct in enumerate(r.contacts):
                q = off[k] + j
                assert ct.b1 == tris[q]
                assert np.array_equal(ct.pos, geo["pos"][q]) and np.array_equal(ct.normal, geo["normal"][q])
                assert ct.penetration_depth == geo["depth"][q]


def test_gst_libccd_is_rejected_for_shape_pairs(gpu_lib):
    shapes = W.random_shapes(4, 68)
    ss = api.ShapeSet.from_workload(shapes)
    a = api.CollisionObject(api.ShapeRef(ss, 0), W.random_poses(1, 0, 1, 1)[0])
    b = api.CollisionObject(api.ShapeRef(ss, 1), W.random_poses(1, 0, 1, 2)[0])
    for call, req, res in ((api.collide, api.CollisionRequest(), api.CollisionResult()),
                           (api.distance, api.DistanceRequest(), api.DistanceResult())):
        assert req.gjk_solver_type == api.GST_LIBCCD  # FCL's default
        with pytest.raises(N.FclGpuError) as e:
            call(a, b, req, res)
        assert e.value.code == N.FCLGPU_ERR_UNSUPPORTED_ and "GST_INDEP" in str(e.value)
    # mesh pairs use no GJK solver: the default request is accepted
    vt = W.perturbed_ellipsoid(3, (0.5, 0.5, 0.5), 0.01, 69)
    m = api.BVHModel.from_arrays(*vt)
    r = api.CollisionResult()
    api.collide(api.CollisionObject(m), api.CollisionObject(m), api.CollisionRequest(), r)
    assert r.numContacts() == 1


@pytest.mark.parametrize("params", [(1e-6, 1e-6, 128, 255), (2.0097183471152322e-14, 2.0097183471152322e-14, 1, 255),
                                    (2.0097183471152322e-14, 2.0097183471152322e-14, 128, 1),
                                    (1e-3, 1e-3, 3, 2)])
def test_solver_parameters_match_oracle(gpu_lib, params):
    """GJKSolver_indep's tolerances and iteration caps: the request tolerance of
    fcl::collide (1e-6), a GJK cap of 1 (status Failed, gjk-inl.h:188), an EPA cap of 1
    (epa-inl.h:309-343) and coarse settings give the oracle's booleans, statuses, depths
    and distances bit for bit."""
    w3 = W.config3(n_pairs=6000, n_shapes=96, seed=71)
    ss = api.ShapeSet.from_workload(w3.shapes)
    try:
        api.set_gjk_solver_params(*params)
        P.set_gjk_solver_params(*params)
        g = api.shape_batch(ss, w3.ia, w3.ib, w3.tf1, w3.tf2)
        o = P.shape_batch(w3.shapes, w3.ia, w3.ib, w3.tf1, w3.tf2, nthreads=8)
    finally:
        api.set_gjk_solver_params()
        P.set_gjk_solver_params()
    for k in ("hit", "status", "depth", "normal", "point", "dist", "p1", "p2"):
        assert np.array_equal(g[k], o[k]), k
    if params[2] == 1:
        assert (g["status"][:, 0] == 2).any()  # GJK Failed (gjk-inl.h:188)


def test_solver_parameters_are_validated(gpu_lib):
    for bad in ((0.0, 1e-6, 128, 255), (1e-6, -1.0, 128, 255), (1e-6, 1e-6, 0, 255), (1e-6, 1e-6, 128, 0)):
        with pytest.raises(N.FclGpuError):
            api.set_gjk_solver_params(*bad)
    assert api.get_gjk_solver_params() == api.SOLVER_DEFAULTS
