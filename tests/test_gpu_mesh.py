"""GPU parity for the OBBRSS mesh path, through the C ABI, against the FP64 oracle.

Collide: counts, contact lists (same triangle pairs in the same DFS order) and
traversal statistics must equal the oracle's exactly in both precision forms.
Distance: min distance, triangle ids and nearest points of the FP64 form must equal
the oracle's bit for bit; the FP32 form must agree within 1e-6 relative (1e-9
absolute floor) and report the witness points of a pair at that distance."""
import numpy as np
import pytest

from fcl_gb300 import api
from fcl_gb300 import workloads as W
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

REL, ABS = 1e-6, 1e-9


def _meshes(w):
    return [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]


def _oracle_collide(w, maxc, nthreads=8):
    om = [O.Mesh(v, t) for v, t in w.meshes]
    counts, contacts, nbv, nleaf = [], [], [], []
    order = []
    for p in range(w.pairs.shape[0]):
        idx = np.nonzero(w.pair == p)[0]
        if idx.size == 0:
            continue
        a, b = om[w.pairs[p, 0]], om[w.pairs[p, 1]]
        c, ct, bv, lf = O.collide_batch(a, b, w.tf2[idx], None if w.tf1 is None else w.tf1[idx],
                                        num_max_contacts=maxc, nthreads=nthreads)
        off = np.concatenate([[0], np.cumsum(c)])
        for j, q in enumerate(idx):
            order.append((q, ct[off[j]:off[j + 1]]))
        counts.append((idx, c)); nbv.append((idx, bv)); nleaf.append((idx, lf))
    n = w.n
    C = np.zeros(n, np.int64); BV = np.zeros(n, np.int64); LF = np.zeros(n, np.int64)
    for idx, c in counts:
        C[idx] = c
    for idx, c in nbv:
        BV[idx] = c
    for idx, c in nleaf:
        LF[idx] = c
    order.sort(key=lambda x: x[0])
    ct = np.concatenate([x[1] for x in order]) if order else np.zeros((0, 2), np.int32)
    return C, ct, BV, LF


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("maxc", [1, 100000])
def test_collide_config0_matches_oracle(gpu_lib, precision, maxc):
    w = W.config0(n_poses=2000)
    ms = _meshes(w)
    out = api.collide_batch(ms, w.pairs, None, w.tf2, num_max_contacts=maxc, precision=precision,
                            statistics=True)
    C, ct, BV, LF = _oracle_collide(w, maxc)
    assert np.array_equal(out["counts"], C)
    assert np.array_equal(out["contacts"], ct)
    assert np.array_equal(out["num_bv_tests"], BV)
    assert np.array_equal(out["num_leaf_tests"], LF)
    if precision == "fp64":
        assert out["num_rechecks"].sum() == 0
    else:
        assert out["num_rechecks"].sum() <= 0.01 * (BV.sum() + LF.sum())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_collide_reference_fixture(gpu_lib, golden, precision):
    ms = [api.BVHModel.from_arrays(golden["env_v"], golden["env_t"]),
          api.BVHModel.from_arrays(golden["rob_v"], golden["rob_t"])]
    tf = golden["tf"]
    out = api.collide_batch(ms, [[0, 1]], None, tf, num_max_contacts=1 << 30, precision=precision,
                            statistics=True)
    env = O.Mesh(golden["env_v"], golden["env_t"]); rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    c, ct, bv, lf = O.collide_batch(env, rob, tf, num_max_contacts=1 << 30)
    assert np.array_equal(out["counts"], c) and np.array_equal(out["contacts"], ct)
    assert np.array_equal(out["num_bv_tests"], bv) and np.array_equal(out["num_leaf_tests"], lf)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_collide_multi_pair_uneven_with_tf1(gpu_lib, precision):
    w = W.config1(scale=0.004, n_pairs=6, tri_hi=30000, seed=3)
    w.tf1 = W.random_poses(w.n, -0.3, 0.3, 77)
    ms = _meshes(w)
    out = api.collide_batch(ms, w.pairs, w.tf1, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                            precision=precision, statistics=True)
    C, ct, BV, LF = _oracle_collide(w, 100000)
    assert np.array_equal(out["counts"], C)
    assert np.array_equal(out["contacts"], ct)
    assert np.array_equal(out["num_bv_tests"], BV) and np.array_equal(out["num_leaf_tests"], LF)


def test_collide_device_api_torch(gpu_lib):
    import torch
    w = W.config0(n_poses=3000, seed=4)
    ms = _meshes(w)
    tf2 = torch.from_numpy(w.tf2).cuda()
    outs = {}
    for prec in ("fp64", "fp32"):
        o = api.collide_batch(ms, w.pairs, None, tf2, num_max_contacts=100000, precision=prec, statistics=True)
        torch.cuda.synchronize()
        outs[prec] = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in o.items()}
    C, ct, BV, LF = _oracle_collide(w, 100000)
    for prec in outs:
        assert np.array_equal(outs[prec]["counts"], C)
        assert np.array_equal(outs[prec]["contacts"], ct)
        assert np.array_equal(outs[prec]["offsets"][1:], np.cumsum(C))


def test_collide_fp32_equals_fp64_at_scale(gpu_lib):
    # size-independent property at a larger batch: both forms agree exactly
    w = W.config1(scale=0.1, n_pairs=8, tri_hi=100000, seed=9)
    ms = _meshes(w)
    a = api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                          precision="fp64", statistics=True)
    b = api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                          precision="fp32", statistics=True)
    assert np.array_equal(a["counts"], b["counts"]) and np.array_equal(a["contacts"], b["contacts"])
    assert np.array_equal(a["num_bv_tests"], b["num_bv_tests"])
    # every reported pair is a real intersection per the oracle's triangle test
    rng = np.random.default_rng(0)
    sel = rng.choice(np.nonzero(a["counts"])[0], size=min(50, int((a["counts"] > 0).sum())), replace=False)
    for q in sel:
        p = w.pair[q]; A = w.meshes[w.pairs[p, 0]]; B = w.meshes[w.pairs[p, 1]]
        lo, hi = a["offsets"][q], a["offsets"][q + 1]
        pairs = a["contacts"][lo:hi]
        P = A[0][A[1][pairs[:, 0]]].reshape(-1, 9); Q = B[0][B[1][pairs[:, 1]]].reshape(-1, 9)
        assert O.tri_intersect_batch(P, Q, w.tf2[q]).all()


def test_collide_empty_and_zero_contacts(gpu_lib):
    w = W.config0(n_poses=10, freq=4)
    ms = _meshes(w)
    out = api.collide_batch(ms, w.pairs, None, w.tf2[:0], num_max_contacts=1)
    assert out["counts"].shape == (0,) and out["total_contacts"] == 0
    out = api.collide_batch(ms, w.pairs, None, w.tf2, num_max_contacts=0)
    assert out["counts"].sum() == 0


def test_distance_fp64_bit_exact(gpu_lib):
    w = W.config0(n_poses=400, seed=2)
    ms = _meshes(w)
    out = api.distance_batch(ms, w.pairs, None, w.tf2, nearest_points=True, precision="fp64", statistics=True)
    a = O.Mesh(*w.meshes[0]); b = O.Mesh(*w.meshes[1])
    d, ids, pts, nbv, nl = O.distance_batch(a, b, w.tf2, nearest=True, nthreads=8)
    assert np.array_equal(out["min_distance"], d)
    assert np.array_equal(out["ids"], ids)
    assert np.array_equal(out["nearest_points"], pts)
    assert np.array_equal(out["num_bv_tests"], nbv) and np.array_equal(out["num_leaf_tests"], nl)


def test_distance_reference_fixture(gpu_lib, golden):
    ms = [api.BVHModel.from_arrays(golden["env_v"], golden["env_t"]),
          api.BVHModel.from_arrays(golden["rob_v"], golden["rob_t"])]
    out = api.distance_batch(ms, [[0, 1]], None, golden["tf"], nearest_points=True, precision="fp64")
    env = O.Mesh(golden["env_v"], golden["env_t"]); rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    for i in range(golden["tf"].shape[0]):
        assert out["min_distance"][i] == O.brute_distance(env, rob, golden["tf"][i])


def _dist_check(out, d, pts):
    got = out["min_distance"]
    err = np.abs(got - d)
    tol = np.maximum(REL * np.abs(d), ABS)
    assert np.all(err <= tol), f"max rel err {np.max(err / np.maximum(np.abs(d), ABS))}"
    pos = d > 0
    if pos.any():
        perr = np.abs(out["nearest_points"][pos] - pts[pos]).max(axis=(1, 2))
        scale = np.maximum(np.abs(pts[pos]).max(axis=(1, 2)), 1.0)
        assert np.all(perr <= REL * scale + ABS)


def test_distance_fp32_config0(gpu_lib):
    w = W.config0(n_poses=1500, seed=3)
    ms = _meshes(w)
    out = api.distance_batch(ms, w.pairs, None, w.tf2, nearest_points=True, precision="fp32", statistics=True)
    a = O.Mesh(*w.meshes[0]); b = O.Mesh(*w.meshes[1])
    d, ids, pts, _, _ = O.distance_batch(a, b, w.tf2, nearest=True, nthreads=8)
    _dist_check(out, d, pts)


def test_distance_fp32_separated_multi_pair_with_margins(gpu_lib):
    w = W.config2(total_poses=3000, n_pairs=6, tri_hi=30000, seed=4)
    ms = _meshes(w)
    out = api.distance_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, nearest_points=True,
                             precision="fp32", margins=w.margin, statistics=True)
    om = [O.Mesh(v, t) for v, t in w.meshes]
    d = np.empty(w.n); pts = np.empty((w.n, 2, 3))
    for p in range(w.pairs.shape[0]):
        idx = np.nonzero(w.pair == p)[0]
        dd, _, pp, _, _ = O.distance_batch(om[w.pairs[p, 0]], om[w.pairs[p, 1]], w.tf2[idx], nearest=True, nthreads=8)
        d[idx] = dd; pts[idx] = pp
    _dist_check(out, d, pts)
    assert np.array_equal(out["within_margin"].astype(bool), d <= w.margin)


def test_distance_fp32_tf1_and_fixture(gpu_lib, golden):
    ms = [api.BVHModel.from_arrays(golden["env_v"], golden["env_t"]),
          api.BVHModel.from_arrays(golden["rob_v"], golden["rob_t"])]
    tf = golden["tf"]
    tf1 = W.random_poses(tf.shape[0], -100, 100, 5)
    out = api.distance_batch(ms, [[0, 1]], tf1, tf, nearest_points=True, precision="fp32")
    env = O.Mesh(golden["env_v"], golden["env_t"]); rob = O.Mesh(golden["rob_v"], golden["rob_t"])
    d, ids, pts, _, _ = O.distance_batch(env, rob, tf, tf1=tf1, nearest=True)
    _dist_check(out, d, pts)


def test_distance_values_alone_match_oracle(gpu_lib):
    """ids=False, nearest_points=False: one warp per query (certified FP32 bounds, FP64
    triDistance near the best) -- the distances equal the full call's bit for bit and
    the oracle's up to one FP64 rounding, for separated multi-pair poses, for touching
    and intersecting poses, and after a vertex update (refitted volumes: the FP64
    form)."""
    w = W.config2(total_poses=3000, n_pairs=6, tri_hi=30000, seed=7)
    ms = _meshes(w)
    full = api.distance_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, nearest_points=True,
                              precision="fp32")
    vals = api.distance_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, nearest_points=False, ids=False,
                              precision="fp32")
    assert "ids" not in vals
    np.testing.assert_array_equal(vals["min_distance"], full["min_distance"])
    om = [O.Mesh(v, t) for v, t in w.meshes]
    for p in range(w.pairs.shape[0]):
        idx = np.nonzero(w.pair == p)[0]
        dd, _, _, _, _ = O.distance_batch(om[w.pairs[p, 0]], om[w.pairs[p, 1]], w.tf2[idx], nearest=False,
                                          nthreads=8)
        # the smallest FP64 triDistance over all triangle pairs; FCL's may be the same
        # distance through another pair (a shared vertex), rounded differently
        np.testing.assert_allclose(vals["min_distance"][idx], dd, rtol=4e-16, atol=0)
    w0 = W.config0(n_poses=600, seed=8)
    m0 = _meshes(w0)
    a = O.Mesh(*w0.meshes[0]); b = O.Mesh(*w0.meshes[1])
    for step in range(2):
        v0 = api.distance_batch(m0, w0.pairs, None, w0.tf2, nearest_points=False, ids=False, precision="fp32")
        d0, _, _, _, _ = O.distance_batch(a, b, w0.tf2, nearest=False, nthreads=8)
        np.testing.assert_allclose(v0["min_distance"], d0, rtol=4e-16, atol=0)
        if step == 0:
            assert (d0 == 0).any() and (d0 > 0).any()
            v1 = w0.meshes[1][0] + np.random.default_rng(9).normal(0, 0.003, w0.meshes[1][0].shape)
            m0[1].update_vertices(v1)
            b.update(v1)


def test_distance_rejects_out_of_range_pair_index(gpu_lib):
    """A pair index outside the pair table is not read: the device entry point skips
    that query, sets the status word and returns FCLGPU_ERR_DEVICE_STATUS; the other
    queries keep their results."""
    import torch
    from fcl_gb300 import native as N
    w = W.config0(n_poses=8, freq=2)
    ms = _meshes(w)
    tf2 = torch.from_numpy(w.tf2).cuda()
    pq = torch.zeros(8, dtype=torch.int32, device="cuda")
    pq[3] = 7
    with pytest.raises(N.FclGpuError) as e:
        api.distance_batch(ms, w.pairs, None, tf2, pair_of_query=pq, precision="fp32")
    assert e.value.code == N.FCLGPU_ERR_DEVICE_STATUS
    good = api.distance_batch(ms, w.pairs, None, tf2, pair_of_query=torch.zeros_like(pq), precision="fp32")
    assert torch.isfinite(good["min_distance"]).all()


def _largest_c1_workload(n_per=100):
    """The C1 pairs that hold the meshes of 150k-200k triangles (tree depth about 38),
    n_per poses each with C1's translations U[-1.5,1.5]^3."""
    big = [3, 13, 16, 52]
    ms = W.mesh_pair_set_subset(big)
    ids = sorted(ms)
    local = {k: i for i, k in enumerate(ids)}
    pairs = np.array([[local[2 * p], local[2 * p + 1]] for p in big], np.int32)
    pair = np.repeat(np.arange(len(big), dtype=np.int32), n_per)
    tf2 = W.random_poses(pair.shape[0], -1.5, 1.5, 21)
    return W.MeshPairWorkload(meshes=[ms[k] for k in ids], pairs=pairs, pair=pair, tf2=tf2, name="c1_largest")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_collide_largest_c1_meshes_match_oracle(gpu_lib, precision):
    """Exhaustive contacts (num_max_contacts = 100,000) on the largest C1 meshes: counts,
    contact lists in DFS order and traversal statistics equal the oracle's."""
    w = _largest_c1_workload()
    assert max(t.shape[0] for _, t in w.meshes) >= 150000
    ms = _meshes(w)
    out = api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                            precision=precision, statistics=True)
    C, ct, BV, LF = _oracle_collide(w, 100000)
    assert (C > 0).sum() >= 50 and C.max() > 1000
    assert np.array_equal(out["counts"], C)
    assert np.array_equal(out["contacts"], ct)
    assert np.array_equal(out["num_bv_tests"], BV) and np.array_equal(out["num_leaf_tests"], LF)


def test_distance_fp32_largest_c1_meshes(gpu_lib):
    """Distance on the largest C1 meshes at C2's separations: the FP32 form against the oracle."""
    w = _largest_c1_workload(60)
    w.tf2 = W.random_poses(w.n, 1.5, 4.0, 22)
    ms = _meshes(w)
    out = api.distance_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, nearest_points=True,
                             precision="fp32")
    om = [O.Mesh(v, t) for v, t in w.meshes]
    d = np.empty(w.n); pts = np.empty((w.n, 2, 3))
    for p in range(w.pairs.shape[0]):
        idx = np.nonzero(w.pair == p)[0]
        dd, _, pp, _, _ = O.distance_batch(om[w.pairs[p, 0]], om[w.pairs[p, 1]], w.tf2[idx], nearest=True,
                                           nthreads=8)
        d[idx] = dd; pts[idx] = pp
    _dist_check(out, d, pts)


def test_collide_capacity_retry_and_stack_limit(gpu_lib):
    """Error paths of the collide batch, forced through the test limits: record and
    work-item scratch far too small (the batch doubles them and runs again, with the
    same result), and a traversal stack limit below the trees' depth (the device
    reports it and the call returns FCLGPU_ERR_DEVICE_STATUS)."""
    from fcl_gb300 import native as N
    w = W.config1(scale=0.004, n_pairs=6, tri_hi=30000, seed=3)
    ms = _meshes(w)

    def run():
        return api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                                 precision="fp32", statistics=True, budget=64)

    ref = run()
    assert ref["contacts"].shape[0] > 1000
    try:
        N.check(N.lib().fclgpu_set_collide_test_limits(16, w.n + 8, 0), "limits")
        got = run()
        for k in ("counts", "contacts", "num_bv_tests", "num_leaf_tests"):
            assert np.array_equal(got[k], ref[k]), k
        N.check(N.lib().fclgpu_set_collide_test_limits(0, 0, 6), "limits")
        with pytest.raises(N.FclGpuError) as e:
            run()
        assert e.value.code == N.FCLGPU_ERR_DEVICE_STATUS and "stack" in str(e.value)
    finally:
        N.check(N.lib().fclgpu_set_collide_test_limits(0, 0, 0), "limits")
    again = run()
    assert np.array_equal(again["contacts"], ref["contacts"])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_collide_persistent_launch_matches_round_launches(gpu_lib, precision):
    """All collide rounds in one cooperative launch (the default) against one launch per
    round: the same counts, contact lists and statistics, many rounds deep (budget 64),
    and the oracle's on the C0 pair."""
    from fcl_gb300 import native as N
    w = W.config1(scale=0.004, n_pairs=6, tri_hi=30000, seed=4)
    ms = _meshes(w)

    def run():
        return api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                                 precision=precision, statistics=True, budget=64)

    launches0 = N.lib().fclgpu_kernel_launch_count()
    one = run()
    launches_one = N.lib().fclgpu_kernel_launch_count() - launches0
    try:
        N.check(N.lib().fclgpu_set_collide_persistent(0, 60 * 10**9, 0), "persistent")
        launches0 = N.lib().fclgpu_kernel_launch_count()
        per_round = run()
        launches_rounds = N.lib().fclgpu_kernel_launch_count() - launches0
    finally:
        N.check(N.lib().fclgpu_set_collide_persistent(1, 60 * 10**9, 0), "persistent")
    for k in ("counts", "contacts", "num_bv_tests", "num_leaf_tests"):
        assert np.array_equal(one[k], per_round[k]), k
    assert one["contacts"].shape[0] > 1000
    assert launches_rounds > launches_one + 5  # the per-round form launched every round
    w0 = W.config0(n_poses=500)
    out = api.collide_batch(_meshes(w0), w0.pairs, None, w0.tf2, num_max_contacts=100000, precision=precision,
                            statistics=True, budget=64)
    C, ct, BV, LF = _oracle_collide(w0, 100000)
    assert np.array_equal(out["counts"], C) and np.array_equal(out["contacts"], ct)
    assert np.array_equal(out["num_bv_tests"], BV)


def test_collide_persistent_barrier_timeout_falls_back(gpu_lib):
    """A grid barrier that waits for a block the grid does not have gives up after its
    limit (20 ms here): the launch reports it, the batch runs again one launch per round,
    and the result is unchanged."""
    from fcl_gb300 import native as N
    w = W.config1(scale=0.004, n_pairs=6, tri_hi=30000, seed=5)
    ms = _meshes(w)

    def run():
        return api.collide_batch(ms, w.pairs, None, w.tf2, pair_of_query=w.pair, num_max_contacts=100000,
                                 precision="fp32", statistics=True, budget=64)

    ref = run()
    before = N.lib().fclgpu_collide_persistent_fallbacks()
    try:
        N.check(N.lib().fclgpu_set_collide_persistent(1, 20 * 10**6, 1), "persistent")
        got = run()
    finally:
        N.check(N.lib().fclgpu_set_collide_persistent(1, 60 * 10**9, 0), "persistent")
    after = N.lib().fclgpu_collide_persistent_fallbacks()
    assert after > before  # every batch of the call fell back
    for k in ("counts", "contacts", "num_bv_tests", "num_leaf_tests"):
        assert np.array_equal(got[k], ref[k]), k
    again = run()
    assert np.array_equal(again["contacts"], ref["contacts"])
    assert N.lib().fclgpu_collide_persistent_fallbacks() == after
