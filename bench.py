"""Benchmark of the batched OBBRSS mesh-collide hot path on one GB300.

Workload (the configuration the headline metric is quoted on): 64 mesh pairs of
perturbed icosphere/ellipsoid meshes with 500-200,000 triangles (log-uniform), each
pair with 2,000-50,000 Haar-uniform poses (log-uniform; ~1.1M queries in total),
translations U[-1.5,1.5]^3, exhaustive contacts (num_max_contacts = 100,000).
A step = one batched collide over all queries, inputs resident in HBM.  Timed
with CUDA events on the launching stream; L2 is flushed between steps.

Reported: queries/s of the FP32 + FP64-recheck form (value), the plain FP64 GPU
form beside it with the exact-hit check (identical counts and contact lists), the
same metric end to end through the host C ABI (pinned host buffers, copies in the
timed region), the roofline of the traversal kernel, the FP64 CPU oracle timed on
the host cores on a bounded sample, and SM clocks sampled during the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "queries/s batched FP32+FP64-recheck vs plain GPU (exact hits); p50/p99 request ms"
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of the collide kernel (all
# rounds in one cooperative launch) per C1 step, from ncu on two small cases of the same
# workload (5 % and 20 % of the poses, the 128-register variant the autotuner picks; mean
# of 5 steps each): 82.94 GB at 55,143 queries and 212.52 GB at 220,586.  Traffic grows less
# than in proportion to the queries (the poses of one mesh pair share its tree in L2), so a
# full step is priced by the straight line through the two points, a + b * queries.
C1_TRAFFIC_A = 39.75e9
# timed calls of the plain FP64 form (on its subset), after one warm-up call
FP64_REPEATS = 2
C1_TRAFFIC_B = 783226.0  # bytes per query
C1_TRAFFIC_VARIANT = 1
UNIT = "queries/s"
WORKLOAD = "c1_exhaustive_contacts_64pairs_500-200k_tris"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def _max_over_ranks(x: float, device, world: int) -> float:
    """The slowest rank's time (the job's time): all-reduce MAX over the process group."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x: float, device, world: int) -> float:
    """Units processed by all ranks: all-reduce SUM over the process group."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


_WORKLOADS = {}


def _workload(args, rank):
    """The C1 workload of this rank (generated once per process)."""
    from fcl_gb300 import workloads as W
    key = (args.scale, rank, args.pairs, args.tri_hi)
    if key not in _WORKLOADS:
        _WORKLOADS[key] = W.config1(scale=args.scale, seed=1 + 1000 * rank, n_pairs=args.pairs, tri_hi=args.tri_hi)
    return _WORKLOADS[key]


# ------------------------------------------------------------------------------------
# reference arm: the reference's CPU algorithm (the FP64 oracle restatement; FCL itself
# cannot be compiled here) on all host cores, bounded sample per step
# ------------------------------------------------------------------------------------
def _cpu_sample(w, n_sample, seed=0):
    from fcl_gb300 import workloads as W
    return W.subsample(w, n_sample, seed)


def _time_cpu(w_sample, nthreads, results=None):
    """Times the oracle's collide over the sample; fills results[p] = (sample indices,
    counts, contacts) when a dict is given."""
    from oracle import pyoracle as O
    om = {}
    for p in np.unique(w_sample.pair):
        for m in w_sample.pairs[p]:
            if m not in om:
                om[m] = O.Mesh(*w_sample.meshes[m])
    t0 = time.perf_counter()
    total = 0
    for p in np.unique(w_sample.pair):
        idx = np.nonzero(w_sample.pair == p)[0]
        c, ct, _, _ = O.collide_batch(om[w_sample.pairs[p, 0]], om[w_sample.pairs[p, 1]], w_sample.tf2[idx],
                                      num_max_contacts=100000, nthreads=nthreads)
        total += int(c.sum())
        if results is not None:
            results[int(p)] = (idx, c, ct)
    return time.perf_counter() - t0, total


def _oracle_check(w, sample_idx, results, gpu):
    """Compares the GPU's counts and contact lists of the sampled queries with the
    oracle's (same triangle pairs in the same order)."""
    counts = gpu["counts"].cpu().numpy()
    offs = gpu["offsets"].cpu().numpy()
    cont = gpu["contacts"].cpu().numpy()
    ok = True
    for p, (idx, c, ct) in results.items():
        q = sample_idx[idx]
        ok &= bool(np.array_equal(counts[q], c))
        if not ok:
            break
        off = np.concatenate([[0], np.cumsum(c)])
        for j, qq in enumerate(q):
            if not np.array_equal(cont[offs[qq]:offs[qq + 1]], ct[off[j]:off[j + 1]]):
                ok = False
                break
    return ok


def _time_cpu_distance(w_sample, nthreads):
    from oracle import pyoracle as O
    om = {}
    for p in np.unique(w_sample.pair):
        for m in w_sample.pairs[p]:
            if m not in om:
                om[m] = O.Mesh(*w_sample.meshes[m])
    t0 = time.perf_counter()
    for p in np.unique(w_sample.pair):
        idx = np.nonzero(w_sample.pair == p)[0]
        O.distance_batch(om[w_sample.pairs[p, 0]], om[w_sample.pairs[p, 1]], w_sample.tf2[idx], nearest=True,
                         nthreads=nthreads)
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import pyoracle as O
    O.build()
    threads = O.hardware_threads()
    w = _workload(args, 0)
    n_sample = args.cpu_sample
    times = []
    for s in range(args.warmup + args.steps):
        ws = _cpu_sample(w, n_sample, seed=s)
        dt, _ = _time_cpu(ws, threads)
        if s >= args.warmup:
            times.append(dt)
    qps = n_sample / float(np.mean(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "queries": w.n, "sample_per_step": n_sample},
        "cpu_baseline": {"value": qps, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample} queries drawn uniformly from the {w.n}-query workload per step"},
        "e2e": {"value": qps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------------------
# serving: motion-checking requests against a resident broadphase scene
# ------------------------------------------------------------------------------------
def _serving_expected_cpu(w, reqs, threads, first_chunk=1, max_chunk=512):
    """The reference's CPU path for the same requests and the same request semantics:
    the dynamic AABB tree manager with the default callbacks on the host cores,
    waypoints checked in order in the server's chunks (1, 2, 4, ... up to 512) --
    collide (num_max_contacts = 1) for a chunk, stop at the first contact, otherwise
    distance for the chunk.  Returns requests/s."""
    from fcl_gb300 import workloads as W
    from oracle import pyoracle as O
    om = [O.Mesh(v, t) for v, t in w.meshes]
    G = O.Geoms(w.shapes, om)
    ns = w.shapes.n
    gid = np.where(w.refs[:, 0] == 1, ns + w.refs[:, 1], w.refs[:, 1]).astype(np.int32)
    S = O.Scene(G, gid, w.tf)
    lg = np.where(w.robot.link_refs[:, 0] == 1, ns + w.robot.link_refs[:, 1], w.robot.link_refs[:, 1])
    t0 = time.perf_counter()
    for r in reqs:
        poses = W.robot_fk(w.robot, r.base, r.q)
        K, L = poses.shape[:2]
        k0, chunk = 0, first_chunk
        while k0 < K:
            k1 = min(K, k0 + chunk)
            chunk = min(2 * chunk, max_chunk)
            qg = np.tile(lg, k1 - k0).astype(np.int32)
            tf = poses[k0:k1].reshape((k1 - k0) * L, 12)
            c = S.collide(qg, tf, max_contacts=1, use_tree=True, nthreads=threads)
            if (c["num_contacts"] > 0).any():
                break
            S.distance(qg, tf, use_tree=True, nthreads=threads)
            k0 = k1
    return len(reqs) / (time.perf_counter() - t0)


def run_serving(args):
    from fcl_gb300 import api
    from fcl_gb300 import serving as SV
    from fcl_gb300 import workloads as W
    t0 = time.perf_counter()
    w = W.scene4(n_objects=args.serve_objects or None, seed=4)
    ss = api.ShapeSet.from_workload(w.shapes)
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(w.refs, w.tf)
    setup_s = time.perf_counter() - t0
    nb = 16
    reqs = W.motion_requests(w, args.serve_requests + nb, seed=5)
    srv = api.MotionServer(mgr, w.robot, max_waypoints_per_step=args.serve_step)
    SV.run_burst(srv, reqs[:16])  # warm-up
    # capacity: the throughput of the Poisson run's own requests submitted all at once
    # (how early a request collides, and so its cost, varies much between requests, so a
    # burst of other requests is not a measure of this run's capacity)
    burst = SV.run_burst(srv, reqs[nb:])
    rate = args.serve_rate if args.serve_rate > 0 else 0.5 * burst["requests_per_s"]
    ph = (C.c_double * 16)()
    api.N.lib().fclgpu_broadphase_last_phase_ms(ph)  # reset the phase clocks
    st0 = srv.stats()
    with ClockSampler(0) as cs:
        load = SV.run_poisson(srv, reqs[nb:], rate, seed=6)
    api.N.lib().fclgpu_broadphase_last_phase_ms(ph)
    st1 = srv.stats()
    # the engine's counters over the Poisson run alone
    st = {k: st1[k] - st0[k] for k in st1 if k != "max_step_waypoints"}
    srv.close()
    out = {
        "workload": f"scene of {w.n} objects (primitives and 500-5000-tri icospheres, 25% meshes) in a 20^3 box; "
                    f"20-link robot (10 capsules, 10 x 2000-tri meshes); K ~ logU[10,500] waypoints",
        "objects": w.n, "links": w.robot.n_links,
        "capacity_requests_per_s": burst["requests_per_s"],
        "capacity_measure": "the same requests submitted at once",
        "arrival_rate_per_s": rate, "offered_rate_per_s": load["offered_rate_per_s"], "requests": load["requests"],
        "throughput_requests_per_s": load["throughput_requests_per_s"],
        "sustained_requests_per_s": load["sustained_requests_per_s"],
        "latency_p50_first_half_ms": load["latency_first_half_p50_ms"],
        "latency_p50_second_half_ms": load["latency_second_half_p50_ms"],
        "p50_ms": load["p50_ms"], "p99_ms": load["p99_ms"], "mean_ms": load["mean_ms"], "max_ms": load["max_ms"],
        "waypoints": int(sum(r.q.shape[0] for r in reqs[nb:])),
        "engine": {k: st[k] for k in ("steps", "waypoints", "queries", "candidates", "busy_ms", "collide_ms",
                                      "distance_ms")},
        # broadphase wall-clock phases over the Poisson run (fclgpu_broadphase_last_phase_ms):
        # setup + candidates, shape pairs, mesh-shape pairs, mesh-mesh pairs, reduction
        "phases_ms": {"collide": [round(x, 1) for x in ph[0:5]], "distance": [round(x, 1) for x in ph[8:13]]},
        # candidates, mesh-shape pairs and mesh-mesh pairs evaluated in those phases
        "phase_pairs": {"collide": [int(x) for x in ph[5:8]], "distance": [int(x) for x in ph[13:16]]},
        "scene_setup_s": setup_s, "clocks": cs.summary(),
    }
    if not args.no_cpu:
        from oracle import pyoracle as O
        O.build()
        threads = O.hardware_threads()
        sample = reqs[nb:nb + args.serve_cpu_sample]
        out["cpu_baseline"] = {"value": _serving_expected_cpu(w, sample, threads), "unit": "requests/s",
                               "cores": threads, "kind": "port",
                               "sample": f"{len(sample)} of the requests, dynamic AABB tree manager "
                                         "(collide + distance per link and waypoint, in the server's "
                                         "chunks of 1, 2, 4, ... waypoints, stopping at the first contact)"}
    return out


# ------------------------------------------------------------------------------------
# secondary workloads: the distance batch and the convex-pair batch
# ------------------------------------------------------------------------------------
def _time_device(fn, steps, warmup, stream, flush):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ms = []
    for i in range(steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms))


def run_secondary(args, meshes, stream, flush):
    """Distance batch (1M poses over the same 64 mesh pairs, translations U[1.5,4]^3,
    margins U[0.01,0.2]) in both forms, and the 4M convex-pair batch (GJK/EPA)."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    out = {}
    dev = flush.device
    if args.only == "shapes":
        return {"shapes": _run_shapes(args, stream, flush)}
    if args.only == "c0":
        return {"c0": _run_c0(args, stream, flush)}
    if args.only == "refit":
        return {"refit": _run_refit(args, stream, flush)}
    if args.only == "contacts":
        return {"contacts": _run_contacts(args, meshes, stream, flush)}
    if args.only == "ccd":
        return {"ccd": _run_ccd(args, meshes, stream, flush)}
    if args.only == "front":
        return {"front": _run_front(args, meshes, stream, flush)}
    if meshes is None:  # the distance section alone: the mesh set of the C1/C2 workloads
        w1 = _workload(args, 0)
        meshes = [api.BVHModel.from_arrays(*m) for m in w1.meshes]
    w2 = W.config2(total_poses=int(1_000_000 * args.scale), n_pairs=args.pairs, tri_hi=args.tri_hi)
    tf2 = torch.from_numpy(w2.tf2).to(dev)
    pq = torch.from_numpy(w2.pair).to(dev)
    mg = torch.from_numpy(w2.margin).to(dev)

    def dist(prec, t=tf2, p=pq, m=mg):
        return api.distance_batch(meshes, w2.pairs, None, t, pair_of_query=p, nearest_points=True, precision=prec,
                                  margins=m, stream=stream.cuda_stream)

    ms32 = _time_device(lambda: dist("fp32"), 2, 1, stream, flush)
    sub = torch.from_numpy(np.sort(np.random.default_rng(7).choice(w2.n, size=max(1, w2.n // 10),
                                                                     replace=False))).to(dev)
    t_s, p_s, m_s = tf2[sub].contiguous(), pq[sub].contiguous(), mg[sub].contiguous()
    ms64 = _time_device(lambda: dist("fp64", t_s, p_s, m_s), 1, 1, stream, flush)
    a = dist("fp32", t_s, p_s, m_s)
    b = dist("fp64", t_s, p_s, m_s)
    torch.cuda.synchronize()
    d32, d64 = a["min_distance"].cpu().numpy(), b["min_distance"].cpu().numpy()
    rel = np.abs(d32 - d64) / np.maximum(np.abs(d64), 1e-300)
    out["distance"] = {
        "workload": "c2_distance_1M_poses_64pairs", "queries": w2.n,
        "fp32_value": w2.n / (ms32 / 1000.0), "fp64_value": sub.numel() / (ms64 / 1000.0), "unit": "queries/s",
        "fp32_ms_per_step": ms32, "fp64_ms_per_step_on_subset": ms64, "subset": int(sub.numel()),
        "max_rel_err_vs_fp64": float(rel.max()), "p99_rel_err_vs_fp64": float(np.percentile(rel, 99)),
        "within_margin_equal": bool(torch.equal(a["within_margin"], b["within_margin"])),
    }
    if not args.no_cpu:
        from oracle import pyoracle as O
        threads = O.hardware_threads()
        k = min(w2.n, 4000)
        dt = _time_cpu_distance(W.subsample(w2, k, seed=3), threads)
        out["distance"]["cpu_baseline"] = {"value": k / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                                           "sample": f"{k} queries drawn uniformly from the {w2.n}-query workload"}
    if args.only == "distance":
        return out
    out["c0"] = _run_c0(args, stream, flush)
    out["shapes"] = _run_shapes(args, stream, flush)
    out["refit"] = _run_refit(args, stream, flush)
    out["contacts"] = _run_contacts(args, meshes, stream, flush)
    out["ccd"] = _run_ccd(args, meshes, stream, flush)
    out["front"] = _run_front(args, meshes, stream, flush)
    return out


def _run_ccd(args, meshes, stream, flush):
    """fcl::continuousCollide (default request: naive solver, 10 samples, translation
    motion) on the C1 mesh pairs: 100,000 motions drawn like the C1 queries' pairs, each
    starting separated (translation +-U[1.5,4]^3, Haar rotation) and moving towards the
    other object to -U[0,1] times its start translation; CPU baseline = the oracle on all
    host cores (BVHs built beforehand)."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    w1 = _workload(args, 0)
    if meshes is None:
        meshes = [api.BVHModel.from_arrays(*m) for m in w1.meshes]
    n = max(1, int(100_000 * args.scale))
    rng = np.random.default_rng(17)
    pq = w1.pair[rng.integers(0, w1.n, n)].astype(np.int32)
    b0 = W.random_poses(n, 1.5, 4.0, 18)
    b0[:, :, 3] *= rng.choice([-1.0, 1.0], size=(n, 3))
    b1 = b0.copy()
    b1[:, :, 3] *= -rng.uniform(0.0, 1.0, (n, 1))   # towards the other object, ending short of or past it
    dev = flush.device
    t0, t1, tq = (torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (b0, b1, pq))
    res = {}

    def run():
        res["g"] = api.continuous_collide_batch(meshes, w1.pairs, None, None, t0, t1, pair_of_query=tq,
                                                stream=stream.cuda_stream)

    ms = _time_device(run, 2, 1, stream, flush)
    g = res["g"]
    hit = g["is_collide"].cpu().numpy()
    toc = g["time_of_contact"].cpu().numpy()
    out = {"workload": f"{n} translation motions over the 64 C1 mesh pairs, 10 samples each", "motions": n,
           "ms_per_step": ms, "value": n / (ms / 1000.0), "unit": "motions/s",
           "colliding_fraction": float(hit.mean()), "mean_time_of_contact_colliding":
               float(toc[hit > 0].mean()) if hit.any() else None}
    from oracle import pyoracle as O
    om = {}
    chk = np.sort(rng.choice(n, size=min(200, n), replace=False))
    ok = True
    for q in chk:
        a, b = w1.pairs[pq[q]]
        for m in (a, b):
            if m not in om:
                om[m] = O.Mesh(*w1.meshes[m])
        h2, t2, _, _ = O.continuous_collide_batch(om[a], om[b], b0[q:q + 1], b1[q:q + 1])
        ok &= bool(h2[0] == hit[q] and t2[0] == toc[q])
    out["oracle_checked_motions"] = int(chk.size)
    out["exact_vs_oracle"] = ok
    if not args.no_cpu:
        threads = O.hardware_threads()
        k = min(n, 1000)
        sel = np.sort(rng.choice(n, size=k, replace=False))
        for p in np.unique(pq[sel]):   # the oracle's BVHs are built before the timed region
            for m in w1.pairs[p]:
                if m not in om:
                    om[m] = O.Mesh(*w1.meshes[m])
        t_start = time.perf_counter()
        for p in np.unique(pq[sel]):
            idx = sel[pq[sel] == p]
            a, b = w1.pairs[p]
            O.continuous_collide_batch(om[a], om[b], b0[idx], b1[idx], nthreads=threads)
        dt = time.perf_counter() - t_start
        out["cpu_baseline"] = {"value": k / dt, "unit": "motions/s", "cores": threads, "kind": "port",
                               "sample": f"{k} of the motions"}
    out["conservative_advancement"] = _run_ca(args, w1, meshes, pq, b0, b1, stream, flush)
    return out


def _run_ca(args, w1, meshes, pq, b0, b1, stream, flush):
    """The same motions with CCDC_CONSERVATIVE_ADVANCEMENT (FCL's oriented OBBRSS node, FP64
    distance traversals until the step is <= 1e-5), one motion per thread: the first half of
    them in one batch (one thread per motion needs a large batch to fill the GPU), host
    inputs through the C ABI (the start collide batch and the CA kernel), after a
    1,000-motion warm-up batch; oracle check on 100 motions."""
    from fcl_gb300 import api
    from oracle import pyoracle as O
    rng = np.random.default_rng(23)
    n = max(1, b0.shape[0] // 2)
    q, a, b = pq[:n], b0[:n], b1[:n]
    res = {}

    def run(k=n):
        res["g"] = api.continuous_collide_batch(meshes, w1.pairs, None, None, a[:k], b[:k], pair_of_query=q[:k],
                                                solver="conservative_advancement")

    run(min(n, 1000))
    t_start = time.perf_counter()
    run()
    dt = time.perf_counter() - t_start
    g = res["g"]
    out = {"workload": f"{n} of those translation motions, conservative advancement", "motions": n,
           "ms_per_step": dt * 1e3, "value": n / dt, "unit": "motions/s", "timing": "host wall clock, host inputs",
           "colliding_fraction": float(g["is_collide"].mean()), "mean_iterations": float(g["iterations"].mean()),
           "max_iterations": int(g["iterations"].max())}
    chk = np.sort(rng.choice(n, size=min(100, n), replace=False))
    om = {}
    ok = True
    for k in chk:
        p0, p1 = w1.pairs[q[k]]
        for m in (p0, p1):
            if m not in om:
                om[m] = O.Mesh(*w1.meshes[m])
        h, t, _, _, it = O.ca_batch(om[p0], om[p1], a[k:k + 1], b[k:k + 1])
        ok &= bool(h[0] == g["is_collide"][k] and t[0] == g["time_of_contact"][k] and it[0] == g["iterations"][k])
    out["oracle_checked_motions"] = int(chk.size)
    out["exact_vs_oracle"] = ok
    if not args.no_cpu:
        threads = O.hardware_threads()
        k = min(n, 400)
        s2 = np.sort(rng.choice(n, size=k, replace=False))
        for p in np.unique(q[s2]):
            for m in w1.pairs[p]:
                if m not in om:
                    om[m] = O.Mesh(*w1.meshes[m])
        t_start = time.perf_counter()
        for p in np.unique(q[s2]):
            idx = s2[q[s2] == p]
            p0, p1 = w1.pairs[p]
            O.ca_batch(om[p0], om[p1], a[idx], b[idx], nthreads=threads)
        dt = time.perf_counter() - t_start
        out["cpu_baseline"] = {"value": k / dt, "unit": "motions/s", "cores": threads, "kind": "port",
                               "sample": f"{k} of the motions"}
    return out


def _run_front(args, meshes, stream, flush):
    """Front-list coherence (collide(node, front_list)) on the C1 mesh pairs: 10,000 C1
    poses; fronts built by a full traversal, then propagated to nearby poses (translation
    +-0.01, rotation +-0.005 rad per Euler angle) with num_max_contacts = 1, against a plain
    collide at the new poses; host inputs through the C ABI, host wall clock.  Oracle check
    of 50 propagated queries (contacts, fronts, statistics)."""
    from fcl_gb300 import api
    from oracle import pyoracle as O
    w1 = _workload(args, 0)
    if meshes is None:
        meshes = [api.BVHModel.from_arrays(*m) for m in w1.meshes]
    rng = np.random.default_rng(29)
    n = max(1, int(10_000 * args.scale))
    sel = np.sort(rng.choice(w1.n, size=n, replace=False))
    pq, tf0 = w1.pair[sel], w1.tf2[sel].reshape(-1, 3, 4)
    ang = rng.uniform(-0.005, 0.005, (n, 3))
    tf1 = tf0.copy()
    for k in range(n):
        cx, cy, cz = np.cos(ang[k])
        sx, sy, sz = np.sin(ang[k])
        Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
        Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
        Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
        tf1[k, :, :3] = tf0[k, :, :3] @ (Rx @ Ry @ Rz)
    tf1[:, :, 3] += rng.uniform(-0.01, 0.01, (n, 3))
    t_start = time.perf_counter()
    base = api.collide_front_batch(meshes, w1.pairs, None, tf0, pair_of_query=pq, num_max_contacts=1 << 30)
    build_s = time.perf_counter() - t_start
    fronts = base["fronts"]
    res = {}

    def prop():
        res["f"] = api.collide_front_batch(meshes, w1.pairs, None, tf1, fronts=fronts, pair_of_query=pq,
                                           num_max_contacts=1, statistics=True)

    def plain():
        res["p"] = api.collide_batch(meshes, w1.pairs, None, tf1, pair_of_query=pq, num_max_contacts=1,
                                     statistics=True)

    prop()
    plain()
    t_start = time.perf_counter()
    prop()
    t_prop = time.perf_counter() - t_start
    t_start = time.perf_counter()
    plain()
    t_plain = time.perf_counter() - t_start
    f, p = res["f"], res["p"]
    out = {"workload": f"{n} C1 poses, fronts propagated to nearby poses, num_max_contacts=1", "queries": n,
           "front_entries": int(base["front"].shape[0]), "front_build_s": build_s,
           "propagate_ms": t_prop * 1e3, "value": n / t_prop, "unit": "queries/s",
           "plain_collide_ms": t_plain * 1e3, "timing": "host wall clock, host inputs",
           "same_verdicts_as_plain": bool(np.array_equal(f["counts"] > 0, p["counts"] > 0)),
           "bv_tests_propagate": int(f["num_bv_tests"].sum()), "bv_tests_plain": int(p["num_bv_tests"].sum())}
    chk = np.sort(rng.choice(n, size=min(50, n), replace=False))
    om = {}
    ok = True
    for k in chk:
        a, b = w1.pairs[pq[k]]
        for m in (a, b):
            if m not in om:
                om[m] = O.Mesh(*w1.meshes[m])
        c, fr, nbv, _ = O.collide_front(om[a], om[b], tf1[k], front=fronts[k], num_max_contacts=1)
        lo, hi = f["contact_offsets"][k], f["contact_offsets"][k + 1]
        ok &= bool(np.array_equal(f["contacts"][lo:hi], c) and np.array_equal(f["fronts"][k], fr)
                   and f["num_bv_tests"][k] == nbv)
    out["oracle_checked_queries"] = int(chk.size)
    out["exact_vs_oracle"] = ok
    return out


def _run_c0(args, stream, flush):
    """The reference's CPU-runnable configuration: the 5,120-triangle perturbed
    ellipsoid pair (radii (1, 0.7, 0.5), B scaled 0.8), 10,000 Haar poses with
    translations U[-2,2]^3; per pose collide (num_max_contacts = 1) and distance with
    nearest points.  Both forms timed on the GPU; every query checked against the
    oracle (collide bit for bit, distance within 1e-6 relative); CPU baseline = the
    oracle on all host cores."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    w = W.config0(n_poses=10_000, seed=1)
    ms = [api.BVHModel.from_arrays(*m) for m in w.meshes]
    dev = flush.device
    tf2 = torch.from_numpy(w.tf2).to(dev)

    def col(prec):
        return api.collide_batch(ms, w.pairs, None, tf2, num_max_contacts=1, precision=prec,
                                 stream=stream.cuda_stream)

    def dist(prec):
        return api.distance_batch(ms, w.pairs, None, tf2, nearest_points=True, precision=prec,
                                  stream=stream.cuda_stream)

    out = {"workload": "c0_5120tri_pair_10k_poses", "queries": w.n, "unit": "queries/s"}
    for name, fn in (("collide", col), ("distance", dist)):
        for prec in ("fp32", "fp64"):
            ms_ = _time_device(lambda: fn(prec), 5, 3, stream, flush)
            out[f"{name}_{prec}_value"] = w.n / (ms_ / 1000.0)
    c = col("fp32")
    d = dist("fp32")
    torch.cuda.synchronize()
    if not args.no_cpu:
        from oracle import pyoracle as O
        threads = O.hardware_threads()
        a, b = O.Mesh(*w.meshes[0]), O.Mesh(*w.meshes[1])
        t0 = time.perf_counter()
        oc, ocont, _, _ = O.collide_batch(a, b, w.tf2, num_max_contacts=1, nthreads=threads)
        t1 = time.perf_counter()
        od, _, opts, _, _ = O.distance_batch(a, b, w.tf2, nearest=True, nthreads=threads)
        t2 = time.perf_counter()
        gd = d["min_distance"].cpu().numpy()
        rel = np.abs(gd - od) / np.maximum(np.abs(od), 1e-9)
        out["oracle_collide_exact"] = bool(np.array_equal(c["counts"].cpu().numpy(), oc) and
                                           np.array_equal(c["contacts"].cpu().numpy(), ocont))
        out["oracle_distance_max_rel_err"] = float(rel.max())
        out["cpu_baseline"] = {"collide_value": w.n / (t1 - t0), "distance_value": w.n / (t2 - t1),
                               "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": "all 10,000 queries"}
    return out


def _run_contacts(args, meshes, stream, flush):
    """collide() with enable_contact (contact position, normal, depth per contact) on a
    5% sample of the C1 queries, num_max_contacts = 100,000: the pair traversal (FP32 +
    FP64 recheck) plus the FP64 contact pass, against the same sample without contact
    geometry; 300 queries checked bit for bit against the oracle; CPU baseline = the
    oracle on all host cores."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    w1 = _workload(args, 0)
    if meshes is None:
        meshes = [api.BVHModel.from_arrays(*m) for m in w1.meshes]
    w = W.subsample(w1, max(1, w1.n // 20), seed=5)
    dev = flush.device
    tf2 = torch.from_numpy(w.tf2).to(dev)
    pq = torch.from_numpy(w.pair).to(dev)
    res = {}

    def run():
        res["g"] = api.collide_contacts_batch(meshes, w.pairs, None, tf2, pair_of_query=pq, num_max_contacts=100000,
                                              precision="fp32", stream=stream.cuda_stream)

    def pairs_only():
        api.collide_batch(meshes, w.pairs, None, tf2, pair_of_query=pq, num_max_contacts=100000, precision="fp32",
                          stream=stream.cuda_stream)

    ms = _time_device(run, 2, 1, stream, flush)
    ms_pairs = _time_device(pairs_only, 2, 1, stream, flush)
    g = res["g"]
    total = int(g["total_contacts"])
    out = {"workload": f"c1 sample of {w.n} queries, enable_contact, num_max_contacts=100000", "queries": w.n,
           "contacts": total, "ms_per_step": ms, "value": w.n / (ms / 1000.0), "unit": "queries/s",
           "contacts_per_s": total / (ms / 1000.0), "pairs_only_ms_per_step": ms_pairs}
    # bit-exact check of a sample against the oracle
    from oracle import pyoracle as O
    rng = np.random.default_rng(2)
    chk = np.sort(rng.choice(w.n, size=min(300, w.n), replace=False))
    off = g["offsets"].cpu().numpy()
    ids, pos = g["contacts"].cpu().numpy(), g["pos"].cpu().numpy()
    nrm, dep = g["normal"].cpu().numpy(), g["depth"].cpu().numpy()
    om = {}
    ok = True
    for q in chk:
        a, b = w.pairs[w.pair[q]]
        for m in (a, b):
            if m not in om:
                om[m] = O.Mesh(*w.meshes[m])
        c, i2, p2, n2, d2 = O.collide_contacts_batch(om[a], om[b], w.tf2[q:q + 1], num_max_contacts=100000)
        r = slice(off[q], off[q + 1])
        ok &= bool(np.array_equal(ids[r], i2) and np.array_equal(pos[r], p2) and np.array_equal(nrm[r], n2)
                   and np.array_equal(dep[r], d2))
    out["oracle_checked_queries"] = int(chk.size)
    out["bit_exact_vs_oracle"] = ok
    if not args.no_cpu:
        threads = O.hardware_threads()
        k = min(w.n, 2000)
        ws = W.subsample(w, k, seed=3)
        for p in np.unique(ws.pair):   # the oracle's BVHs are built before the timed region
            for m in ws.pairs[p]:
                if m not in om:
                    om[m] = O.Mesh(*ws.meshes[m])
        t0 = time.perf_counter()
        for p in np.unique(ws.pair):
            idx = np.nonzero(ws.pair == p)[0]
            a, b = ws.pairs[p]
            O.collide_contacts_batch(om[a], om[b], ws.tf2[idx], num_max_contacts=100000, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": k / dt, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{k} queries drawn uniformly from the {w.n}-query sample"}
    return out


def _run_refit(args, stream, flush):
    """BVHModel update + bottom-up refit (endUpdateModel()) of the largest mesh of the
    C1 set, on a fresh copy of it: the vertices are perturbed (N(0, 0.01^2)) and refitted
    on the device; CPU baseline = the oracle's sequential refit of the same update."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    w1 = _workload(args, 0)
    k = int(np.argmax([t.shape[0] for _, t in w1.meshes]))
    v, t = w1.meshes[k]
    g = api.BVHModel.from_arrays(v, t)
    rng = np.random.default_rng(11)
    frames = [torch.from_numpy(v + rng.normal(0, 0.01, v.shape)).to(flush.device) for _ in range(4)]
    g.update_vertices(frames[0], stream=stream.cuda_stream)  # warm-up
    torch.cuda.synchronize()
    ms = []
    for f in frames[1:]:
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.update_vertices(f, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    out = {"workload": f"bottom-up refit of a {t.shape[0]}-triangle mesh after a vertex update",
           "triangles": int(t.shape[0]), "ms_per_refit": float(np.mean(ms)),
           "value": t.shape[0] / (float(np.mean(ms)) / 1000.0), "unit": "triangles/s"}
    if not args.no_cpu:
        from oracle import pyoracle as O
        o = O.Mesh(v, t)
        t0 = time.perf_counter()
        o.update(frames[1].cpu().numpy())
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": t.shape[0] / dt, "unit": "triangles/s", "cores": 1, "kind": "port",
                               "sample": "one refit of the same mesh (FCL's refit is sequential)"}
    out["build"] = _run_build(args, v, t)
    return out


def _run_build(args, v, t):
    """BVHModel construction (beginModel / addSubModel / endModel, FCL's PCA fit and MEAN
    split) of the same mesh on the GPU (fclgpu_mesh_create_on_device, host arrays in,
    wall clock including the upload) against the host build of the same library, and the
    GPU rebuild of endReplaceModel(refit = false); the trees are compared node for node.
    CPU baseline = the oracle's build (one thread; FCL's build is sequential)."""
    from fcl_gb300 import api
    api.BVHModel.from_arrays(v, t, build="device")  # warm-up
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        d = api.BVHModel.from_arrays(v, t, build="device")
        ts.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    h = api.BVHModel.from_arrays(v, t)
    host_s = time.perf_counter() - t0
    same = all(np.array_equal(a.view(np.uint64), b.view(np.uint64)) if a.dtype == np.float64 else np.array_equal(a, b)
               for a, b in zip(h.get_nodes(), d.get_nodes()))
    rng = np.random.default_rng(12)
    nv = v + rng.normal(0, 0.01, v.shape)
    t0 = time.perf_counter()
    d.replace_vertices(nv, refit=False)
    rebuild_s = time.perf_counter() - t0
    dev_s = float(np.median(ts))
    out = {"workload": f"OBBRSS build of the {t.shape[0]}-triangle mesh", "triangles": int(t.shape[0]),
           "ms_per_build": dev_s * 1e3, "value": t.shape[0] / dev_s, "unit": "triangles/s",
           "host_build_ms": host_s * 1e3, "rebuild_ms": rebuild_s * 1e3, "timing": "host wall clock",
           "identical_to_host_build": bool(same)}
    if not args.no_cpu:
        from oracle import pyoracle as O
        t0 = time.perf_counter()
        O.Mesh(v, t)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": t.shape[0] / dt, "unit": "triangles/s", "cores": 1, "kind": "port",
                               "sample": "one build of the same mesh"}
    return out


def _run_shapes(args, stream, flush):
    """The 4M convex-pair batch (GJK/EPA, closed forms), FP64 reference arithmetic."""
    import torch
    from fcl_gb300 import api
    from fcl_gb300 import workloads as W
    dev = flush.device
    w3 = W.config3(n_pairs=int(4_000_000 * args.scale))
    ss = api.ShapeSet.from_workload(w3.shapes)
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    ia, ib, t1, t2 = d(w3.ia), d(w3.ib), d(w3.tf1), d(w3.tf2)
    ms3 = _time_device(lambda: api.shape_batch(ss, ia, ib, t1, t2, stream=stream.cuda_stream), 2, 1, stream, flush)
    out = {"workload": "c3_convex_4M_pairs_gst_indep", "pairs": w3.n, "value": w3.n / (ms3 / 1000.0),
           "unit": "pairs/s", "ms_per_step": ms3, "form": "fp64"}
    if not args.no_cpu:
        from oracle import pyoracle as O
        threads = O.hardware_threads()
        k = w3.n  # about 1 s on 16 cores
        t0 = time.perf_counter()
        O.shape_batch(w3.shapes, w3.ia[:k], w3.ib[:k], w3.tf1[:k], w3.tf2[:k], nthreads=threads)
        out["cpu_baseline"] = {"value": k / (time.perf_counter() - t0), "unit": "pairs/s",
                               "cores": threads, "kind": "port", "sample": f"all {k} pairs"}
    return out


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def run_gpu(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from fcl_gb300 import api, native
    native.check(native.lib().fclgpu_init(local), "fclgpu_init")
    L = native.lib()

    if args.only != "all":
        # one secondary section on its own (profiling runs); prints that section only
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=torch.device("cuda", local))
        stream = torch.cuda.Stream(device=local)
        if args.only == "serving":
            print(json.dumps({"serving": run_serving(args)}))
        else:
            print(json.dumps(run_secondary(args, None, stream, flush)))
        return

    w = _workload(args, rank)
    t0 = time.time()
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        meshes = list(ex.map(lambda m: api.BVHModel.from_arrays(*m), w.meshes))
    build_s = time.time() - t0

    dev = torch.device("cuda", local)
    tf2 = torch.from_numpy(w.tf2).to(dev)
    pq = torch.from_numpy(w.pair).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream(dev)

    def step(prec, stats=False):
        return api.collide_batch(meshes, w.pairs, None, tf2, pair_of_query=pq, num_max_contacts=100000,
                                 precision=prec, statistics=stats, stream=stream.cuda_stream, budget=args.budget)

    # autotuned knobs of the collide rounds (outside the timed region; results do not
    # depend on them)
    tuning = None
    if not args.no_tune:
        t_tune = time.time()
        tuning = api.autotune_collide(meshes, w.pairs, None, tf2, pair_of_query=pq, num_max_contacts=100000,
                                      sample=args.tune_sample)
        tuning["seconds"] = time.time() - t_tune

    # reference run for exact-hit check and algorithmic byte counts (outside timing)
    ref64 = step("fp64", stats=True)
    fp32 = step("fp32", stats=True)
    torch.cuda.synchronize()
    exact = bool(torch.equal(ref64["counts"], fp32["counts"]) and torch.equal(ref64["contacts"], fp32["contacts"])
                 and torch.equal(ref64["num_bv_tests"], fp32["num_bv_tests"]))
    n_bv = int(fp32["num_bv_tests"].sum())
    n_leaf = int(fp32["num_leaf_tests"].sum())
    n_rc = int(fp32["num_rechecks"].sum())
    total_contacts = int(fp32["total_contacts"])
    n = w.n
    # algorithmic bytes of one launch: 192 B per BV-pair test (two 96-B packed nodes),
    # 96 B per leaf pair (two triangles), 48 B per pose, 4 B count + 8 B per contact
    alg_bytes = 192.0 * n_bv + 96.0 * n_leaf + 48.0 * n + 4.0 * n + 8.0 * total_contacts

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            step(prec)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        launches0 = L.fclgpu_kernel_launch_count()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        kms = []
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            step(prec)
            ev[i][1].record(stream)
            km = C.c_double()
            native.check(L.fclgpu_last_kernel_time(C.byref(km)), "fclgpu_last_kernel_time")
            kms.append(km.value)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        return float(np.sum(ms)), kms, L.fclgpu_kernel_launch_count() - launches0

    with ClockSampler(local) as clk:
        total_ms, kms, launches = timed("fp32", args.steps, args.warmup)
    clocks = clk.summary()
    t_step = _max_over_ranks(total_ms / args.steps, dev, world)
    n_all = _sum_over_ranks(float(n), dev, world)  # ranks hold their own seeded workloads
    value = n_all / (t_step / 1000.0)

    # plain FP64 GPU form (the drop-in denominator), timed on a uniform subset of the
    # queries because it is ~20x slower
    value64 = t64 = None
    kms64 = [float("nan")]
    if not args.no_fp64:
        sub = np.sort(np.random.default_rng(5).choice(n, size=max(1, int(n * args.fp64_scale)), replace=False))
        sub_t = torch.from_numpy(sub).to(dev)
        tf2_s, pq_s = tf2[sub_t].contiguous(), pq[sub_t].contiguous()

        def step64():
            return api.collide_batch(meshes, w.pairs, None, tf2_s, pair_of_query=pq_s, num_max_contacts=100000,
                                     precision="fp64", stream=stream.cuda_stream, budget=args.budget)
        step64()  # warm-up (tables, scratch)
        torch.cuda.synchronize()
        t64s, kms64 = [], []
        for rep in range(FP64_REPEATS):  # L2 flushed before each timed call
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.fill_(float(rep + 1))
            ev0.record(stream)
            step64()
            ev1.record(stream)
            torch.cuda.synchronize()
            km = C.c_double()
            native.check(L.fclgpu_last_kernel_time(C.byref(km)), "fclgpu_last_kernel_time")
            kms64.append(km.value)
            t64s.append(ev0.elapsed_time(ev1))
        t64 = _max_over_ranks(float(np.mean(t64s)), dev, world)
        value64 = _sum_over_ranks(float(sub.size), dev, world) / (t64 / 1000.0)

    # end to end through the host C ABI: pinned host inputs, H2D + kernels + D2H per step
    tf2_h = torch.from_numpy(w.tf2).pin_memory()
    pq_h = torch.from_numpy(w.pair).pin_memory()
    counts_h = torch.empty(n, dtype=torch.int32).pin_memory()
    offs_h = torch.empty(n + 1, dtype=torch.int64).pin_memory()
    cont_h = torch.empty((max(total_contacts, 1), 2), dtype=torch.int32).pin_memory()
    meshes_c = (C.c_void_p * len(meshes))(*[m.handle.value for m in meshes])
    pairs_np = np.ascontiguousarray(w.pairs, np.int32)
    req = native.CollideRequest(100000, native.FP32_RECHECK, 0, args.budget)

    def e2e_step():
        res = native.CollideResult(counts_h.data_ptr(), offs_h.data_ptr(), cont_h.data_ptr(), cont_h.shape[0],
                                   None, None, None, 0)
        native.check(L.fclgpu_collide_batch(meshes_c, len(meshes), pairs_np.ctypes.data, pairs_np.shape[0], n,
                                            pq_h.data_ptr(), None, tf2_h.data_ptr(), C.byref(req), C.byref(res),
                                            stream.cuda_stream), "fclgpu_collide_batch")
        return res

    e2e_ms = []
    if not args.no_e2e:
        e2e_step()
        torch.cuda.synchronize()
    for i in range(0 if args.no_e2e else args.steps):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = e2e_step()
        torch.cuda.synchronize()
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    e2e_hits = bool(np.array_equal(counts_h.numpy(), fp32["counts"].cpu().numpy())) if e2e_ms else None
    t_e2e = _max_over_ranks(float(np.mean(e2e_ms)) if e2e_ms else float("nan"), dev, world)
    h2d = n * (96 + 4)
    d2h = n * 4 + (n + 1) * 8 + total_contacts * 8

    # roofline of the traversal kernel
    peak, peak_kind = _peaks()
    k_ms = float(np.mean(kms))
    achieved = alg_bytes / (k_ms / 1000.0) / 1e9
    # DRAM bytes (read + write) of the round kernels of one timed step of the default
    # workload, from one ncu capture of that step; other workloads have no capture
    default_workload = args.pairs == 64 and args.tri_hi == 200000
    variant = api.get_collide_tuning()[2]
    traffic = C1_TRAFFIC_A + C1_TRAFFIC_B * n if (default_workload and variant == C1_TRAFFIC_VARIANT) else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_kind": peak_kind,
            "kernel": "k_collide_persist (FP32 + FP64 recheck, warp-batched leaves), all rounds of one step",
            "kernel_ms": k_ms, "algorithmic_bytes_per_launch": alg_bytes,
            "traffic_source": "small-case ncu captures (5 % and 20 % of the poses), linear in the queries",
            "dram_gbs_estimated": None if traffic is None else traffic / (k_ms / 1000.0) / 1e9}

    cpu = None
    oracle_checked = (0, None)
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import pyoracle as O
        O.build()
        threads = O.hardware_threads()
        ws = _cpu_sample(w, args.cpu_sample, seed=123)
        results = {}
        dt, _ = _time_cpu(ws, threads, results)
        cpu = {"value": args.cpu_sample / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} queries drawn uniformly from the {n}-query workload"}
        from fcl_gb300 import workloads as W
        oracle_checked = (ws.n, _oracle_check(w, W.subsample_indices(n, args.cpu_sample, 123), results, fp32))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (f64 recheck)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "queries": n, "mesh_pairs": int(w.pairs.shape[0]),
                       "triangles_total": int(sum(m[1].shape[0] for m in w.meshes)),
                       "num_max_contacts": 100000, "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "tuning": tuning},
            "clocks": clocks,
            "e2e": {"value": n_all / (t_e2e / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e, "exact_hits": e2e_hits},
            "gpu_launches": int(launches),
            "roofline": roof,
            "cpu_baseline": cpu,
            "plain_fp64": {"value": value64, "unit": UNIT, "ms_per_step": t64,
                           "kernel_ms": float(np.mean(kms64)), "queries_timed": None if args.no_fp64 else
                           max(1, int(n * args.fp64_scale)), "timed_calls": None if args.no_fp64 else FP64_REPEATS},
            "fp32_vs_fp64_speedup": None if value64 is None else value / value64,
            "exact_hits": exact,
            # the CPU-baseline sample (uniform over the headline queries) checked against
            # the oracle: counts and contact lists in DFS order
            "oracle_checked_queries": oracle_checked[0], "oracle_exact": oracle_checked[1],
            "stats": {"bv_tests": n_bv, "leaf_tests": n_leaf, "fp64_rechecks": n_rc,
                      "recheck_rate": n_rc / max(1, n_bv + n_leaf), "contacts": total_contacts,
                      "colliding_fraction": float((fp32["counts"] > 0).float().mean().item()),
                      "mesh_build_s": build_s},
        }
        if world == 1 and not args.no_secondary:
            line["secondary"] = run_secondary(args, meshes, stream, flush)
        if world == 1 and not args.no_serving:
            line["serving"] = run_serving(args)
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fcl_gb300", choices=["fcl_gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="pose-count scale of the workload")
    ap.add_argument("--pairs", type=int, default=64, help="mesh pairs (64 in the headline workload)")
    ap.add_argument("--tri-hi", type=int, default=200000, help="largest triangle count of the mesh set")
    ap.add_argument("--budget", type=int, default=0, help="BV tests per work item per round (0 = default)")
    ap.add_argument("--cpu-sample", type=int, default=2000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 form")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host end-to-end measurement")
    ap.add_argument("--fp64-scale", type=float, default=0.1,
                    help="fraction of the queries the plain FP64 form is timed on")
    ap.add_argument("--no-serving", action="store_true", help="skip the motion-checking request loop")
    ap.add_argument("--no-tune", action="store_true", help="keep the default collide knobs (no autotuning)")
    ap.add_argument("--no-secondary", action="store_true", help="skip the distance and convex-pair batches")
    ap.add_argument("--only", default="all", choices=["all", "c0", "distance", "shapes", "refit", "contacts", "ccd", "front",
                                                      "serving"],
                    help="run one section alone (profiling); the full line needs 'all'")
    ap.add_argument("--tune-sample", type=int, default=131072, help="queries the autotuner times each setting on")
    ap.add_argument("--serve-objects", type=int, default=0, help="scene objects (0 = the seeded logU draw)")
    ap.add_argument("--serve-requests", type=int, default=3000, help="requests in the Poisson run")
    ap.add_argument("--serve-rate", type=float, default=0.0, help="arrivals/s (0 = 0.5 x measured capacity)")
    ap.add_argument("--serve-step", type=int, default=4096, help="waypoints per loop step")
    ap.add_argument("--serve-cpu-sample", type=int, default=3000, help="requests timed on the CPU baseline")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
