"""Open-loop load generation against a MotionServer: Poisson arrivals at a stated rate,
latency percentiles and throughput.

The server timestamps each request itself (submit -> result ready, on the host's
steady clock), so the numbers include queueing, admission, every step that carried
the request's waypoints and the result readback.
"""
from __future__ import annotations

import threading
import time

import numpy as np


def run_burst(server, requests) -> dict:
    """Submit every request at once and wait for all: capacity in requests/s."""
    t0 = time.perf_counter()
    ids = [server.submit(r.base, r.q) for r in requests]
    res = [server.wait(i) for i in ids]
    dt = time.perf_counter() - t0
    return {"requests": len(requests), "seconds": dt, "requests_per_s": len(requests) / dt, "results": res}


def run_poisson(server, requests, rate: float, seed: int = 0) -> dict:
    """Submit `requests` at Poisson arrival times of the given rate (requests/s) from
    one thread while another collects the results."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(requests))
    arrivals = np.cumsum(gaps) - gaps[0]
    ids: list = [None] * len(requests)
    ready = [threading.Event() for _ in requests]
    results: list = [None] * len(requests)
    submit_at = np.zeros(len(requests))
    t0 = time.perf_counter()

    def submitter():
        for i, r in enumerate(requests):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            submit_at[i] = time.perf_counter() - t0
            ids[i] = server.submit(r.base, r.q)
            ready[i].set()

    th = threading.Thread(target=submitter)
    th.start()
    for i in range(len(requests)):
        ready[i].wait()
        results[i] = server.wait(ids[i])
    th.join()
    t_end = time.perf_counter()
    lat = np.array([r["latency_ms"] for r in results])
    queue = np.array([r["queue_ms"] for r in results])
    # steady state: completions per second over the middle 60 % of the arrival window
    # (the first 20 % fill the pipeline, the drain after the last arrival is excluded); a
    # server that keeps up completes requests at the arrival rate there, and its latency
    # does not grow with the arrival index.  A request completes at its submission plus
    # the latency the server measured (submit -> result), not when this thread, which
    # collects the results in submission order, gets to it.
    T = float(arrivals[-1])
    lo_t, hi_t = 0.2 * T, 0.8 * T
    completed = submit_at + lat / 1e3
    done_in = int(np.count_nonzero((completed >= lo_t) & (completed < hi_t)))
    half = len(requests) // 2
    return {
        "requests": len(requests),
        "arrival_rate_per_s": rate,
        "offered_seconds": T,
        "offered_rate_per_s": (len(requests) - 1) / float(submit_at[-1] - submit_at[0]) if len(requests) > 1 else float("nan"),
        "seconds": t_end - t0,
        "throughput_requests_per_s": len(requests) / (t_end - t0),
        "sustained_requests_per_s": done_in / (hi_t - lo_t) if hi_t > lo_t else float("nan"),
        "latency_first_half_p50_ms": float(np.percentile(lat[:half], 50)) if half else float("nan"),
        "latency_second_half_p50_ms": float(np.percentile(lat[half:], 50)) if half else float("nan"),
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "mean_ms": float(lat.mean()),
        "max_ms": float(lat.max()),
        "queue_p50_ms": float(np.percentile(queue, 50)),
        "results": results,
    }


def main(argv=None) -> None:
    """Command line: build the motion-checking scene (seeded), then run a burst and,
    optionally, Poisson arrivals; prints one JSON line with the engine statistics and
    the broadphase phase times of the last call."""
    import argparse
    import ctypes as C
    import json

    from . import api, native
    from . import workloads as W
    ap = argparse.ArgumentParser(prog="python -m fcl_gb300.serving")
    ap.add_argument("--objects", type=int, default=0, help="scene objects (0 = the seeded draw)")
    ap.add_argument("--burst", type=int, default=16, help="requests submitted at once")
    ap.add_argument("--poisson", type=int, default=0, help="requests at Poisson arrivals after the burst")
    ap.add_argument("--rate", type=float, default=0.0, help="arrivals/s (0 = 0.7 x the burst's rate)")
    ap.add_argument("--step", type=int, default=4096, help="waypoints per loop step")
    ap.add_argument("--seed", type=int, default=4)
    a = ap.parse_args(argv)
    native.check(native.lib().fclgpu_init(0), "fclgpu_init")
    w = W.scene4(n_objects=a.objects or None, seed=a.seed)
    ss = api.ShapeSet.from_workload(w.shapes)
    meshes = [api.BVHModel.from_arrays(v, t) for v, t in w.meshes]
    mgr = api.DynamicAABBTreeCollisionManager(ss, meshes)
    mgr.registerObjects(w.refs, w.tf)
    reqs = W.motion_requests(w, a.burst + a.poisson, seed=a.seed + 1)
    srv = api.MotionServer(mgr, w.robot, max_waypoints_per_step=a.step)
    out = {"objects": w.n}
    b = run_burst(srv, reqs[:a.burst])
    out["burst"] = {k: b[k] for k in ("requests", "seconds", "requests_per_s")}
    if a.poisson:
        p = run_poisson(srv, reqs[a.burst:], a.rate or 0.7 * b["requests_per_s"], seed=a.seed + 2)
        out["poisson"] = {k: v for k, v in p.items() if k != "results"}
    out["engine"] = srv.stats()
    ph = (C.c_double * 16)()
    native.check(native.lib().fclgpu_broadphase_last_phase_ms(C.cast(ph, C.c_void_p)), "fclgpu_broadphase_last_phase_ms")
    out["phases"] = list(ph)
    srv.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
