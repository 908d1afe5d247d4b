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
    t0 = time.perf_counter()

    def submitter():
        for i, r in enumerate(requests):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
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
    return {
        "requests": len(requests),
        "arrival_rate_per_s": rate,
        "offered_seconds": float(arrivals[-1]),
        "seconds": t_end - t0,
        "throughput_requests_per_s": len(requests) / (t_end - t0),
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "mean_ms": float(lat.mean()),
        "max_ms": float(lat.max()),
        "queue_p50_ms": float(np.percentile(queue, 50)),
        "results": results,
    }
