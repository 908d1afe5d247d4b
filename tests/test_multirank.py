"""The N > 1 host logic of bench.py on CPU: two gloo ranks (127.0.0.1).

Each rank holds its own seeded workload (weak scaling, no exchange on the data path);
the job's time is the slowest rank's and its units are the sum over ranks; the
reference arm runs on rank 0 only."""
import os
import socket
import types

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    args = types.SimpleNamespace(scale=0.002, pairs=4, tri_hi=2000)
    w = bench._workload(args, rank)
    cpu = torch.device("cpu")
    t = bench._max_over_ranks(10.0 * (rank + 1), cpu, world)
    n_all = bench._sum_over_ranks(float(w.n), cpu, world)
    fp = torch.tensor([float(w.n), float(np.asarray(w.tf2).sum())], dtype=torch.float64)
    got = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(got, fp)
    dist.destroy_process_group()
    q.put((rank, t, n_all, [g.tolist() for g in got]))


def test_two_gloo_ranks_weak_scaling():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=240) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n_all, fps in out:
        assert t == 10.0 * world                      # the slowest rank's time
        assert n_all == fps[0][0] + fps[1][0]          # units of all ranks
        assert fps[0][1] != fps[1][1]                  # each rank has its own poses
    assert out[0][3] == out[1][3]                      # every rank saw the same gather


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    args = types.SimpleNamespace(scale=0.002, pairs=4, tri_hi=2000, cpu_sample=10, warmup=0, steps=1, gpus=2)
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
