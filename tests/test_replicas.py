"""The multi-GPU mode is replicas only: every rank runs the whole workload
independently and the bench reports the slowest rank.  Checked on the CPU
with two gloo ranks, each running the same small implicit step on the oracle
(no GPU involved)."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import time

    import torch
    import torch.distributed as dist

    import bench
    import oracle
    from svfsi_gb300 import problems
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, rank, world)
    p = problems.heats_cube(3, nsteps=2)
    oracle.set_threads(1)
    eq = oracle.OracleEquation(p)
    t0 = time.perf_counter()
    for _ in range(p.nsteps):
        eq.step()
    dt = time.perf_counter() - t0 + 0.01 * rank  # distinct per-rank times
    tmax = bench.max_over_ranks_(dt, world, "cpu")
    times = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(times, torch.tensor([dt], dtype=torch.float64))
    Y = eq.state()[1]
    sums = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(sums, torch.tensor([float(np.sum(Y * Y))], dtype=torch.float64))
    dist.barrier()
    out[rank] = (tmax, max(float(t) for t in times), [float(s) for s in sums],
                 bench.job_value(tmax, world))
    dist.destroy_process_group()


def test_two_gloo_replicas():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=300)
        assert pr.exitcode == 0
    for r in range(2):
        tmax, tgathered, sums, val = out[r]
        assert tmax == tgathered              # max over ranks
        assert sums[0] == sums[1]             # identical replicas
        assert abs(val - tmax / 2) < 1e-15    # whole-job s/step of 2 replicas
