"""Multi-GPU host logic on the CPU: two gloo ranks shard a sweep by trial, each solves its
own trials (here with the CPU oracle), and an all-reduce of counts gives the totals of a
single-process run.  The data path has no collective; only the metrics are reduced."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _trials():
    n = np.array([256, 256, 512, 512, 256, 512, 256, 512], np.int32)
    m = np.array([128, 64, 256, 128, 160, 300, 100, 200], np.int32)
    k = np.array([6, 20, 10, 60, 8, 30, 40, 12], np.int32)
    return n, m, k, np.arange(8, dtype=np.uint32)


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gaga_gb300 import sweep
    from oracle import gbo

    n, m, k, tid = _trials()
    idx = sweep.shard(np.arange(len(n)), rank, world)
    ok, iters, err = gbo.solve_dense_trials(n[idx], m[idx], k[idx], 99, tid[idx], threads=1)
    t = torch.tensor([float(ok), float(len(idx)), float(iters.sum())], dtype=torch.float64)
    dist.all_reduce(t)
    out[rank] = t.tolist()
    dist.destroy_process_group()


def test_two_rank_sharding_matches_single_process():
    from oracle import gbo

    n, m, k, tid = _trials()
    ok1, iters1, _ = gbo.solve_dense_trials(n, m, k, 99, tid, threads=1)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    assert out[0] == [float(ok1), float(len(n)), float(iters1.sum())]


def test_rank_waves_are_disjoint():
    from gaga_gb300 import sweep

    world, steps = 4, 5
    waves = [sweep.rank_wave(r, world, s) for r in range(world) for s in range(steps)]
    assert len(set(waves)) == world * steps
    parts = [set(sweep.shard(np.arange(100), r, 3)) for r in range(3)]
    assert set().union(*parts) == set(range(100)) and sum(len(p) for p in parts) == 100


@pytest.mark.parametrize("world", [2, 4, 8, 16])
def test_rank_trials_are_disjoint(world):
    """Every rank's waves hold distinct trials for any world size: the trial ids (the seeds
    of A and x) never repeat across ranks and steps, while the grid points do."""
    from gaga_gb300 import sweep

    steps, total, parts = 3, 3072, 4
    seen = []
    for r in range(world):
        for s in range(steps):
            n, m, k, tid = sweep.wave_trials(total, parts, sweep.rank_wave(r, world, s))
            assert len(tid) == total // parts
            seen.extend(tid.tolist())
    assert len(seen) == len(set(seen))
