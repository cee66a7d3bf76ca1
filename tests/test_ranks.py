"""The multi-process path of bench.py (one process per GPU, launched by
torchrun) with two gloo ranks on CPU: the barrier, the max-over-ranks time,
the whole-job value, and the reference arm's rule that only rank 0 works and
prints.  The step shards as independent replicas, so these collectives are
the only exchange there is."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch as th
    import torch.distributed as dist

    import bench

    r, w, local = bench.init_ranks(th)
    bench.barrier(th)
    t = bench.max_over_ranks(th, 0.5 + rank)
    value = bench.job_value(1000, w, t)

    class Args:
        steps = 1
        warmup = 0

    ref_rc = bench.run_reference(Args()) if rank != 0 else None
    bench.barrier(th)
    out.put((r, w, local, dist.get_backend(), t, value, ref_rc))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, out)) for k in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:3] for r in results] == [(0, 2, 0), (1, 2, 1)]
    for r in results:
        assert r[3] == "gloo"
        assert r[4] == 1.5                 # the slowest rank's time on every rank
        assert r[5] == 1000 * 2 / 1.5      # units of both ranks over that time
    assert results[1][6] == 0              # the reference arm: rank 1 returns without work
