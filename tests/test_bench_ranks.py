"""bench.py's multi-rank host logic on CPU: two gloo ranks (one process per
GPU in a real run; the path shards nothing, so each rank runs a replica).

Every rank joins the process group, the timed totals are reduced with the
maximum over ranks, the barrier brackets the timed region, and under
--impl reference only rank 0 works and prints. No GPU is touched.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank), XFEM_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    bench.barrier(w)
    total = bench.reduce_max(1.0 + rank, w)
    printed = []
    orig_print = print
    try:
        import builtins
        builtins.print = lambda *a, **k: printed.append(a)
        # the reference arm: rank 0 alone runs it; the other ranks return at once
        if r != 0:
            bench.run_reference(None, w, r)
    finally:
        builtins.print = orig_print
    bench.barrier(w)
    out.put((r, w, local, total, len(printed)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_split_the_reference_arm():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, out)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 2.0 for r in res)  # the maximum over ranks, on every rank
    assert res[1][4] == 0  # rank 1 printed nothing for the reference arm


def test_single_rank_needs_no_process_group(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.delenv("RANK", raising=False)
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (1, 0, 0)
    assert bench.reduce_max(3.5, w) == 3.5
    bench.barrier(w)
