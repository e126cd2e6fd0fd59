"""The N>1 host path on the CPU: two gloo ranks, as bench.py runs them under torchrun.

Windows are independent, so ranks share no data: each verifies its own seeded batch and
the only collectives are the host-side barrier, max of the timed seconds and sum of the
integers. Shards of one range tile it exactly (sieve/rung_scan3.cpp:1022-1027)."""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as td  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "erdos-strauss_gb300"))
    import bench
    import workloads
    ws, r, local = bench.dist()
    assert (ws, r, local) == (world, rank, rank)
    wins = workloads.batch_windows(64, seed=workloads.SEED + r)
    ints = bench.integers(wins)
    bench.barrier(ws)
    total = bench.allsum(ws, ints)
    slowest = bench.allmax(ws, 1.0 + r)
    # each rank's shard of one range, gathered to check the tiling
    lo, hi = 10 ** 12, 10 ** 12 + 987654321
    a, b = workloads.shard_bounds(lo, hi, r, ws)
    t = torch.tensor([a, b], dtype=torch.int64)
    gathered = [torch.zeros(2, dtype=torch.int64) for _ in range(ws)]
    td.all_gather(gathered, t)
    out[r] = (ints, total, slowest, [tuple(int(x) for x in g.tolist()) for g in gathered], wins[0])
    td.destroy_process_group()


def test_two_gloo_ranks_weak_scaling_and_shard_tiling():
    world = 2
    mgr = mp.get_context("spawn").Manager()     # no fork: earlier tests may have left threads
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    (i0, t0, m0, sh0, w0), (i1, t1, m1, sh1, w1) = out[0], out[1]
    assert t0 == t1 == i0 + i1                 # all ranks' integers
    assert m0 == m1 == 2.0                     # the slowest rank's time
    assert w0 != w1                            # each rank its own windows
    assert sh0 == sh1
    lo, hi = 10 ** 12, 10 ** 12 + 987654321
    assert sh0[0][0] == lo and sh0[-1][1] == hi
    assert all(sh0[i][1] == sh0[i + 1][0] for i in range(world - 1))


def test_reference_arm_rank_other_than_zero_does_no_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        windows, warmup, steps, cpu_windows = 4, 0, 1, 2
    called = []
    monkeypatch.setattr(bench, "cpu_baseline", lambda *a, **k: called.append(1))
    bench.run_reference(A(), 2, 1)
    assert not called


def test_shard_bounds_tile_including_empty_shards():
    sys.path.insert(0, os.path.join(ROOT, "erdos-strauss_gb300"))
    import workloads
    for lo, hi, n in ((100, 107, 8), (10 ** 12, 10 ** 12 + 5, 7), (5, 5, 3), (10 ** 18, 10 ** 18 + 10 ** 9, 64)):
        prev = lo
        for i in range(n):
            a, b = workloads.shard_bounds(lo, hi, i, n)
            assert a <= b
            if a < hi:
                assert a == prev
                prev = b
        assert prev == hi
