"""The N>1 host path of bench.py on CPU: two gloo ranks on 127.0.0.1 check the
max/sum reductions the bench times with and the instance sharding of the
bicrystal batch (disjoint, covering, balanced)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mx = bench.max_over_ranks(10.0 + 5.0 * rank, world)
        sm = bench.sum_over_ranks(1.0 + rank, world)
        lo, hi = bench.shard_range(1001, rank, world)
        got = torch.tensor([lo, hi], dtype=torch.int64)
        parts = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(parts, got)
        out.put((rank, mx, sm, [tuple(p.tolist()) for p in parts]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, parts in res:
        assert mx == 15.0          # the slowest rank's time
        assert sm == 3.0
        assert parts == [(0, 501), (501, 1001)]


@pytest.mark.parametrize("n,world", [(0, 2), (1, 4), (7, 3), (512, 8), (1001, 2)])
def test_shard_range_partitions(n, world):
    import bench
    spans = [bench.shard_range(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    sizes = [hi - lo for lo, hi in spans]
    assert max(sizes) - min(sizes) <= 1


def test_single_rank_reductions_are_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.sum_over_ranks(2.0, 1) == 2.0
