"""The sharded bicrystal batch end to end: two gloo ranks, each stepping its
own contiguous share of one seeded batch (no data crosses ranks), gather their
per-instance results, and the union equals a single-rank run of the whole
batch bit for bit.  Both ranks run on cuda:0; their kernels never wait on one
another, so sharing one GPU is only a matter of time slicing."""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N_INST, STEPS = 6, 40


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _batch(lo, hi):
    from mpf3d.batched import BatchedBicrystals, sample_batch
    dims, q, dT, da = sample_batch(N_INST, seed=11, sizes_xy=(32, 48), sizes_z=(32,))
    return BatchedBicrystals(dims[lo:hi], q[lo:hi], dT[lo:hi], da[lo:hi], base_height=8.0, slots=4)


def _run(lo, hi):
    b = _batch(lo, hi)
    b.step(STEPS, use_graph=False)
    b.check()
    hl, hr, v1, v2 = b.fronts()
    return [np.asarray(x, np.float64) for x in (hl, hr, v1, v2)], [b.dense(i) for i in range(hi - lo)]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "multiphasefield-solidification-v2_gb300"))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        lo, hi = bench.shard_range(N_INST, rank, world)
        obs, dense = _run(lo, hi)
        parts = [None] * world
        dist.all_gather_object(parts, (lo, hi, obs, dense))
        if rank == 0:
            out.put(parts)
    finally:
        dist.destroy_process_group()


def test_two_ranks_step_disjoint_shards_like_one():
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = q.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref_obs, ref_dense = _run(0, N_INST)
    spans = [(lo, hi) for lo, hi, _, _ in parts]
    assert spans == [(0, 3), (3, 6)]
    for lo, hi, obs, dense in parts:
        for a, b in zip(obs, ref_obs):
            assert np.array_equal(a, b[lo:hi])
        for i in range(hi - lo):
            assert np.array_equal(dense[i], ref_dense[lo + i])
