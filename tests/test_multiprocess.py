"""N > 1 path on CPU: two gloo ranks each solve their contiguous trajectory shard (the oracle
stands in for the per-GPU solve) and rank 0's gather equals the single-process solve,
including the EM noise streams, which depend on the global trajectory index."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT / "diffeqgpu.jl_gb300"))
    sys.path.insert(0, str(ROOT / "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    import oracle
    from degpu.shard import gather_to_rank0, shard_range
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        B = 1001
        rng = np.random.default_rng(3)
        p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
        u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
        I = shard_range(B, world, rank)
        _, us, _, na, _ = oracle.solve("lorenz", "tsit5", u0[I.start:I.stop], p[I.start:I.stop], [0, 5],
                                       adaptive=True, dt=0.1, L=2, abstol=1e-8, reltol=1e-6, time_f64=True,
                                       nthreads=1)
        g = gather_to_rank0(us)
        # shard_range covers every trajectory exactly once
        cover = gather_to_rank0(np.arange(I.start, I.stop, dtype=np.int64))
        if rank == 0:
            q.put((g, cover))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_match_single_process():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    g, cover = q.get(timeout=240)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    B = 1001
    rng = np.random.default_rng(3)
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    _, us, _, _, _ = oracle.solve("lorenz", "tsit5", u0, p, [0, 5], adaptive=True, dt=0.1, L=2, abstol=1e-8,
                                  reltol=1e-6, time_f64=True)
    assert np.array_equal(cover, np.arange(B))
    assert np.array_equal(g.view(np.uint32), us.view(np.uint32))


@pytest.mark.parametrize("B,world", [(10, 3), (1, 4), (0, 2), (1 << 20, 8)])
def test_shard_range_partition(B, world):
    sys.path.insert(0, str(ROOT / "diffeqgpu.jl_gb300"))
    from degpu.shard import shard_range
    rs = [shard_range(B, world, r) for r in range(world)]
    assert sum(len(r) for r in rs) == B
    assert all(a.stop == b.start for a, b in zip(rs, rs[1:]))
    assert max(len(r) for r in rs) - min(len(r) for r in rs) <= 1
