"""Target partition across ranks (utc_gb300/shard.py), host side on CPU.

* The splits: the reference's (n // nranks bodies each, one more for the
  first n % nranks ranks, benchapps/nbody/utc-snode-mgpu/mgpu/
  body_task_mgpu.cu:41-49) and the whole-block split of the directed kernel
  cover 0..n-1 once, in rank order.
* Two and three gloo ranks, each advancing only its own targets with the oracle
  (oracle.step_range, the share of one thread of the reference's multi-GPU
  task) and exchanging positions with ShardExchange after every step, end
  with every body's state equal to the single-process oracle run bit for
  bit (each target's sum does not depend on the partition), uneven ranges
  included.
"""
import os
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [0, 1, 5, 7, 1000, 1023, 65537])
@pytest.mark.parametrize("nranks", [1, 2, 3, 8])
def test_splits_cover_every_body_once(n, nranks):
    from utc_gb300.shard import block_split, reference_split

    for ranges in (reference_split(n, nranks), block_split(n, 1024, nranks)):
        assert len(ranges) == nranks
        nxt = 0
        for first, count in ranges:
            assert first == nxt and count >= 0
            nxt = first + count
        assert nxt == n
    counts = [c for _, c in reference_split(n, nranks)]
    assert max(counts) - min(counts) <= 1
    blocks = [(c + 1023) // 1024 for _, c in block_split(n, 1024, nranks)]
    assert max(blocks) - min(blocks) <= 1


def _rank(rank, world, port, n, steps, outdir):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from utc_gb300.shard import ShardExchange, reference_split

    pos, vel = oracle.randomize(1, n, np.float32)
    eps2, damping, dt = np.float32(0.01), np.float32(0.999), np.float32(0.016)
    ranges = reference_split(n, world)
    first, count = ranges[rank]
    ex = ShardExchange(ranges, rank, dtype=torch.float32, device="cpu")
    cur, nxt = pos.copy(), pos.copy()
    for _ in range(steps):
        oracle.step_range(cur, nxt, vel, first, first + count, eps2, damping, dt, nthreads=2)
        ex.all_gather(torch.from_numpy(nxt))  # numpy and torch share the rows
        cur, nxt = nxt, cur
    ex.all_gather(torch.from_numpy(vel))
    np.save(os.path.join(outdir, f"pos{rank}.npy"), cur)
    np.save(os.path.join(outdir, f"vel{rank}.npy"), vel)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n,world", [(1024, 2), (1001, 2), (1001, 3)])
def test_gloo_ranks_equal_the_single_run(tmp_path, n, world):
    import oracle

    oracle.build()
    steps = 5
    ctx = mp.get_context("spawn")
    port = 29530 + (n % 7) + 10 * world
    procs = [ctx.Process(target=_rank, args=(r, world, port, n, steps, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    pos, vel = oracle.randomize(1, n, np.float32)
    want_p, want_v = oracle.step(pos, vel, np.float32(0.01), np.float32(0.999), np.float32(0.016), steps)
    for r in range(world):
        got_p = np.load(tmp_path / f"pos{r}.npy")
        got_v = np.load(tmp_path / f"vel{r}.npy")
        assert got_p.tobytes() == want_p.tobytes()
        assert got_v.tobytes() == want_v.tobytes()
