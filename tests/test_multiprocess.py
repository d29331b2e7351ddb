"""The N>1 bench path: independent member shards per rank, no data-path
collective; the host-side timing reduction (max over ranks) and the
aggregate throughput are checked with world_size 2 over gloo on the CPU."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # per-rank shard seeds differ; per-rank elapsed times differ
    seed = 1234 + 100000 * rank
    t = torch.tensor([0.5 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    B = 256
    value = world * B * bench.T_BENCH / float(t)
    out[rank] = (seed, float(t), value)
    dist.destroy_process_group()


def test_two_rank_shards_and_max_time_reduction():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = 29517
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] != out[1][0]            # distinct member shards
    assert out[0][1] == out[1][1] == 1.5     # both ranks see the max time
    assert out[0][2] == pytest.approx(2 * 256 * 1440 / 1.5)
