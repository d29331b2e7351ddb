"""The N>1 bench path: independent member shards per rank, no data-path
collective.  Two gloo ranks on the CPU run bench.py's own rank split
(shard_seed), its time reduction (reduce_max_time, the maximum over ranks)
and its whole-job throughput (job_throughput) around a stub integration that
stands in for the GPU work: each rank "integrates" its own shard of seeded
members and reports its own elapsed time."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

B, STEPS = 8, 1440


def _stub_integration(seed, B):
    """Member b of the shard draws its parameters from seed + b, as
    workloads.forced_ensemble does; returns the shard's per-member taurad."""
    return np.array([10.0 ** np.random.default_rng(seed + b).uniform(4.0, 6.0) for b in range(B)])


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    seed = bench.shard_seed(rank)
    taurad = _stub_integration(seed, B)
    elapsed = 0.5 + rank  # per-rank times differ; the job's time is the slowest rank's
    t_max = bench.reduce_max_time(elapsed, world, "cpu")
    value = bench.job_throughput(world, B, STEPS, t_max)
    out[rank] = (seed, taurad.tolist(), t_max, value)
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
    assert out[0][0] != out[1][0]                           # distinct shard seeds
    assert set(out[0][1]).isdisjoint(out[1][1])             # distinct members
    assert out[0][2] == out[1][2] == 1.5                    # both ranks see the max time
    assert out[0][3] == out[1][3] == pytest.approx(2 * B * STEPS / 1.5)


def test_single_rank_reduction_is_identity():
    import bench

    assert bench.reduce_max_time(2.5, 1, "cpu") == 2.5
    assert bench.job_throughput(1, 256, 1440, 2.0) == 256 * 1440 / 2.0
    assert bench.shard_seed(0) == 1234 and bench.shard_seed(3) == 1234 + 300000
