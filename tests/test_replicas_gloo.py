"""Multi-GPU here means independent replicas (no data-path collective).  The
host logic of that path -- max-over-ranks timing, whole-job value, rank-0-only
reporting -- is exercised with world_size-2 gloo process groups on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist = bench.init_dist(world, "gloo")
    w, r, l = bench.dist_env()
    assert (w, r, l) == (world, rank, rank)
    # each replica reports its own elapsed time; the job time is the max
    elapsed = 10.0 + rank
    m = bench.max_over_ranks(dist, elapsed)
    out[rank] = m
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert dict(out) == {0: 11.0, 1: 11.0}


def test_reference_arm_rank_nonzero_exits_quietly(monkeypatch):
    import bench
    args = bench.parse_args(["--impl", "reference", "--steps", "1", "--warmup", "1"])
    assert bench.run_reference(args, world=2, rank=1) is None


def test_launch_count_and_single_rank_helpers():
    import bench
    assert bench.launches_per_rollout(200, False) == 4 * 200 + 3
    assert bench.launches_per_rollout(200, True) == 4 * 200 + 3 + 1 + 199 // 16
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.init_dist(1, "gloo") is None
