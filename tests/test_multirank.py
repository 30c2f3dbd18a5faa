"""The N>1 bench path on CPU: two gloo ranks (one process each), the same
rank-dependent pieces the GPU ranks use -- each rank's panel has its own
seeds (independent colonies, no data exchange), and the reported time is the
slowest rank's (MAX all-reduce), so the job value is units of all ranks over
that time (weak scaling)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        panels = {name: bench.make_workload(name, rank) for name in ("throughput", "uneven", "large")}
        elapsed = 10.0 + 5.0 * rank                      # a slower second rank
        slowest = bench.max_over_ranks(elapsed, world)
        dist.barrier()
        queue.put((rank, {name: wl.seeds.tolist() for name, wl in panels.items()}, slowest,
                   {name: wl.colonies for name, wl in panels.items()}))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_ranks_shard_without_exchange():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = {}
    for _ in range(world):
        rank, seeds, slowest, colonies = queue.get(timeout=240)
        results[rank] = (seeds, slowest, colonies)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for name in ("throughput", "uneven", "large"):
        a, b = set(results[0][0][name]), set(results[1][0][name])
        assert a.isdisjoint(b), name                      # disjoint colony seeds per rank
        assert results[0][2][name] == results[1][2][name]  # same per-rank work (weak scaling)
    assert results[0][1] == results[1][1] == 15.0          # both report the slowest rank's time
    # whole-job value = all ranks' units over the slowest time
    units = results[0][2]["throughput"] * 32 * 20
    assert np.isclose(world * units / results[0][1], 2 * units / 15.0)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert not torch.distributed.is_initialized()
