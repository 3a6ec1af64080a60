"""The N > 1 bench path on the host: each rank renders its own frame range of
one render (seed offset by the frames before it) and the job's time is the
slowest rank's. Two gloo ranks on the CPU; no GPU involved."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 7.5 * rank, device="cpu")
    out[rank] = (bench.rank_seed(1, rank, 64), t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_distinct_samples_and_the_slowest_time():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    seeds = [out[r][0] for r in range(world)]
    times = [out[r][1] for r in range(world)]
    assert seeds == [1, 65]  # rank 1 starts where rank 0's 64 frames end
    assert times == [17.5, 17.5]


def test_single_process_is_its_own_maximum():
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.rank_seed(5, 0, 64) == 5
