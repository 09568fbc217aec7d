"""The multi-GPU form of the path is replicas only (nothing in a frame is exchanged between GPUs): the
host-side logic of `bench.py --gpus N` run as two gloo ranks on the CPU - every replica draws its own
frames of the workload, and the job's time is the slowest rank's, which every rank receives."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                       LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (world, rank, rank)
        frames = bench.frame_indices(8, bench.replica_offset(rank))
        ms = bench.max_over_ranks(1.0 + rank * 0.5, world)  # rank 1 is the slower replica
        results[rank] = (frames, ms)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_rank, args=(world, port, results), nprocs=world, join=True)
        res = dict(results)
    assert set(res) == {0, 1}
    f0, ms0 = res[0]
    f1, ms1 = res[1]
    assert ms0 == ms1 == 1.5                      # max over ranks, on every rank
    assert not set(f0) & set(f1)                  # different frames per replica
    assert all(0 <= f < 256 for f in f0 + f1)
    # the job's throughput as the bench reports it: N frames per slowest-rank frame time
    assert world * 1e3 / ms0 == pytest.approx(1333.333, rel=1e-6)


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5, 1) == 2.5
