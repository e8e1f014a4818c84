"""The multi-GPU path's host logic (bench.py under torchrun: replicas, one rank a GPU, no data-path collective), run as
two `gloo` ranks on the CPU: the slowest rank's time is what every rank reports, the job's value is the ranks' paths
over it, and two replicas of the same render (the oracle standing in for each rank's GPU) give the same picture.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle
    from shadytracer_gb300 import scenes
    # each rank's own time for its replica; the job reports the slowest
    ms = bench.reduce_max(100.0 + 50.0 * rank, dist)
    s = scenes.floor_furnace(width=16, height=16)
    r = oracle.render(s, 2, threads=1)
    dist.barrier()
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), r.rgb)
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write("%r %r" % (ms, bench.replica_value(world, 16 * 16 * 2, ms)))
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    world, port = 2, free_port()
    mp.start_processes(rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    vals = [open(tmp_path / ("rank%d.txt" % k)).read().split() for k in range(world)]
    for ms, v in vals:
        assert float(ms) == 150.0                                     # the slowest rank's time, on every rank
        assert float(v) == pytest.approx(2 * 512 / 0.150 / 1e6)
    a, b = np.load(tmp_path / "rank0.npy"), np.load(tmp_path / "rank1.npy")
    assert np.array_equal(a, b)                                       # replicas: the same render, bit for bit


def test_one_rank_needs_no_group():
    import bench
    assert bench.reduce_max(7.5) == 7.5
    assert bench.replica_value(1, 1_000_000, 1000.0) == pytest.approx(1.0)
