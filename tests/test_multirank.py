"""The multi-rank host logic of bench.py on two CPU ranks (gloo).

Several GPUs run replicas over independent orientation shards (the path has
no exchange step); the only collective is the max-over-ranks of the step
time.  Checked here without a GPU: shards are distinct per rank and rank 0's
shard is the single-GPU workload; the reduction gives every rank the
slowest rank's time.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        q = bench.rank_shard(256, 0, rank)
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, dist, torch.device("cpu"))
        np.save(os.path.join(out_dir, f"q{rank}.npy"), q)
        np.save(os.path.join(out_dir, f"t{rank}.npy"), np.array([slowest]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_slowest_time(tmp_path):
    world = 2
    tmp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    import bench
    q0, q1 = np.load(tmp_path / "q0.npy"), np.load(tmp_path / "q1.npy")
    np.testing.assert_array_equal(q0, bench.uniform_quaternions(256, 0))  # rank 0 = the 1-GPU workload
    assert not np.any(np.all(np.isclose(q0[:, None, :], q1[None, :, :]), axis=-1))  # disjoint shards
    np.testing.assert_allclose(np.linalg.norm(q1, axis=1), 1.0)
    for r in range(world):
        assert float(np.load(tmp_path / f"t{r}.npy")[0]) == pytest.approx(15.0)


def test_single_rank_needs_no_collective():
    import bench
    assert bench.max_over_ranks(3.5, None, None) == 3.5
