"""Host logic of bench.py's multi-GPU mode, run as two gloo ranks on the CPU.

The projection does not shard (one GPU per projection); under torchrun each
rank solves its own seeded instance, and the only collectives are a barrier
and the max-reduce of the timed region's length.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench._dist()
        assert (w, r, local) == (world, rank, rank)
        dist.barrier()
        t_max = bench.reduce_max(10.0 + 5.0 * rank, dist, "cpu")
        case = bench.make_case("c1", r)
        np.save(out / f"r{rank}.npy", np.array([t_max, float(np.sum(case.arrays["ustar"]))]))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_and_seed(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), tmp_path), nprocs=world, join=True)
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    assert r0[0] == r1[0] == 15.0          # every rank gets the slowest rank's time
    assert r0[1] != r1[1]                  # each rank solves its own seeded instance


def test_single_rank_reduce_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_max(3.25, None, "cpu") == 3.25
