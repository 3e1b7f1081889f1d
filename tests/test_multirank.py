"""The multi-rank path of bench.py on CPU: two processes over a gloo group.
Every rank casts its own rays over the replicated scene (weak scaling, no
collective on the data path), and the job's time is the maximum over ranks."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "beamcast-gx-v1.0-beta-_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times = bench.max_over_ranks(dist, [1.5 + rank, 7.0 - rank], torch.device("cpu"))
        rays = bench.rank_rays(rank, 2048)
        q.put((rank, times, rays))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp

    from bcgx import scenes
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, times, rays = q.get(timeout=120)
        out[rank] = (times, rays)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max over ranks, on every rank
    assert out[0][0] == out[1][0] == [2.5, 7.0]
    # rank 0 casts the single-GPU workload's rays; rank 1 its own
    assert np.array_equal(out[0][1], scenes.random_rays(2048, seed=scenes.SEED_RAYS))
    assert not np.array_equal(out[0][1], out[1][1])
    assert out[1][1].shape == (2048, 8)


def test_single_process_max_is_identity():
    import torch

    import bench
    assert bench.max_over_ranks(None, [3.0, 4.0], torch.device("cpu")) == [3.0, 4.0]
