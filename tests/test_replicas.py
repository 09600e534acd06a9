"""The multi-GPU (replica) host logic with two gloo ranks on the CPU.

Each rank takes its shard of a batch of slices, projects it with the CPU
oracle (standing in for its GPU), and the shards gathered over the group
equal the unsharded result; the job time is the max over ranks.
"""
import os
import socket

import numpy as np
import pytest

from pridediff_gb300.replicas import max_over_ranks, shard, shard_bounds


def test_shard_bounds_cover_every_item_once():
    for n in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_bounds(n, r, world)
                seen.extend(range(lo, hi))
                assert hi - lo in (n // world, n // world + 1)
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(5)
        imgs = rng.random((5, 24, 20)).astype(np.float32)
        ang = (np.arange(30) * 2 * np.pi / 30).astype(np.float32)
        opt = [20, 24, 31, 1.0, 1.0, 1.2, 300.0, 600.0, 0.0, 0.0, 0.0]
        mine = np.stack(shard(list(imgs), rank, world))
        sino = oracle.run2d("flat", "proj", mine, ang, opt, "f", 1)
        # gather the shards in rank order (test only; the product path has no collective)
        sizes = [None] * world
        dist.all_gather_object(sizes, sino.shape[0])
        parts = [None] * world
        dist.all_gather_object(parts, sino)
        t = max_over_ranks(1.0 + rank)
        if rank == 0:
            whole = oracle.run2d("flat", "proj", imgs, ang, opt, "f", 1)
            out.put((np.array_equal(np.concatenate(parts), whole), sizes, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_project_and_reduce():
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    equal, sizes, t = q.get(timeout=10)
    assert equal
    assert sizes == [3, 2]
    assert t == 2.0
