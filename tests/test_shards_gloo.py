"""The multi-GPU host logic (shots sharded over ranks, gradient sum, max-time
over ranks) with world_size 2 over gloo on CPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from taichi_sim_gb300 import shards


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shot_gradient(shot, shape=(6, 5)):
    """Stand-in for one shot's gradient: deterministic per shot."""
    rng = np.random.default_rng(1000 + shot)
    return rng.standard_normal(shape)


def _worker(rank, size, port, n_shots, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=size)
    try:
        mine = shards.shot_shard(n_shots)
        grad = torch.zeros(6, 5, dtype=torch.float64)
        for s in mine:
            grad += torch.as_tensor(_shot_gradient(s))
        shards.reduce_gradients([grad])
        slowest = shards.max_over_ranks(1.0 + rank)
        out.put((rank, mine, grad.numpy(), slowest))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n_shots", [16, 7])
def test_shots_sharded_and_gradients_summed_over_two_ranks(n_shots):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_shots, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort(key=lambda r: r[0])
    shots = sorted(s for _, mine, _, _ in results for s in mine)
    assert shots == list(range(n_shots))                      # every shot exactly once
    full = sum(_shot_gradient(s) for s in range(n_shots))
    for _, _, grad, slowest in results:
        np.testing.assert_allclose(grad, full, rtol=1e-12)   # both ranks hold the total
        assert slowest == 2.0                                 # max over ranks


def test_shard_helpers_single_process():
    assert shards.world() == (0, 1)
    parts = [shards.shot_shard(10, r, 3) for r in range(3)]
    assert parts == [[0, 1, 2, 3], [4, 5, 6], [7, 8, 9]]
    costs = [512 * 768 * 64, 768 * 768 * 64, 1024 * 768 * 64]
    owned = [shards.weighted_shard(costs, r, 2) for r in range(2)]
    assert sorted(owned[0] + owned[1]) == [0, 1, 2] and owned[0] == [2]
    with pytest.raises(ValueError):
        shards.shot_shard(4, 2, 2)
