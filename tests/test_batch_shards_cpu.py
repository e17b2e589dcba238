"""Sharding a batch of independent circuits over several GPUs (host logic,
CPU only): the cost-balanced plan, and the reassembly of per-rank results in
circuit order with two gloo ranks on 127.0.0.1."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from pennylane_lightning_kokkos.batch import gather_shards, shard_plan  # noqa: E402


def test_shard_plan_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 1000, size=257).astype(float)
    for world in (1, 2, 3, 8):
        shards = shard_plan(costs, world)
        assert len(shards) == world
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(costs)))
        loads = [costs[s].sum() for s in shards]
        # greedy largest-first: the spread is at most the largest single cost
        assert max(loads) - min(loads) <= costs.max()
        for s in shards:
            assert s == sorted(s)
    assert shard_plan([5.0, 5.0], 4) == [[0], [1], [], []]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    shards = shard_plan(costs, world)
    mine = shards[rank]
    # stand-in results that identify the circuit: <H> = index / 2, gradient = [index, index + 1]
    ev = [i / 2.0 for i in mine]
    grads = [np.array([i, i + 1.0]) for i in mine]
    out = gather_shards(dist, shards, ev, grads)
    q.put((rank, None if out[0] is None else (out[0].tolist(), [g.tolist() for g in out[1]])))
    dist.barrier()
    dist.destroy_process_group()


def test_gather_shards_two_ranks():
    costs = [float(c) for c in np.random.default_rng(1).integers(1, 50, size=23)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[1] is None
    ev, grads = res[0]
    assert ev == [i / 2.0 for i in range(len(costs))]
    assert grads == [[i, i + 1.0] for i in range(len(costs))]
