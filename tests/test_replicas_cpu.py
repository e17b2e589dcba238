"""Replica (N > 1) path of bench.py on CPU: two gloo ranks on 127.0.0.1.

Each rank runs an independent workload; the reported value is the bytes of
all ranks over the slowest rank's time, and the reference arm runs on rank 0
only (the other ranks exit without work)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [10.0, 25.0][rank]
    nbytes = [1e9, 3e9][rank]
    out = bench.aggregate_ranks(dist, torch, ms, nbytes)
    ref = bench.run_reference_arm(bench.parse_args(["--impl", "reference", "--steps", "1", "--warmup", "0",
                                                    "--nq", "8"]), rank)
    q.put((rank, out, ref is None))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_aggregate_and_reference_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        r, out, ref_none = q.get(timeout=180)
        res[r] = (out, ref_none)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert res[r][0] == (25.0, 4e9)  # max time, summed bytes on every rank
    assert res[0][1] is False  # rank 0 runs the reference arm
    assert res[1][1] is True   # other ranks return without work
