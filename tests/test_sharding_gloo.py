"""Multi-rank host logic on CPU (gloo, world_size 2): the instance partition
of batches, the cross-rank gather and max-time reduction the benchmark uses,
and failure detection when one rank dies before a collective."""
from __future__ import annotations

import os
import socket
import time

import numpy as np
import pytest
import torch.multiprocessing as mp


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_covers_and_balances():
    from fidibench_gb300.batch import random_instances
    from fidibench_gb300.sharding import imbalance, partition_instances
    specs = random_instances(256, 20261203)
    sizes = [int(np.prod(s["n"])) for s in specs]
    for ws in (1, 2, 4, 8):
        parts = partition_instances(sizes, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        assert imbalance(sizes, parts) < 1.01
    assert partition_instances([5, 5, 5], 2) == partition_instances([5, 5, 5], 2)


def _worker(rank, ws, port, q, fail_rank):
    from fidibench_gb300.sharding import (gather_by_index, init_host_group, partition_instances,
                                          reduce_max)
    try:
        dist = init_host_group(rank, ws, "127.0.0.1", port, timeout_s=5.0)
        sizes = [10, 7, 7, 3, 3, 1]
        mine = partition_instances(sizes, ws)[rank]
        if rank == fail_rank:
            os._exit(3)  # a rank that dies between steps
        vals = gather_by_index({i: 100.0 + i for i in mine}, len(sizes))
        t = reduce_max(1.0 + rank)
        q.put((rank, "ok", vals.tolist(), t))
        dist.destroy_process_group()
    except Exception as e:  # noqa: BLE001
        q.put((rank, "error", type(e).__name__, str(e)[:200]))


def _run(ws, fail_rank=-1, wait=60.0):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q, fail_rank)) for r in range(ws)]
    for p in procs:
        p.start()
    out = []
    deadline = time.time() + wait
    expected = ws - (1 if fail_rank >= 0 else 0)
    while len(out) < expected and time.time() < deadline:
        try:
            out.append(q.get(timeout=1.0))
        except Exception:  # noqa: BLE001
            pass
    for p in procs:
        p.join(timeout=10)
        if p.is_alive():
            p.kill()
    return out


def test_gather_and_reduce_two_ranks():
    out = _run(2)
    assert len(out) == 2
    for rank, status, vals, t in out:
        assert status == "ok", (rank, vals)
        assert vals == [100.0 + i for i in range(6)]
        assert t == 2.0


def test_dead_rank_is_detected_not_hung():
    t0 = time.time()
    out = _run(2, fail_rank=1, wait=60.0)
    assert time.time() - t0 < 60.0
    assert len(out) == 1
    rank, status = out[0][0], out[0][1]
    assert rank == 0 and status == "error"


@pytest.mark.parametrize("ws", [3])
def test_three_ranks(ws):
    out = _run(ws)
    assert sorted(o[0] for o in out) == list(range(ws))
    assert all(o[1] == "ok" for o in out)
