"""Multi-process replica logic of bench.py on CPU (gloo, world size 2): the
path shards with no data exchange, ranks only agree on timing (max) and
totals (sum)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local, dist = bench.dist_init()
    mx = bench.allreduce_max(dist, 10.0 + rank)
    sm = bench.allreduce_sum(dist, 1.0 + rank)
    bench.barrier(dist)
    q.put((r, w, mx, sm))
    dist.destroy_process_group()


def test_two_rank_reductions():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 and r[2] == 11.0 and r[3] == 3.0 for r in res)
