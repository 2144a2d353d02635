"""bench.py --gpus N runs N independent replicas, one per GPU, with no
collective on the data path: the job's walker updates are the sum over the
ranks and its time is the slowest rank's.  Checked with two gloo ranks on the
CPU (rendezvous on 127.0.0.1)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        from bench import combine_ranks

        # rank r processed 10 (r + 1) updates in 1 + r device seconds and
        # 5 (r + 1) updates in 2 + r seconds end to end
        q.put((rank, combine_ranks(10.0 * (rank + 1), 1.0 + rank, 5.0 * (rank + 1), 2.0 + rank, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_replicas_sum_updates_and_take_the_slowest_time():
    torch_mp = pytest.importorskip("torch.multiprocessing")
    ctx = torch_mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in procs:
            rank, vals = q.get(timeout=120)
            out[rank] = vals
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    # every rank sees the job totals: 10 + 20 updates over max(1, 2) s, and
    # 5 + 10 updates over max(2, 3) s end to end
    assert out[0] == out[1] == (30.0, 2.0, 15.0, 3.0)
