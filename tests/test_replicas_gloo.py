"""The multi-process (replica) plumbing of bench.py on CPU: world size 2 over
gloo, barrier and max-over-ranks timing (one process per GPU on a box)."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup("gloo")
    assert (w, r, local) == (ws, rank, rank)
    bench.barrier(w)
    # each replica reports its own step time; the job's time is the slowest
    out[rank] = bench.max_over_ranks(w, 10.0 + rank)
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_barrier_and_max_over_ranks():
    ws = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, ws, port, out)) for r in range(ws)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 11.0, 1: 11.0}

