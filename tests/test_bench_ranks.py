"""The replicas' host side of bench.py on CPU: two `gloo` ranks run its rank set-up, barrier and max-over-ranks
reduction (the timing every rank reports goes through them), with no GPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    w, r, local = bench.dist_init()
    bench.barrier(w)
    t = bench.allmax(w, 10.0 + 5.0 * r)  # each rank's time; every rank must get the slowest
    bench.barrier(w)
    q.put((r, w, local, t))
    dist.destroy_process_group()


def test_bench_rank_setup_barrier_and_allmax_with_gloo():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_bench_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_init() == (1, 0, 0)
    bench.barrier(1)
    assert bench.allmax(1, 3.5) == 3.5
