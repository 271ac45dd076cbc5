"""The multi-GPU form of the path is replicas (windows never exchange data):
bench.py's rank bookkeeping -- process group, barrier, max-over-ranks time,
whole-job sum -- checked with two gloo ranks on CPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    r, w, _ = bench.dist_setup()
    assert dist.get_backend() == "gloo"
    bench.dist_barrier(w)
    slowest = bench.dist_max(0.5 + r, w)          # per-rank elapsed seconds
    windows = 1000
    q.put((r, w, slowest, windows * w / slowest))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    pytest.importorskip("torch")
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get() for _ in range(2))
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[2] == 1.5 for o in out)          # both see the slowest rank's time
    assert all(o[3] == pytest.approx(2000 / 1.5) for o in out)
