"""The multi-GPU form of the path is replicas (windows never exchange data):
every rank processes its own image pair, the ranks meet at a barrier, the
time is the slowest rank's and the value the whole job's windows over it.

* Two gloo ranks on CPU run that rank path of bench.py (dist_setup,
  dist_barrier, dist_max) around a real window workload -- each rank its own
  seeded 1024^2 pair through the oracle (the CPU checker stands in for the
  GPU pass here) -- and the test checks every rank's vectors against a
  single-process run and the aggregate against the ranks' own timings.
* `python bench.py --gpus 2` outside torchrun launches two ranks itself
  (checked with the reference arm, which runs on CPU).
* The bench line's DRAM traffic is withheld once the kernel sources differ
  from those its ncu capture ran.
"""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "openpiv-cxx_gb300")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _pair_vectors(orc, pair):
    from opiv_gb300 import synth

    a, b = synth.config1(pair=pair)
    grid = orc.grid(1024, 1024, 32, 32, 0.5)
    vec, pk, secs = orc.process_windows(a.astype(np.float64), b.astype(np.float64), grid, 32, 1,
                                        False, 1)
    return vec, pk, secs


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    for p in (ROOT, PKG):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import bench
    from oracle import oracle

    r, w, _ = bench.dist_setup()
    assert dist.get_backend() == "gloo"
    orc = oracle.get("port")
    bench.dist_barrier(w)
    vec, pk, secs = _pair_vectors(orc, r)        # this rank's replica: its own pair
    slowest = bench.dist_max(secs, w)
    bench.dist_barrier(w)
    q.put((r, w, secs, slowest, vec.shape[0] * w / slowest, vec, pk))
    dist.destroy_process_group()


def test_two_replicas_gloo(orc):
    pytest.importorskip("torch")
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in range(2)), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    slowest = max(o[2] for o in out)
    assert all(o[3] == slowest for o in out)            # every rank sees the slowest time
    assert all(o[4] == pytest.approx(2 * 3969 / slowest) for o in out)
    for r, _, _, _, _, vec, pk in out:                  # each replica's results are its pair's
        ref_vec, ref_pk, _ = _pair_vectors(orc, r)
        assert np.array_equal(pk, ref_pk)
        assert np.array_equal(vec, ref_vec, equal_nan=True)
    assert not np.array_equal(out[0][5], out[1][5])     # two different pairs


def test_bench_launches_its_ranks(orc, tmp_path):
    pytest.importorskip("torch")
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl",
                        "reference", "--steps", "1", "--warmup", "3", "--reference-seconds", "2"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1                               # rank 0 alone prints
    assert lines[0]["impl"] == "reference" and lines[0]["config"]["ranks"] == 2


def test_bench_traffic_tracks_kernel_sources(monkeypatch):
    """The bench line's DRAM traffic comes from an ncu capture of the kernel
    sources it records (SHA-256 prefixes): reported while they match,
    withheld (null, with the reason) once a source differs."""
    import hashlib

    sys.path.insert(0, ROOT)
    import bench

    src = os.path.join(ROOT, "openpiv-cxx_gb300", "csrc", "piv_tc_kernel.cuh")
    with open(src, "rb") as f:
        digest = hashlib.sha256(f.read()).hexdigest()[:16]
    monkeypatch.setitem(bench.KERNEL_TRAFFIC, "tc", {"bytes": 1234, "sources": {"piv_tc_kernel.cuh": digest}})
    nbytes, note = bench.kernel_traffic("tc")
    assert nbytes == 1234 and "ncu capture" in note
    monkeypatch.setitem(bench.KERNEL_TRAFFIC, "tc", {"bytes": 1234, "sources": {"piv_tc_kernel.cuh": "0" * 16}})
    nbytes, note = bench.kernel_traffic("tc")
    assert nbytes is None and "piv_tc_kernel.cuh changed" in note
