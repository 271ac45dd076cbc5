"""The example program (openpiv-cxx_gb300/examples/process_gb300.cpp, the
reference's examples/process with the per-window loop on the GPU) run on a
synthetic PGM pair; its printed vectors against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from opiv_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "openpiv-cxx_gb300", "lib", "process_gb300")


def write_pgm(path, img):
    h, w = img.shape
    with open(path, "wb") as f:
        f.write(f"P5\n{w} {h}\n255\n".encode())
        f.write(img.astype(np.uint8).tobytes())


@pytest.mark.parametrize("ffttype,mode", [("complex", 1), ("real", 0)])
def test_process_example_matches_oracle(orc, lib, tmp_path, ffttype, mode):
    a, b = synth.config1()
    pa, pb = str(tmp_path / "a.pgm"), str(tmp_path / "b.pgm")
    write_pgm(pa, a)
    write_pgm(pb, b)
    r = subprocess.run([EXE, "-s", "32", "-o", "0.5", "-f", ffttype, pa, pb],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.array([[float(t) for t in line.split(",")] for line in r.stdout.strip().splitlines()])
    grid = orc.grid(1024, 1024, 32, 32, 0.5)
    ref, _, _ = orc.process_windows(a.astype(np.float64), b.astype(np.float64), grid, 32, mode,
                                    False, os.cpu_count() or 4)
    assert got.shape == ref.shape
    assert np.array_equal(got[:, :2], ref[:, :2])
    nan = np.isnan(ref[:, 2:4])
    assert np.array_equal(np.isnan(got[:, 2:4]), nan)
    # printed with 6 significant digits: |u| < 100 -> at most 5e-5 rounding
    assert np.nanmax(np.abs(np.where(nan, 0, got[:, 2:4] - ref[:, 2:4]))) < 1e-4
    assert "processing time" in r.stderr


def test_cpp_facade_batch(lib, tmp_path):
    """The C++ facade's piv_batch (tests/cpp/test_facade_batch.cpp): the
    queue schedule after autotune() equals the streams schedule bit for bit
    on two synthetic pairs through 64/32/16 px passes."""
    exe = tmp_path / "test_facade_batch"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "openpiv-cxx_gb300", "cpp"),
                    os.path.join(ROOT, "tests", "cpp", "test_facade_batch.cpp"),
                    "-L", os.path.join(ROOT, "openpiv-cxx_gb300", "lib"), "-lopenpiv_gb300",
                    "-Wl,-rpath," + os.path.join(ROOT, "openpiv-cxx_gb300", "lib"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
