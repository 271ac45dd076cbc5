"""The reference-typed drop-in header (openpiv-cxx_gb300/cpp/openpiv_gpu.h) on
the GPU.

* The process example's per-window loop with the correlator swapped to
  openpiv::gpu::FFT (tests/cpp/process_dropin.cpp, built here against the
  test-only stand-in types, and against the reference's own headers where
  this machine has them) runs the 1024^2 8-bit pair with 32 px windows at
  50 % step (3,969 windows): its printed vectors equal the oracle's bit for
  bit, in both correlation modes, with and without the limited search, and
  the PocketFFT modes equal the complex mode.
* gpu::process_grid (the whole loop as one pass) matches within the parity
  tolerances: x, y exact, u, v within 1e-4 px.
* FFT::transform, transform_real and auto_correlate (the batch C ABI behind
  gpu::FFT) are bit-identical to the oracle for 4 .. 64 px windows.
"""
import os
import subprocess

import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth
from test_dropin import REFERENCE, build_harness

pytestmark = pytest.mark.gpu

UV_TOL = 1e-4


@pytest.fixture(scope="module")
def harness(tmp_path_factory, lib):
    d = tmp_path_factory.mktemp("dropin")
    exes = {"standin": build_harness(d / "process_dropin")}
    if os.path.isdir(os.path.join(REFERENCE, "openpiv")):
        exes["reference"] = build_harness(d / "process_dropin_ref", REFERENCE)
    a, b = synth.config1()
    fa, fb = d / "a.u8", d / "b.u8"
    a.tofile(fa)
    b.tofile(fb)
    return exes, a, b, str(fa), str(fb)


def run(exe, fa, fb, fft_type, limit, grid=False):
    args = [exe, "1024", "1024", fa, fb, "32", "0.5", fft_type, "1" if limit else "0"]
    if grid:
        args.append("grid")
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return np.array([[float(x) for x in line.split(",")] for line in r.stdout.strip().splitlines()])


def oracle_vectors(orc, a, b, mode, limit):
    grid = orc.grid(1024, 1024, 32, 32, 0.5)
    vec, _, _ = orc.process_windows(a.astype(np.float64), b.astype(np.float64), grid, 32, mode, limit)
    return vec


@pytest.mark.parametrize("kind", ["standin", "reference"])
@pytest.mark.parametrize("fft_type,mode", [("complex", og.CORR_COMPLEX), ("real", og.CORR_REAL)])
@pytest.mark.parametrize("limit", [False, True])
def test_per_window_loop_equals_oracle(harness, orc, kind, fft_type, mode, limit):
    exes, a, b, fa, fb = harness
    if kind not in exes:
        pytest.skip("reference sources not on this machine")
    got = run(exes[kind], fa, fb, fft_type, limit)
    ref = oracle_vectors(orc, a, b, mode, limit)
    assert got.shape == ref.shape
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).any(1).sum()} windows differ"


def test_pocket_modes_equal_complex(harness):
    exes, _, _, fa, fb = harness
    c = run(exes["standin"], fa, fb, "complex", False)
    for t in ("pocket", "pocket_real"):
        p = run(exes["standin"], fa, fb, t, False)
        assert np.array_equal(p, c, equal_nan=True), t


@pytest.mark.parametrize("fft_type,mode", [("complex", og.CORR_COMPLEX), ("real", og.CORR_REAL)])
@pytest.mark.parametrize("limit", [False, True])
def test_process_grid_within_tolerance(harness, orc, fft_type, mode, limit):
    exes, a, b, fa, fb = harness
    got = run(exes["standin"], fa, fb, fft_type, limit, grid=True)
    ref = oracle_vectors(orc, a, b, mode, limit)
    assert np.array_equal(got[:, :2], ref[:, :2])
    assert np.array_equal(np.isnan(got[:, 2:4]), np.isnan(ref[:, 2:4]))
    d = np.nan_to_num(np.abs(got[:, 2:4] - ref[:, 2:4]))
    assert d.max() < UV_TOL


@pytest.mark.parametrize("w", [4, 8, 16, 32, 64])
def test_spectral_api_bit_identical(orc, w):
    rng = np.random.default_rng(100 + w)
    n = 5
    z = rng.normal(size=(n, w, w)) + 1j * rng.normal(size=(n, w, w))
    a = rng.integers(0, 4096, size=(n, w, w)).astype(np.float64)
    b = rng.integers(0, 4096, size=(n, w, w)).astype(np.float64)
    fwd = og.transform_batch(z, og.FORWARD)
    rev = og.transform_batch(z, og.REVERSE)
    oa, ob = og.transform_real_batch(a, b)
    ac = og.auto_correlate_batch(a.astype(np.complex128))
    for k in range(n):
        assert np.array_equal(fwd[k], orc.transform(z[k], -1))
        assert np.array_equal(rev[k], orc.transform(z[k], +1))
        ra, rb = orc.transform_real(a[k], b[k])
        assert np.array_equal(oa[k], ra) and np.array_equal(ob[k], rb)
        # auto_correlate composed from the oracle's transforms: |A|^2 as
        # (A conj A).real, the unnormalised inverse, real part, swapped
        spec = orc.transform(a[k].astype(np.complex128), -1)
        p2 = spec.real * spec.real - spec.imag * (-spec.imag)
        plane = orc.swap_quadrants(orc.transform(p2.astype(np.complex128), +1).real)
        assert np.array_equal(ac[k].real, plane)
        assert not ac[k].imag.any()
