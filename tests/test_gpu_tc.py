"""Tensor-core DFT-GEMM path (32 x 32 windows): correlation planes against
numpy's FP64 FFT correlation, vectors against the FP64 pass (the
reference's arithmetic on every window), argument errors."""
import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth

pytestmark = pytest.mark.gpu

W = 32
# split BF16 (hi*hi + hi*lo + lo*hi): planes to ~1e-5 of the plane peak,
# displacements far inside the 0.01 px RMS / 0.05 px max target
SPLIT_PLANE_RTOL = 2e-5
SPLIT_RMS, SPLIT_MAX, SPLIT_MISMATCH = 1e-4, 1e-3, 1e-4
# plain BF16: the target itself
BF16_RMS, BF16_MAX, BF16_MISMATCH = 0.01, 0.05, 5e-3
# plain FP16 (11-bit significand, scaled): between the two
FP16_RMS, FP16_MAX, FP16_MISMATCH = 1e-3, 1e-2, 1e-3
BOUNDS = {og.PREC_TC_SPLIT_BF16: (SPLIT_RMS, SPLIT_MAX, SPLIT_MISMATCH),
          og.PREC_TC_BF16: (BF16_RMS, BF16_MAX, BF16_MISMATCH),
          og.PREC_TC_SPLIT_FP16: (SPLIT_RMS, SPLIT_MAX, SPLIT_MISMATCH),
          og.PREC_TC_FP16: (FP16_RMS, FP16_MAX, FP16_MISMATCH)}


def _torch():
    return pytest.importorskip("torch")


def reference_planes(a, b, grid):
    """Swapped correlation planes minus the pedestal sum(a) sum(b), FP64."""
    wa = np.stack([a[y:y + W, x:x + W] for x, y in grid]).astype(np.float64)
    wb = np.stack([b[y:y + W, x:x + W] for x, y in grid]).astype(np.float64)
    r = np.fft.ifft2(np.fft.fft2(wb) * np.conj(np.fft.fft2(wa))).real * (W * W)
    ped = wa.sum((1, 2)) * wb.sum((1, 2))
    return np.fft.fftshift(r, axes=(1, 2)) - ped[:, None, None], ped


def run(a, b, step, precision, mode=og.CORR_COMPLEX, limit=False, planes=False):
    torch = _torch()
    h, w = a.shape
    plan = og.Plan(w, h, a.dtype, W, step, mode=mode, limit_search=limit)
    plan.set_precision(precision)
    out = {}
    if planes:
        dpl = torch.zeros((plan.n, W, W), dtype=torch.float32, device="cuda")
        dped = torch.zeros(plan.n, dtype=torch.float64, device="cuda")
        plan.set_plane_output(dpl.data_ptr(), dped.data_ptr())
    vec, pk = plan.process(a, b)
    plan.status()
    out["vec"], out["peak"], out["grid"] = vec, np.where(pk >= 0, pk & og.PEAK_MASK, pk), plan.grid()
    if planes:
        out["planes"], out["ped"] = dpl.cpu().numpy(), dped.cpu().numpy()
    plan.close()
    return out


def displacement_error(got, ref):
    same = got["peak"] == ref["peak"]
    d = (got["vec"][:, 2:4] - ref["vec"][:, 2:4])[same]
    d = d[np.isfinite(d).all(1)]
    return np.sqrt(np.mean(d ** 2)), np.abs(d).max(), 1.0 - same.mean()


@pytest.mark.parametrize("precision,rtol", [(og.PREC_TC_SPLIT_BF16, SPLIT_PLANE_RTOL),
                                            (og.PREC_TC_BF16, 1e-2),
                                            (og.PREC_TC_SPLIT_FP16, SPLIT_PLANE_RTOL),
                                            (og.PREC_TC_FP16, 2e-3)])
def test_planes_match_fp64_fft(precision, rtol):
    a, b = synth.config1()
    got = run(a, b, 16, precision, planes=True)
    ref, ped = reference_planes(a, b, got["grid"])
    if precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT_FP16):
        assert np.array_equal(got["ped"], ped)     # exact: integer sums below 2^24
    err = np.abs(got["planes"] - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
    assert err.max() <= rtol, f"plane error {err.max():.3e} of the plane peak"


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_vectors_against_fp64_pass(mode):
    """config-2 statistics on a 1024^2 crop (16,129 windows at step 8)."""
    a, b = synth.config2(size=1024)
    ref = run(a, b, 8, og.PREC_FP64, mode=mode)
    for precision, (rms_t, max_t, mm_t) in BOUNDS.items():
        got = run(a, b, 8, precision, mode=mode)
        assert np.array_equal(got["vec"][:, :2], ref["vec"][:, :2]), "window centres differ"
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (precision, rms, mx, mm)


def test_full_pair_split_accuracy():
    """All 259,081 windows of the 4096^2 pair: the headline accuracy."""
    a, b = synth.config2()
    ref = run(a, b, 8, og.PREC_FP64)
    got = run(a, b, 8, og.PREC_TC_SPLIT_BF16)
    rms, mx, mm = displacement_error(got, ref)
    assert rms <= SPLIT_RMS and mx <= SPLIT_MAX and mm <= SPLIT_MISMATCH, (rms, mx, mm)


def test_limited_search_and_u8():
    a, b = synth.config1()
    ref = run(a, b, 16, og.PREC_FP64, limit=True)
    got = run(a, b, 16, og.PREC_TC_SPLIT_BF16, limit=True)
    rms, mx, mm = displacement_error(got, ref)
    assert rms <= SPLIT_RMS and mx <= SPLIT_MAX and mm <= SPLIT_MISMATCH


def test_fp64_pass_equals_certified_fp32_path():
    """The FP64 pass and the default path agree on peaks and vectors
    within the parity tolerance (both follow the reference)."""
    a, b = synth.config1()
    f64 = run(a, b, 16, og.PREC_FP64)
    f32 = run(a, b, 16, og.PREC_FP32)
    assert np.array_equal(f64["peak"], f32["peak"])
    d = np.abs(f64["vec"][:, 2:4] - f32["vec"][:, 2:4])
    assert np.nanmax(d) <= 1e-4


def test_precision_argument_errors():
    a = np.zeros((256, 256), np.uint16)
    p16 = og.Plan(256, 256, np.uint16, 16, 8)
    with pytest.raises(og.OpivError) as e:
        p16.set_precision(og.PREC_TC_SPLIT_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    pf = og.Plan(256, 256, np.float32, 32, 8)
    with pytest.raises(og.OpivError) as e:
        pf.set_precision(og.PREC_TC_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    # 262 px wide: 29 windows span 256 px, centred at x = 3
    podd = og.Plan(262, 256, np.uint16, 32, 8)
    assert podd.grid()[0, 0] == 3
    with pytest.raises(og.OpivError) as e:
        podd.set_precision(og.PREC_TC_SPLIT_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    p = og.Plan(256, 256, np.uint16, 32, 8)
    with pytest.raises(og.OpivError) as e:
        p.set_precision(7)
    assert e.value.status == og.ERR_ARG
    p.set_precision(og.PREC_TC_SPLIT_BF16)
    vec, _ = p.process(a, a)
    assert np.all(vec == 0)       # blank frames: no two peaks anywhere
    p.status()


@pytest.mark.parametrize("variant", ["sparse", "noisy"])
def test_precision_sweep_variants(variant):
    """Low seeding (0.005 ppp) and high noise (sigma 80) on the config-2
    field, 1024^2 crop: both tensor-core precisions inside the target."""
    a, b = synth.config4(variant, size=1024)
    ref = run(a, b, 8, og.PREC_FP64)
    for precision, (rms_t, max_t, mm_t) in BOUNDS.items():
        got = run(a, b, 8, precision)
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (variant, precision, rms, mx, mm)
