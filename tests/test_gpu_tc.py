"""Tensor-core DFT-GEMM path (16, 32, 48 and 64 px windows): correlation
planes against numpy's FP64 FFT correlation, vectors against the FP64 pass
(the reference's arithmetic on every window; for 48 px, which the
reference's FFT rejects, FP64 planes through its peak search and fit),
argument errors."""
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
# FP16 data split into hi + lo, FP16 constants single: the constants' rounding
SPLIT2_RMS, SPLIT2_MAX, SPLIT2_MISMATCH = 1e-3, 1e-2, 1e-3
BOUNDS = {og.PREC_TC_SPLIT_BF16: (SPLIT_RMS, SPLIT_MAX, SPLIT_MISMATCH),
          og.PREC_TC_SPLIT2_FP16: (SPLIT2_RMS, SPLIT2_MAX, SPLIT2_MISMATCH),
          og.PREC_TC_BF16: (BF16_RMS, BF16_MAX, BF16_MISMATCH),
          og.PREC_TC_SPLIT_FP16: (SPLIT_RMS, SPLIT_MAX, SPLIT_MISMATCH),
          og.PREC_TC_FP16: (FP16_RMS, FP16_MAX, FP16_MISMATCH)}


def _torch():
    return pytest.importorskip("torch")


def reference_planes(a, b, grid, ia=W, mode=og.CORR_COMPLEX):
    """Swapped correlation planes minus the pedestal sum(a) sum(b) (REAL
    mode: the reference's F4 unpacked-out spectrum rows and column zeroed,
    no pedestal), FP64, any window size."""
    wa = np.stack([a[y:y + ia, x:x + ia] for x, y in grid]).astype(np.float64)
    wb = np.stack([b[y:y + ia, x:x + ia] for x, y in grid]).astype(np.float64)
    fa, fb = np.fft.fft2(wa), np.fft.fft2(wb)
    if mode == og.CORR_REAL:
        for f in (fa, fb):
            f[:, 0, :] = 0
            f[:, ia // 2, :] = 0
            f[:, :, 0] = 0
        ped = np.zeros(len(grid))
    else:
        ped = wa.sum((1, 2)) * wb.sum((1, 2))
    r = np.fft.ifft2(fb * np.conj(fa)).real * (ia * ia)
    return np.fft.fftshift(r, axes=(1, 2)) - ped[:, None, None], ped


def run(a, b, step, precision, mode=og.CORR_COMPLEX, limit=False, planes=False, ia=W, dy=None):
    torch = _torch()
    h, w = a.shape
    if ia == 48:   # not a power of 2: a plan of the tensor-core path alone
        plan = og.Plan(w, h, a.dtype, ia, step, dy, mode=mode, limit_search=limit, tensor_core=precision)
    else:
        plan = og.Plan(w, h, a.dtype, ia, step, dy, mode=mode, limit_search=limit)
        plan.set_precision(precision)
    out = {}
    if planes:
        dpl = torch.zeros((plan.n, ia, ia), dtype=torch.float32, device="cuda")
        dped = torch.zeros(plan.n, dtype=torch.float64, device="cuda")
        plan.set_plane_output(dpl.data_ptr(), dped.data_ptr())
    vec, pk = plan.process(a, b)
    plan.status()
    out["vec"], out["peak"], out["grid"] = vec, np.where(pk >= 0, pk & og.PEAK_MASK, pk), plan.grid()
    if planes:
        out["planes"], out["ped"] = dpl.cpu().numpy(), dped.cpu().numpy()
    plan.close()
    return out


def fp64_reference(a, b, step, ia, mode, orc, limit=False):
    """Vectors of the reference's chain on numpy FP64 planes (any window
    size): find_peaks(plane, 2, 1), fit_simple_gaussian, main.cpp:220-236.
    limit: the peak search on the central ia/2 x ia/2 view of the plane
    (the search rectangle dilated by 0.5, rect.cpp:109-126), the fit on the
    whole plane."""
    h, w = a.shape
    grid = orc.grid_offsets(w, h, ia, ia, step, step)
    planes, ped = reference_planes(a, b, grid, ia, mode)
    vec = np.zeros((len(grid), 5))
    peak = np.full(len(grid), -1, np.int64)
    d0, vw = (ia // 4, ia // 2) if limit else (0, ia)
    for i, (x, y) in enumerate(grid):
        plane = planes[i] + ped[i]
        xy, v = orc.find_peaks(np.ascontiguousarray(plane[d0:d0 + vw, d0:d0 + vw]), 2, 1)
        if len(v) < 2:
            continue
        xy = xy + d0
        fx, fy = orc.fit_simple_gaussian(plane, int(xy[0, 0]), int(xy[0, 1]))
        mx, my = x + ia // 2, y + ia // 2
        vec[i] = (mx, h - my, mx - (x + fx), my - (y + fy), v[0] / v[1] if v[1] > 0 else 0.0)
        peak[i] = xy[0, 1] * ia + xy[0, 0]
    return {"vec": vec, "peak": peak, "grid": grid}


def assert_near_ties(got, ref, planes, rtol, ctx):
    """A peak that differs from the reference's is allowed only at a
    near-tie that the operands' rounding can flip: the FP64 plane at the
    kernel's peak within twice the plane tolerance rtol of the reference's
    peak (a second peak of nearly the same height, or a neighbour of nearly
    the same height when the displacement is close to half a pixel)."""
    for i in np.flatnonzero(got["peak"] != ref["peak"]):
        gp, rp = got["peak"][i], ref["peak"][i]
        assert gp >= 0 and rp >= 0, (ctx, i, gp, rp)
        drop = (planes[i].flat[rp] - planes[i].flat[gp]) / np.abs(planes[i]).max()
        assert drop <= 2 * rtol, (ctx, i, gp, rp, drop)


def displacement_error(got, ref):
    same = got["peak"] == ref["peak"]
    d = (got["vec"][:, 2:4] - ref["vec"][:, 2:4])[same]
    d = d[np.isfinite(d).all(1)]
    return np.sqrt(np.mean(d ** 2)), np.abs(d).max(), 1.0 - same.mean()


@pytest.mark.parametrize("precision,rtol", [(og.PREC_TC_SPLIT_BF16, SPLIT_PLANE_RTOL),
                                            (og.PREC_TC_BF16, 1e-2),
                                            (og.PREC_TC_SPLIT_FP16, SPLIT_PLANE_RTOL),
                                            (og.PREC_TC_FP16, 2e-3),
                                            (og.PREC_TC_SPLIT2_FP16, 1e-3)])
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


def full_range_pair(size):
    """Particle images over the whole 16-bit range (peaks to 65535, clipped):
    window sums up to 2^26, beyond FP32's exact integers."""
    return synth.particle_pair(size, size, ppp=0.03, i0_range=(30000, 65000), noise=300.0,
                               displacement=synth.config2_field, dtype=np.uint16, seed=31,
                               full_scale=65535.0)


@pytest.mark.parametrize("ia,step", [(16, 4), (32, 8), (64, 16)])
def test_full_range_uint16(ia, step):
    """16-bit frames over the full range: the split paths' pedestals stay
    exact (integer window sums, a double product), the planes match numpy's
    FP64 correlation and the vectors the FP64 pass."""
    a, b = full_range_pair(512)
    assert a.max() == 65535
    ref = run(a, b, step, og.PREC_FP64, ia=ia)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT_FP16):
        got = run(a, b, step, precision, planes=True, ia=ia)
        planes, ped = reference_planes(a, b, got["grid"], ia)
        assert np.array_equal(got["ped"], ped), "pedestal not exact"
        err = np.abs(got["planes"] - planes).max(axis=(1, 2)) / np.abs(planes).max(axis=(1, 2))
        assert err.max() <= 5 * SPLIT_PLANE_RTOL, f"plane error {err.max():.3e} of the plane peak"
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= SPLIT_RMS and mx <= SPLIT_MAX and mm <= SPLIT_MISMATCH, (precision, rms, mx, mm)


def test_full_range_uint16_48px(orc):
    """48 px windows on full-range 16-bit frames (pixels to 65535): exact
    pedestals, planes against numpy's FP64 correlation, vectors
    against FP64 planes through the reference's peak search and fit (peaks
    equal but for near-ties)."""
    a, b = full_range_pair(512)
    ref = fp64_reference(a, b, 12, 48, og.CORR_COMPLEX, orc)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT_FP16):
        got = run(a, b, 12, precision, planes=True, ia=48)
        planes, ped = reference_planes(a, b, got["grid"], 48)
        assert np.array_equal(got["ped"], ped), "pedestal not exact"
        err = np.abs(got["planes"] - planes).max(axis=(1, 2)) / np.abs(planes).max(axis=(1, 2))
        assert err.max() <= 5 * SPLIT_PLANE_RTOL, f"plane error {err.max():.3e} of the plane peak"
        assert_near_ties(got, ref, planes, 5 * SPLIT_PLANE_RTOL, precision)
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= SPLIT_RMS and mx <= SPLIT_MAX, (precision, rms, mx, mm)


@pytest.mark.parametrize("step", [16, 8])
@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_limited_search_and_u8(step, mode):
    """8-bit frames with the limited search; step 16 runs row tiles (the
    plain form), step 8 vertical tiles (the grouped form); both modes."""
    a, b = synth.config1()
    ref = run(a, b, step, og.PREC_FP64, mode=mode, limit=True)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16):
        got = run(a, b, step, precision, mode=mode, limit=True)
        rms, mx, mm = displacement_error(got, ref)
        rms_t, max_t, mm_t = BOUNDS[precision]
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (step, mode, precision, rms, mx, mm)


@pytest.mark.parametrize("dy", [3, 4, 8])
def test_vertical_tiles_row_steps(dy):
    """Four windows stacked in a grid column at row steps 3, 4 (each image
    row's coefficients copied into every window containing it) and 8 (one
    shared copy of the tile's rows, each window reading it from its own
    row group): planes, exact pedestals and vectors, both split precisions,
    on a 1024^2 crop whose window count leaves a partial last tile."""
    a, b = synth.config2(size=1024)
    a, b = a[:1000, :1000], b[:1000, :1000]
    ref = run(a, b, 8, og.PREC_FP64, dy=dy)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16):
        got = run(a, b, 8, precision, planes=True, dy=dy)
        assert np.array_equal(got["grid"], ref["grid"])
        planes, ped = reference_planes(a, b, got["grid"])
        assert np.array_equal(got["ped"], ped)
        err = np.abs(got["planes"] - planes).max(axis=(1, 2)) / np.abs(planes).max(axis=(1, 2))
        rtol = SPLIT_PLANE_RTOL if precision == og.PREC_TC_SPLIT_BF16 else 1e-3
        assert err.max() <= rtol, (dy, precision, err.max())
        rms, mx, mm = displacement_error(got, ref)
        rms_t, max_t, mm_t = BOUNDS[precision]
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (dy, precision, rms, mx, mm)


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
    # 16 px windows at x = 4 + 8 i: the generic kernel takes any x position
    p16 = og.Plan(260, 256, np.uint16, 16, 8)
    assert p16.grid()[0, 0] == 2
    p16.set_precision(og.PREC_TC_SPLIT_BF16)
    p16.set_precision(og.PREC_TC_SPLIT2_FP16)
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


# ---- 16, 48 and 64 px windows: the dedicated kernels where the grid allows them
# (16 px: x on multiples of 4, row steps up to 6; 48 px: any regular grid;
# 64 px: x on multiples of 8), else the generic tensor-core kernel ------------
GENERIC = [(16, 8), (48, 24), (64, 32)]        # window, step on the 1024^2 u8 pair
GENERIC_PLANE_RTOL = {og.PREC_TC_SPLIT_BF16: 5e-5, og.PREC_TC_BF16: 2e-2,
                      og.PREC_TC_SPLIT_FP16: 1e-4, og.PREC_TC_FP16: 5e-3,
                      og.PREC_TC_SPLIT2_FP16: 2e-3}


@pytest.mark.parametrize("ia,step", GENERIC)
@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_generic_planes_match_fp64_fft(ia, step, mode):
    a, b = synth.config1()
    for precision, rtol in GENERIC_PLANE_RTOL.items():
        got = run(a, b, step, precision, mode=mode, planes=True, ia=ia)
        ref, ped = reference_planes(a, b, got["grid"], ia, mode)
        assert np.array_equal(got["ped"], ped)     # exact: integer sums below 2^24
        err = np.abs(got["planes"] - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
        assert err.max() <= rtol, f"{ia} px {precision}: plane error {err.max():.3e} of the plane peak"


@pytest.mark.parametrize("ia,step", [(16, 4), (48, 12), (64, 16)])
def test_generic_vectors_against_fp64(ia, step, orc):
    """config-2 statistics on a 1024^2 crop at 75 % overlap: every tensor-
    core precision inside its bounds against the FP64 reference (the FP64
    pass for powers of 2, numpy FP64 planes through the reference's peak
    search and fit for 48 px)."""
    a, b = synth.config2(size=1024)
    ref = fp64_reference(a, b, step, ia, og.CORR_COMPLEX, orc) if ia == 48 else run(a, b, step, og.PREC_FP64, ia=ia)
    for precision, (rms_t, max_t, mm_t) in BOUNDS.items():
        got = run(a, b, step, precision, ia=ia)
        assert np.array_equal(got["grid"], ref["grid"])
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (ia, precision, rms, mx, mm)


# ---- 16 px windows on vertical tiles (eight windows stacked in a grid column:
# row steps 1..6, window x positions on multiples of 4 pixels) ----------------
@pytest.mark.parametrize("dy", [1, 3, 4, 6])
@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_tc16_vertical_tiles_planes(dy, mode):
    """Planes of every precision against numpy's FP64 correlation, exact
    pedestals, and every precision's vectors against the FP64 pass, on a 528^2
    crop of the 8-bit pair (partial last tiles in every grid column)."""
    a, b = synth.config1()
    a, b = np.ascontiguousarray(a[:528, :528]), np.ascontiguousarray(b[:528, :528])
    for precision, rtol in GENERIC_PLANE_RTOL.items():
        got = run(a, b, 4, precision, mode=mode, planes=True, ia=16, dy=dy)
        ref, ped = reference_planes(a, b, got["grid"], 16, mode)
        assert np.array_equal(got["ped"], ped)
        err = np.abs(got["planes"] - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
        assert err.max() <= rtol, f"dy {dy} {precision}: plane error {err.max():.3e} of the plane peak"
    ref = run(a, b, 4, og.PREC_FP64, mode=mode, ia=16, dy=dy)
    for precision, (rms_t, max_t, mm_t) in BOUNDS.items():
        got = run(a, b, 4, precision, mode=mode, ia=16, dy=dy)
        assert np.array_equal(got["grid"], ref["grid"])
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (dy, precision, rms, mx, mm)


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_tc16_limited_search_u16(mode):
    """The limited peak search on 16-bit frames (config-2 statistics), and a
    grid whose x positions are not multiples of 4 (the generic kernel).
    On 16 px windows with the 8 px search area a few windows have an
    ill-conditioned fit, which the operands' rounding moves by up to ~5e-3 px
    (split BF16) and ~3e-2 px (two-MMA split, single FP16 constants), both
    kernels alike: the largest errors are held to 1e-2 and 5e-2 px here, the
    RMS to the usual bounds."""
    a, b = synth.config2(size=1024)
    bounds = {og.PREC_TC_SPLIT_BF16: (SPLIT_RMS, 1e-2, SPLIT_MISMATCH),
              og.PREC_TC_SPLIT2_FP16: (SPLIT2_RMS, 5e-2, SPLIT2_MISMATCH)}
    for dx, dy in ((4, 4), (6, 4)):
        ref = run(a, b, dx, og.PREC_FP64, mode=mode, limit=True, ia=16, dy=dy)
        for precision, (rms_t, max_t, mm_t) in bounds.items():
            got = run(a, b, dx, precision, mode=mode, limit=True, ia=16, dy=dy)
            rms, mx, mm = displacement_error(got, ref)
            assert rms <= rms_t and mx <= max_t and mm <= mm_t, (dx, dy, precision, rms, mx, mm)


@pytest.mark.parametrize("ia,step", [(16, 4), (48, 12), (64, 16)])
@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_blank_frames_16_48_64(ia, step, mode):
    """Blank frames through the 16 px vertical-tile and the 48 and 64 px
    one-window-per-tile kernels: every plane is zero, no strict maximum
    anywhere, so every vector is zero and every peak code -1 (the
    reference's find_peaks returns fewer than two peaks)."""
    a = np.zeros((256, 256), np.uint16)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16, og.PREC_TC_BF16):
        if ia == 48:
            plan = og.Plan(256, 256, np.uint16, ia, step, mode=mode, tensor_core=precision)
        else:
            plan = og.Plan(256, 256, np.uint16, ia, step, mode=mode)
            plan.set_precision(precision)
        vec, pk = plan.process(a, a)
        plan.status()
        assert np.all(vec == 0) and np.all(pk == -1), (ia, precision)
        plan.close()


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_tc48_row_alignments(mode, orc):
    """48 px windows on 512^2 crops of the 8- and 16-bit pairs at steps 8,
    12, 10 and 9, whose window rows start on multiples of 8, 4, 2 and 1
    pixels (the kernel's row loads follow): planes of split BF16 and the FP16
    data split against numpy's FP64 correlation, exact pedestals, vectors
    against the reference's peak search and fit on FP64 planes (peaks equal
    but for near-ties, `assert_near_ties`)."""
    pairs = {"u8": synth.config1(), "u16": synth.config2(size=1024)}
    for name, (a, b) in pairs.items():
        a, b = np.ascontiguousarray(a[:512, :512]), np.ascontiguousarray(b[:512, :512])
        for step in (8, 12, 10, 9):
            ref = fp64_reference(a, b, step, 48, mode, orc)
            for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16):
                got = run(a, b, step, precision, mode=mode, planes=True, ia=48)
                assert np.array_equal(got["grid"], ref["grid"])
                planes, ped = reference_planes(a, b, got["grid"], 48, mode)
                assert np.array_equal(got["ped"], ped), (name, step, precision)
                rtol = GENERIC_PLANE_RTOL[precision]
                err = np.abs(got["planes"] - planes).max(axis=(1, 2)) / np.abs(planes).max(axis=(1, 2))
                assert err.max() <= rtol, (name, step, precision, err.max())
                assert_near_ties(got, ref, planes, rtol, (name, step, precision))
                rms, mx, mm = displacement_error(got, ref)
                rms_t, max_t, _ = BOUNDS[precision]
                assert rms <= rms_t and mx <= max_t, (name, step, precision, rms, mx, mm)


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_generic_kernel_64px_unaligned_grid(mode):
    """64 px windows at an x step of 12 pixels (not a multiple of 8) run the
    generic kernel: its planes against numpy's FP64 correlation and its
    vectors against the FP64 pass, split BF16 and the FP16 data split."""
    a, b = synth.config2(size=1024)
    a, b = np.ascontiguousarray(a[:512, :512]), np.ascontiguousarray(b[:512, :512])
    ref = run(a, b, 12, og.PREC_FP64, mode=mode, ia=64)
    for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16):
        got = run(a, b, 12, precision, mode=mode, planes=True, ia=64)
        planes, ped = reference_planes(a, b, got["grid"], 64, mode)
        assert np.array_equal(got["ped"], ped)
        err = np.abs(got["planes"] - planes).max(axis=(1, 2)) / np.abs(planes).max(axis=(1, 2))
        assert err.max() <= GENERIC_PLANE_RTOL[precision], (precision, err.max())
        rms, mx, mm = displacement_error(got, ref)
        rms_t, max_t, mm_t = BOUNDS[precision]
        assert rms <= rms_t and mx <= max_t and mm <= mm_t, (precision, rms, mx, mm)


def test_limited_search_48px(orc):
    """The limited peak search of the 48 px kernel against FP64 planes
    through the reference's peak search on the central view (peaks equal
    but for near-ties); the recipe itself checked first against the FP64
    pass at 64 px."""
    a, b = synth.config2(size=1024)
    a, b = np.ascontiguousarray(a[:512, :512]), np.ascontiguousarray(b[:512, :512])
    fp64_pass = run(a, b, 16, og.PREC_FP64, limit=True, ia=64)
    recipe = fp64_reference(a, b, 16, 64, og.CORR_COMPLEX, orc, limit=True)
    assert np.array_equal(recipe["peak"], fp64_pass["peak"])
    rms, mx, mm = displacement_error(recipe, fp64_pass)
    assert mx <= 1e-6 and mm == 0, (rms, mx, mm)
    for step in (8, 12):
        ref = fp64_reference(a, b, step, 48, og.CORR_COMPLEX, orc, limit=True)
        planes = None
        for precision in (og.PREC_TC_SPLIT_BF16, og.PREC_TC_SPLIT2_FP16):
            got = run(a, b, step, precision, limit=True, ia=48)
            if planes is None:
                planes, _ = reference_planes(a, b, got["grid"], 48)
            assert_near_ties(got, ref, planes, GENERIC_PLANE_RTOL[precision], (step, precision))
            rms, mx, mm = displacement_error(got, ref)
            rms_t, max_t, _ = BOUNDS[precision]
            assert rms <= rms_t and mx <= max_t, (step, precision, rms, mx, mm)


def test_generic_limited_search_and_errors():
    a, b = synth.config1()
    for ia, step in GENERIC:
        ref = run(a, b, step, og.PREC_FP64, limit=True, ia=ia) if ia != 48 else None
        got = run(a, b, step, og.PREC_TC_SPLIT_BF16, limit=True, ia=ia)
        if ref is not None:
            rms, mx, mm = displacement_error(got, ref)
            assert rms <= SPLIT_RMS and mx <= SPLIT_MAX and mm <= SPLIT_MISMATCH, (ia, rms, mx, mm)
    # a 48 px plan takes no FFT precision and no adjoint; 40 px has no kernel
    p48 = og.Plan(256, 256, np.uint16, 48, 8, tensor_core=og.PREC_TC_BF16)
    for prec in (og.PREC_FP32, og.PREC_FP64):
        with pytest.raises(og.OpivError) as e:
            p48.set_precision(prec)
        assert e.value.status == og.ERR_NOT_POW2
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 48, 8)
    assert e.value.status == og.ERR_NOT_POW2
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 40, 8, tensor_core=og.PREC_TC_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 48, 8, tensor_core=og.PREC_FP32)
    assert e.value.status == og.ERR_ARG


def test_tile_shapes_and_autotune():
    """Both tile shapes of the 32 px kernel (four windows stacked in a grid
    column, four side by side in a grid row) meet the split-BF16 bounds
    against the FP64 pass; the autotuner keeps one of them and a pass after
    it equals a pass with that shape set explicitly."""
    torch = _torch()
    a, b = synth.config2(size=1024)
    ref = run(a, b, 8, og.PREC_FP64)
    h, w = a.shape
    plan = og.Plan(w, h, a.dtype, W, 8)
    assert plan.tile() == og.TILE_AUTO            # FFT path: no choice
    plan.set_precision(og.PREC_TC_SPLIT_BF16)
    assert plan.tile() == og.TILE_VERTICAL        # row step 8: stacked by default
    outs = {}
    for tile in (og.TILE_VERTICAL, og.TILE_HORIZONTAL):
        plan.set_tile(tile)
        assert plan.tile() == tile
        vec, pk = plan.process(a, b)
        plan.status()
        got = {"vec": vec, "peak": np.where(pk >= 0, pk & og.PEAK_MASK, pk)}
        rms, mx, mm = displacement_error(got, ref)
        assert rms <= SPLIT_RMS and mx <= SPLIT_MAX and mm <= SPLIT_MISMATCH, (tile, rms, mx, mm)
        outs[tile] = (vec, pk)
    da = torch.from_numpy(a.view(np.int16)).cuda()
    db = torch.from_numpy(b.view(np.int16)).cuda()
    chosen = plan.autotune(da.data_ptr(), db.data_ptr(), w * 2)
    assert chosen in (og.TILE_VERTICAL, og.TILE_HORIZONTAL)
    vec, pk = plan.process(a, b)
    assert np.array_equal(vec, outs[chosen][0]) and np.array_equal(pk, outs[chosen][1])
    with pytest.raises(og.OpivError):
        plan.set_tile(3)
    plan.close()


def test_mma_wait_timeout_reports_status():
    """The failure path of the bounded MMA waits, without a GPU fault: with
    no MMAs issued every CTA's wait runs out (about a second), the pass
    raises ERR_TIMEOUT, and the next normal pass on the same plan and
    context is correct."""
    a, b = synth.config2(size=256)
    h, w = a.shape
    plan = og.Plan(w, h, a.dtype, W, 8)
    plan.set_precision(og.PREC_TC_SPLIT_BF16)
    good, good_pk = plan.process(a, b)
    plan.test_mma_timeout(True)
    with pytest.raises(og.OpivError) as e:
        plan.process(a, b)
    assert e.value.status == og.ERR_TIMEOUT
    plan.test_mma_timeout(False)
    vec, pk = plan.process(a, b)
    assert np.array_equal(vec, good) and np.array_equal(pk, good_pk)
    plan.close()
    fft = og.Plan(w, h, a.dtype, W, 8)
    with pytest.raises(og.OpivError) as e:
        fft.test_mma_timeout(True)
    assert e.value.status == og.ERR_UNSUPPORTED
    fft.close()
