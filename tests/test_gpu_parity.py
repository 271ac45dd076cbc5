"""GPU parity: the CUDA path, called through the C ABI, against the oracle
(CPU restatement of the reference, itself pinned to the compiled reference)
and against committed outputs of the compiled reference.

Tolerances (from the path's specification):
  * grid coordinates and integer peak locations: bit-exact;
  * FP32 correlation planes: within 1e-5 of the plane's peak magnitude;
  * exact-mode planes: bit-identical;
  * sub-pixel displacements u, v: within 1e-4 px; NaN where the reference
    has NaN (its log of a non-positive neighbour);
  * x, y: exact; sn: |dsn| <= 1e-5 * sn * (1 + sn) (0 where the reference
    has 0) -- sn = p0 / p1 is a ratio of plane values, which are specified to
    1e-5 of the plane peak p0, so p1 is known to 1e-5 * p0 / p1 = 1e-5 * sn.
"""
import os

import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
UV_TOL = 1e-4
SN_RTOL = 1e-5
PLANE_RTOL = 1e-5
THREADS = os.cpu_count() or 4


def peak_codes(ref_pk, w):
    return np.where(ref_pk[:, 0] >= 0, ref_pk[:, 1] * w + ref_pk[:, 0], -1)


def gpu_codes(pk):
    return np.where(pk >= 0, pk & og.PEAK_MASK, -1)


def assert_vectors_match(vec, pk, ref_vec, ref_pk, w, what=""):
    ref_code = peak_codes(ref_pk, w)
    got_code = gpu_codes(pk)
    bad = np.nonzero(got_code != ref_code)[0]
    assert bad.size == 0, f"{what}: {bad.size} integer peaks differ, first windows {bad[:8]}"
    v = vec.astype(np.float64)
    assert np.array_equal(v[:, 0:2], ref_vec[:, 0:2]), f"{what}: x, y differ"
    nan_ref = np.isnan(ref_vec[:, 2:4])
    assert np.array_equal(np.isnan(v[:, 2:4]), nan_ref), f"{what}: NaN pattern differs"
    d = np.where(nan_ref, 0.0, np.abs(v[:, 2:4] - ref_vec[:, 2:4]))
    assert d.max(initial=0.0) <= UV_TOL, f"{what}: max |du|,|dv| = {d.max()}"
    sn_ref = ref_vec[:, 4]
    assert np.array_equal(v[:, 4] == 0, sn_ref == 0), f"{what}: sn zero pattern differs"
    rel = np.abs(v[:, 4] - sn_ref) / np.maximum(np.abs(sn_ref) * (1 + np.abs(sn_ref)), 1e-30)
    rel = np.where(sn_ref == 0, 0.0, rel)
    assert rel.max(initial=0.0) <= SN_RTOL, f"{what}: max sn error / (sn (1 + sn)) {rel.max()}"


def run_both(orc, a, b, ia, step, mode, limit, dtype=None):
    h, w = a.shape
    plan = og.Plan(w, h, a.dtype if dtype is None else dtype, ia, step, mode=mode,
                   limit_search=limit)
    vec, pk = plan.process(a, b)
    grid = plan.grid()
    ref_vec, ref_pk, _ = orc.process_windows(a.astype(np.float64), b.astype(np.float64), grid, ia,
                                             mode, limit, THREADS)
    exact = plan.exact_count()
    plan.close()
    return vec, pk, ref_vec, ref_pk, exact


# ---- correlation planes ----------------------------------------------------
@pytest.mark.parametrize("w", [8, 16, 32, 64])
@pytest.mark.parametrize("mode", [og.CORR_REAL, og.CORR_COMPLEX])
def test_exact_planes_bit_identical(orc, w, mode):
    rng = np.random.default_rng(100 + w + mode)
    a = rng.integers(0, 4096, (6, w, w)).astype(np.float64)
    b = rng.integers(0, 4096, (6, w, w)).astype(np.float64)
    got = og.cross_correlate_batch(a, b, mode, exact=True)
    for k in range(a.shape[0]):
        ref = orc.cross_correlate(a[k], b[k], mode)
        assert np.array_equal(got[k], ref), f"window {k}: max diff {np.abs(got[k] - ref).max()}"


@pytest.mark.parametrize("w", [16, 32, 64])
@pytest.mark.parametrize("mode", [og.CORR_REAL, og.CORR_COMPLEX])
def test_fp32_planes_within_tolerance(orc, w, mode):
    rng = np.random.default_rng(200 + w + mode)
    a = rng.integers(0, 4096, (16, w, w)).astype(np.float64)
    b = np.roll(a, (1, 2), (1, 2)) + rng.integers(0, 200, a.shape)
    got = og.cross_correlate_batch(a, b, mode, exact=False)
    for k in range(a.shape[0]):
        ref = orc.cross_correlate(a[k], b[k], mode)
        err = np.abs(got[k] - ref).max()
        assert err <= PLANE_RTOL * np.abs(ref).max(), f"window {k}: {err}"
        if mode == og.CORR_COMPLEX:   # the mean-free part alone, same bound
            ped = a[k].sum() * b[k].sum()
            assert err <= PLANE_RTOL * np.abs(ref - ped).max()


def test_planes_vs_reference_fixture():
    z = np.load(os.path.join(GOLDEN, "ref_outputs.npz"))
    for name in ("u8_w32", "u16_w32", "u16_w16"):
        a, b, grid = z[f"{name}/a"], z[f"{name}/b"], z[f"{name}/grid"]
        ia = int(z[f"{name}/meta"][0])
        sel = z[f"{name}/planes_sel"]
        wa = np.stack([a[y:y + ia, x:x + ia] for x, y in grid[sel]]).astype(np.float64)
        wb = np.stack([b[y:y + ia, x:x + ia] for x, y in grid[sel]]).astype(np.float64)
        for mode, mname in ((0, "real"), (1, "complex")):
            ref = z[f"{name}/planes_{mname}"]
            assert np.array_equal(og.cross_correlate_batch(wa, wb, mode, exact=True), ref)
            got = og.cross_correlate_batch(wa, wb, mode, exact=False)
            for k in range(len(sel)):
                assert np.abs(got[k] - ref[k]).max() <= PLANE_RTOL * np.abs(ref[k]).max()


# ---- whole passes ---------------------------------------------------------
def test_process_vs_reference_fixtures():
    z = np.load(os.path.join(GOLDEN, "ref_outputs.npz"))
    for name in ("u8_w32", "u16_w32", "u16_w16"):
        a, b, grid = z[f"{name}/a"], z[f"{name}/b"], z[f"{name}/grid"]
        ia, step = (int(v) for v in z[f"{name}/meta"])
        h, w = a.shape
        for mode, mname in ((0, "real"), (1, "complex")):
            for limit in (0, 1):
                plan = og.Plan(w, h, a.dtype, ia, step, mode=mode, limit_search=limit)
                assert np.array_equal(plan.grid(), grid)
                vec, pk = plan.process(a, b)
                assert_vectors_match(vec, pk, z[f"{name}/vec_{mname}_{limit}"],
                                     z[f"{name}/peak_{mname}_{limit}"], ia, f"{name} {mname} {limit}")
                plan.close()


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
@pytest.mark.parametrize("limit", [False, True])
def test_config1_uint8_1024(orc, mode, limit):
    a, b = synth.config1()
    vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 32, 16, mode, limit)
    assert vec.shape[0] == 3969
    assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, "config1")
    if mode == og.CORR_COMPLEX and not limit:
        u = vec[:, 2].astype(np.float64)
        good = np.abs(u + 2.35) < 0.5
        assert good.mean() > 0.9   # the reference convention: u = -shift


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_config2_uint16_4096_full(orc, mode):
    """All 259,081 windows of the 4096^2 12-bit pair at step 8."""
    a, b = synth.config2()
    vec, pk, ref_vec, ref_pk, exact = run_both(orc, a, b, 32, 8, mode, False)
    assert vec.shape[0] == 509 * 509
    assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, f"config2 mode {mode}")
    print(f"config2 mode {mode}: {exact} windows re-decided by the exact pass")


@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_fp64_pass_equals_oracle_config2(orc, mode):
    """The FP64 all-window pass (every window through the exact kernel), the
    accuracy reference of the tensor-core precisions, on all 259,081 windows
    of the 4096^2 12-bit pair: integer peaks identical to the oracle's and
    every vector equal to the oracle's rounded to float32."""
    a, b = synth.config2()
    plan = og.Plan(4096, 4096, np.uint16, 32, 8, mode=mode)
    plan.set_precision(og.PREC_FP64)
    vec, pk = plan.process(a, b)
    grid = plan.grid()
    plan.close()
    ref_vec, ref_pk, _ = orc.process_windows(a.astype(np.float64), b.astype(np.float64), grid, 32,
                                             mode, False, THREADS)
    assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, f"FP64 pass, mode {mode}")
    assert np.all((pk < 0) | ((pk & og.PEAK_EXACT) != 0)), "a window not decided by the exact kernel"
    r32 = ref_vec.astype(np.float32)
    same = (vec == r32) | (np.isnan(vec) & np.isnan(r32))
    assert same.all(), f"{(~same.all(1)).sum()} vectors differ from the oracle's float32 rounding"


def test_w16_uint16(orc):
    a, b = synth.config2(size=1024)
    for mode in (og.CORR_COMPLEX, og.CORR_REAL):
        for limit in (False, True):
            vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 16, 4, mode, limit)
            assert_vectors_match(vec, pk, ref_vec, ref_pk, 16, f"w16 {mode} {limit}")


def test_w64_uint16(orc):
    """64 x 64 windows (the shared-memory kernel) at step 16 and step 24."""
    a, b = synth.config2(size=1024)
    for step in (16, 24):
        for mode in (og.CORR_COMPLEX, og.CORR_REAL):
            for limit in (False, True):
                vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 64, step, mode, limit)
                assert_vectors_match(vec, pk, ref_vec, ref_pk, 64, f"w64/{step} {mode} {limit}")


def test_float32_frames(orc):
    a, b = synth.config5(size=512)
    for mode in (og.CORR_COMPLEX, og.CORR_REAL):
        vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 32, 16, mode, False)
        assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, f"f32 {mode}")


# ---- edge cases ------------------------------------------------------------
@pytest.mark.parametrize("value", [0, 1, 4095, 65535])
def test_constant_frames_give_no_peaks(orc, value):
    a = np.full((96, 128), value, np.uint16)
    for mode in (og.CORR_COMPLEX, og.CORR_REAL):
        vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, a.copy(), 32, 16, mode, False)
        assert np.all(pk == -1) and np.all(vec == 0)
        assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, "constant")


def test_single_window_and_margins(orc):
    rng = np.random.default_rng(9)
    for (h, w), step in (((32, 32), 16), ((70, 100), 16), ((33, 65), 8), ((47, 131), 13)):
        a = rng.integers(0, 256, (h, w)).astype(np.uint8)
        b = np.roll(a, (1, -2), (0, 1))
        for mode in (og.CORR_COMPLEX, og.CORR_REAL):
            vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 32, step, mode, False)
            assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, f"{h}x{w}/{step}")


def test_saturated_uint16_full_range(orc):
    rng = np.random.default_rng(4)
    a = rng.integers(60000, 65536, (128, 128)).astype(np.uint16)
    b = np.roll(a, (3, 1), (0, 1))
    for mode in (og.CORR_COMPLEX, og.CORR_REAL):
        vec, pk, ref_vec, ref_pk, _ = run_both(orc, a, b, 32, 8, mode, False)
        assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, "saturated")


def test_periodic_windows_use_exact_pass(orc):
    """Periodic windows give exactly tied correlation peaks; the FP32 pass
    must hand them to the exact pass, which must pick the same peak as the
    reference's std::sort."""
    rng = np.random.default_rng(21)
    tile = rng.integers(0, 256, (8, 8)).astype(np.uint8)
    a = np.tile(tile, (16, 16))
    b = np.roll(a, (2, 3), (0, 1))
    for mode in (og.CORR_COMPLEX, og.CORR_REAL):
        vec, pk, ref_vec, ref_pk, exact = run_both(orc, a, b, 32, 16, mode, False)
        assert exact > 0
        assert np.any(pk & og.PEAK_EXACT)
        assert_vectors_match(vec, pk, ref_vec, ref_pk, 32, f"periodic {mode}")


# ---- API behaviour ---------------------------------------------------------
def test_two_launches_per_pass():
    a, b = synth.config1()
    plan = og.Plan(1024, 1024, np.uint8, 32, 16)
    n0 = og.kernel_launch_count()
    plan.process(a, b)
    assert og.kernel_launch_count() - n0 == 2


def test_device_buffers_match_host_call():
    torch = pytest.importorskip("torch")
    a, b = synth.config1()
    plan = og.Plan(1024, 1024, np.uint8, 32, 16)
    vec_h, pk_h = plan.process(a, b)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    dvec = torch.zeros((plan.n, 5), dtype=torch.float32, device="cuda")
    dpk = torch.zeros(plan.n, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    # uploads and fills ran on torch's current stream: order the pass after them
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.process_device(da.data_ptr(), db.data_ptr(), 1024, dvec.data_ptr(), dpk.data_ptr(),
                            s.cuda_stream)
    s.synchronize()
    assert np.array_equal(dvec.cpu().numpy(), vec_h)
    assert np.array_equal(dpk.cpu().numpy(), pk_h)


def test_argument_errors():
    plan = og.Plan(128, 128, np.uint16, 32, 16)
    a = np.zeros((128, 128), np.uint16)
    with pytest.raises(og.OpivError) as e:
        plan.process_into(a.ctypes.data, a.ctypes.data, 100, np.zeros(plan.n * 5, np.float32).ctypes.data, None)
    assert e.value.status == og.ERR_ARG
    with pytest.raises(og.OpivError) as e:
        plan.process(a[:, :64], a[:, :64])
    assert e.value.status == og.ERR_SIZE_MISMATCH
    with pytest.raises(og.OpivError) as e:
        og.Plan(128, 128, np.uint16, 32, 16, device=1 << 20)
    assert e.value.status == og.ERR_ARG
    with pytest.raises(og.OpivError) as e:
        og.Plan(512, 512, np.uint16, 128, 16)
    assert e.value.status == og.ERR_UNSUPPORTED


# ---- multi-pass window offsetting -----------------------------------------------
@pytest.mark.parametrize("mode", [og.CORR_COMPLEX, og.CORR_REAL])
def test_multipass_64_32_16_vs_oracle_chain(orc, mode):
    """Three passes (64, 32, 16 px at 50 % step) of a vortex + offset field on
    a 1024 x 768 12-bit pair: every pass's integer peaks and displacements
    bit-exact, vectors within tolerance, against the oracle's chain."""
    from oracle import oracle as O

    def field(x, y):
        cx, cy, rc, vmax = 512.0, 384.0, 150.0, 8.0
        dx, dy = x - cx, y - cy
        r2 = dx * dx + dy * dy + 1e-9
        vt = vmax * (1.0 + 0.5 / 0.7153) * (rc / np.sqrt(r2)) * (1 - np.exp(-1.2564 * r2 / rc**2))
        s = vt / np.sqrt(r2)
        return -dy * s + 1.3, dx * s - 0.7

    a, b = synth.particle_pair(768, 1024, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                               displacement=field, dtype=np.uint16, seed=synth.SEED_BASE + 3000,
                               full_scale=4095.0)
    passes = [(64, 32), (32, 16), (16, 8)]
    mp = og.MultiPass(1024, 768, np.uint16, passes, mode=mode)
    mp.process(a, b)
    ref = O.multipass(orc, a, b, passes, mode, threads=THREADS)
    for k, (ia, _) in enumerate(passes):
        vec, pk, disp = mp.results(k)
        assert np.array_equal(mp.grid(k), ref[k]["grid"])
        assert_vectors_match(vec, pk, ref[k]["vec"], ref[k]["peak"], ia, f"pass {k}")
        assert np.array_equal(disp, ref[k]["disp"]), f"pass {k}: integer displacements differ"
    mp.close()


@pytest.mark.parametrize("mode", [og.CORR_POCKET, og.CORR_POCKET_REAL])
def test_pocket_modes_are_the_circular_correlation(mode):
    """PocketFFT::cross_correlate and ::cross_correlate_real (c2c and r2c/c2r
    with fct 1.0) both give the true circular correlation: the same results
    as the complex mode, whose planes match numpy's FFT correlation."""
    a, b = synth.config1()
    p1 = og.Plan(1024, 1024, np.uint8, 32, 16, mode=mode)
    p2 = og.Plan(1024, 1024, np.uint8, 32, 16, mode=og.CORR_COMPLEX)
    v1, k1 = p1.process(a, b)
    v2, k2 = p2.process(a, b)
    assert np.array_equal(v1, v2) and np.array_equal(k1, k2)
    rng = np.random.default_rng(8)
    wa = rng.integers(0, 256, (4, 32, 32)).astype(np.float64)
    wb = rng.integers(0, 256, (4, 32, 32)).astype(np.float64)
    got = og.cross_correlate_batch(wa, wb, mode)
    ref = np.fft.fftshift(np.fft.ifft2(np.fft.fft2(wb) * np.conj(np.fft.fft2(wa))).real * 1024,
                          axes=(1, 2))
    for k in range(4):
        assert np.abs(got[k] - ref[k]).max() <= PLANE_RTOL * np.abs(ref[k]).max()


# ---- batches of image pairs -----------------------------------------------------
def test_batch_graph_matches_per_pair_multipass():
    """Pairs of different sizes through the 64/32/16 schedule as one batch:
    eager submission, the first graph call (eager run + capture) and graph
    replays after new frames are uploaded all give exactly the per-pair
    MultiPass results."""
    sizes = [(512, 384), (768, 512), (1024, 1024)]
    passes = [(64, 32), (32, 16), (16, 8)]
    frames = []
    for i, (w, h) in enumerate(sizes):
        for j in range(2):
            frames.append(synth.particle_pair(
                h, w, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                displacement=synth.lamb_oseen(w / 2.0, h / 2.0, offset=(1.1 - i, 0.4 + j)),
                dtype=np.uint16, seed=synth.SEED_BASE + 3900 + 10 * i + j, full_scale=4095.0))
    expect = []
    for i, (w, h) in enumerate(sizes):
        per = []
        for j in range(2):
            mp = og.MultiPass(w, h, np.uint16, passes)
            mp.process(*frames[2 * i + j])
            per.append([mp.results(k) for k in range(len(passes))])
            mp.close()
        expect.append(per)
    batch = og.Batch(sizes, np.uint16, passes)

    def check(j, label):
        for i in range(len(sizes)):
            for k in range(len(passes)):
                got = batch.results(i, k)
                ref = expect[i][j][k]
                for g, r, name in zip(got, ref, ("vectors", "peaks", "displacements")):
                    assert np.array_equal(g, r), f"{label}: pair {i} pass {k} {name} differ"

    for i in range(len(sizes)):
        batch.upload(i, *frames[2 * i])
    batch.run(use_graph=False)
    check(0, "eager")
    before = og.kernel_launch_count()
    batch.run(use_graph=True)             # eager run + capture
    check(0, "first graph call")
    for j in (1, 0, 1):
        for i in range(len(sizes)):
            batch.upload(i, *frames[2 * i + j])
        batch.run(use_graph=True)         # replay
        check(j, f"replay {j}")
    assert og.kernel_launch_count() - before == 4 * 2 * len(sizes) * len(passes)
    assert batch.window_count(2, 2) == 127 * 127
    # the pipelined host call: same final-pass results, frames of both sets,
    # one of them behind a padded row pitch
    for j in (0, 1, 0):
        fr = [frames[2 * i + j] for i in range(len(sizes))]
        if j == 1:
            padded = np.zeros((sizes[0][1], sizes[0][0] + 24), np.uint16)
            pb = padded.copy()
            padded[:, :sizes[0][0]], pb[:, :sizes[0][0]] = fr[0]
            fr[0] = (padded[:, :sizes[0][0]], pb[:, :sizes[0][0]])
        before = og.kernel_launch_count()
        if j == 1:   # non-contiguous views reach the C call with their own pitch
            last = len(passes) - 1
            outs = [(np.zeros((batch.window_count(i, last), 5), np.float32),
                     np.zeros(batch.window_count(i, last), np.int32)) for i in range(len(sizes))]
            batch.process_into([a.ctypes.data for a, _ in fr], [b.ctypes.data for _, b in fr],
                               [a.strides[0] for a, _ in fr], [v.ctypes.data for v, _ in outs],
                               [p.ctypes.data for _, p in outs])
        else:
            outs = batch.process(fr)
        assert og.kernel_launch_count() - before == 2 * len(sizes) * len(passes)
        for i, (vec, pk) in enumerate(outs):
            ref = expect[i][j][len(passes) - 1]
            assert np.array_equal(vec, ref[0]), f"process {j}: pair {i} vectors differ"
            assert np.array_equal(pk, ref[1]), f"process {j}: pair {i} peaks differ"
    with pytest.raises(og.OpivError):
        batch.process(frames[:2])
    batch.close()


# ---- pipelined host call --------------------------------------------------------
@pytest.mark.parametrize("precision", [og.PREC_FP32, og.PREC_TC_SPLIT_BF16])
def test_process_pairs_equals_single_calls(precision):
    """opiv_process_pairs (uploads, passes and downloads of neighbouring
    pairs overlapped) gives exactly what one opiv_process_pair per pair
    gives, in order."""
    pairs = [synth.particle_pair(256, 384, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                                 displacement=lambda x, y, s=s: (np.full_like(x, 0.7 * s), np.full_like(y, -1.1)),
                                 dtype=np.uint16, seed=synth.SEED_BASE + 7000 + s, full_scale=4095.0)
             for s in range(3)]
    plan = og.Plan(384, 256, np.uint16, 32, 8)
    plan.set_precision(precision)
    single = [plan.process(a, b) for a, b in pairs]
    seq = pairs + pairs[::-1]
    got = plan.process_pairs(seq)
    for (v, p), (rv, rp) in zip(got, single + single[::-1]):
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)) and np.array_equal(p, rp)
    assert plan.process_pairs([]) == []
    plan.close()
