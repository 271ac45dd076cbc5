"""Pins the oracle (CPU restatement, oracle/opiv_oracle.cpp) before it is
trusted as the checker: against the reference tests' own known answers,
against committed outputs of the compiled reference, and -- where the
reference sources are on this machine -- against the compiled reference
live, bit for bit."""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as f:
        return json.load(f)


def ref_outputs():
    return np.load(os.path.join(GOLDEN, "ref_outputs.npz"))


# ---- the reference tests' known answers -------------------------------------
@pytest.mark.parametrize("case", kats()["grid"], ids=lambda c: c["cite"])
def test_grid_kats(orc, case):
    (iw, ih), (aw, ah) = case["image"], case["ia"]
    if "frac" in case:
        g = orc.grid(iw, ih, aw, ah, case["frac"])
    else:
        g = orc.grid_offsets(iw, ih, aw, ah, *case["offsets"])
    assert sorted(map(tuple, g.tolist())) == sorted(map(tuple, case["origins"]))


def test_grid_errors(orc):
    assert orc.grid(100, 100, 32, 32, 1.5) == -1
    assert orc.grid(100, 100, 32, 32, -0.1) == -1
    assert orc.grid(0, 100, 32, 32, 0.5) == -2
    assert orc.grid(100, 100, 0, 32, 0.5) == -3
    assert orc.grid(100, 100, 32, 32, 0.0) == -4          # step truncates to 0
    assert orc.grid(16, 100, 32, 32, 0.5) == -5


@pytest.mark.parametrize("case", kats()["peaks"], ids=lambda c: c["cite"])
def test_find_peaks_kats(orc, case):
    im = np.zeros(case["size"][::-1])
    for x, y, v in case["spikes"]:
        im[y, x] = v
    xy, v = orc.find_peaks(im, case["num"], 1)
    assert xy.tolist() == case["centres"]
    assert v.tolist() == case["values"]


def test_swap_quadrants_kat(orc):
    k = kats()["swap_quadrants"]
    w, h = k["size"]
    im = np.zeros((h, w))
    xs, ys = np.meshgrid(np.arange(w), np.arange(h))
    im[:] = np.where(xs < w // 2, 1, 2) * np.where(ys < h // 2, 1, 4)
    out = orc.swap_quadrants(im)
    q = [out[:h // 2, :w // 2], out[:h // 2, w // 2:], out[h // 2:, :w // 2], out[h // 2:, w // 2:]]
    assert [float(x.mean()) for x in q] == k["after"]


def _sinusoid(n, mirror=False):
    w, h = np.meshgrid(np.arange(n), np.arange(n))
    ww = (n - w) if mirror else w
    return 128 * np.sin(2 * math.pi * ww / 8 + 2 * math.pi * h / 8)


def test_fft_kat(orc):
    k = kats()["fft"]
    n = k["size"]
    X = orc.transform(_sinusoid(n).astype(np.complex128), -1)
    mask = np.zeros((n, n), bool)
    for x, y in k["spikes"]:
        mask[y, x] = True
    assert np.all(np.abs(X[mask]) > 0)
    assert np.all(np.abs(X[~mask]) ** 2 < k["tol_abs_sqr"])


def test_fft_real_kat(orc):
    k = kats()["fft"]
    n = k["size"]
    A, B = orc.transform_real(_sinusoid(n), _sinusoid(n, mirror=True))
    for im, spikes in ((A, k["spikes_a"]), (B, k["spikes_b"])):
        mask = np.zeros((n, n), bool)
        for x, y in spikes:
            mask[y, x] = True
        assert np.all(np.abs(im[mask]) > 0)
        assert np.all(np.abs(im[~mask]) ** 2 < k["tol_abs_sqr"])


def test_fft_errors(orc):
    with pytest.raises(RuntimeError):
        orc.transform(np.zeros((400, 512), np.complex128))
    with pytest.raises(RuntimeError):
        orc.transform(np.zeros((512, 400), np.complex128))


def test_inverse_roundtrip(orc):
    rng = np.random.default_rng(3)
    z = rng.normal(size=(32, 64)) + 1j * rng.normal(size=(32, 64))
    back = orc.transform(orc.transform(z, -1), +1) / z.size
    np.testing.assert_allclose(back, z, atol=1e-12)
    np.testing.assert_allclose(orc.transform(z, -1), np.fft.fft2(z), atol=1e-9)


# ---- committed outputs of the compiled reference ---------------------------
def _fixtures():
    z = ref_outputs()
    return sorted({k.split("/")[0] for k in z.files})


@pytest.mark.parametrize("name", _fixtures())
def test_port_matches_reference_fixtures(orc, name):
    z = ref_outputs()
    a, b, grid = z[f"{name}/a"], z[f"{name}/b"], z[f"{name}/grid"]
    ia, step = (int(v) for v in z[f"{name}/meta"])
    h, w = a.shape
    assert np.array_equal(orc.grid_offsets(w, h, ia, ia, step, step), grid)
    sel = z[f"{name}/planes_sel"]
    fa, fb = a.astype(np.float64), b.astype(np.float64)
    for mode, mname in ((0, "real"), (1, "complex")):
        planes = orc.correlate_windows(fa, fb, grid[sel], ia, mode)
        assert np.array_equal(planes, z[f"{name}/planes_{mname}"])
        for limit in (0, 1):
            vec, pk, _ = orc.process_windows(fa, fb, grid, ia, mode, limit, 2)
            assert np.array_equal(pk, z[f"{name}/peak_{mname}_{limit}"])
            assert np.array_equal(vec, z[f"{name}/vec_{mname}_{limit}"], equal_nan=True)


# ---- live comparison with the compiled reference -----------------------------
@pytest.mark.parametrize("w", [4, 8, 16, 32, 64])
@pytest.mark.parametrize("mode", [0, 1])
def test_port_bit_exact_vs_reference(orc, ref_lib, w, mode):
    rng = np.random.default_rng(w * 10 + mode)
    for _ in range(3):
        a = rng.integers(0, 4096, (w, w)).astype(np.float64)
        b = rng.integers(0, 4096, (w, w)).astype(np.float64)
        assert np.array_equal(orc.cross_correlate(a, b, mode), ref_lib.cross_correlate(a, b, mode))


def test_port_process_vs_reference(orc, ref_lib):
    rng = np.random.default_rng(11)
    a = rng.integers(0, 256, (200, 264)).astype(np.float64)
    b = np.roll(a, (2, -3), (0, 1)) + rng.normal(0, 4, a.shape)
    grid = orc.grid(264, 200, 32, 32, 0.25)
    assert np.array_equal(grid, ref_lib.grid(264, 200, 32, 32, 0.25))
    for mode in (0, 1):
        for limit in (0, 1):
            v1, p1, _ = orc.process_windows(a, b, grid, 32, mode, limit, 1)
            v2, p2, _ = ref_lib.process_windows(a, b, grid, 32, mode, limit, 3)
            assert np.array_equal(p1, p2)
            assert np.array_equal(v1, v2, equal_nan=True)


def test_port_transform_real_vs_reference(orc, ref_lib):
    rng = np.random.default_rng(5)
    a, b = rng.normal(size=(2, 32, 32))
    A1, B1 = orc.transform_real(a, b)
    A2, B2 = ref_lib.transform_real(a, b)
    assert np.array_equal(A1, A2) and np.array_equal(B1, B2)
    z = a + 1j * b
    assert np.array_equal(orc.transform(z, -1), ref_lib.transform(z, -1))
    assert np.array_equal(orc.transform(z, +1), ref_lib.transform(z, +1))


def test_reference_rejects_non_square(ref_lib):
    """The reference's FFT::transform / transform_real resize their scratch
    to the input size instead of its transpose (fft.h:102, :145), so the
    transpose check (image_utils.impl.h:330-333) throws for non-square
    images: only square windows are usable through its FFT class."""
    rng = np.random.default_rng(5)
    a, b = rng.normal(size=(2, 16, 32))
    with pytest.raises(RuntimeError):
        ref_lib.transform_real(a, b)
    with pytest.raises(RuntimeError):
        ref_lib.transform(a + 0j, -1)


def test_multipass_chain_vs_reference(orc, ref_lib):
    """The window-offsetting chain (composed from reference calls) gives the
    same result through the restatement and through the compiled reference."""
    from oracle import oracle as O
    rng = np.random.default_rng(12)
    a = rng.integers(0, 4096, (192, 256)).astype(np.float64)
    b = np.roll(a, (-6, 9), (0, 1)) + rng.normal(0, 10, a.shape)
    for mode in (0, 1):
        r1 = O.multipass(orc, a, b, [(64, 32), (32, 16), (16, 8)], mode)
        r2 = O.multipass(ref_lib, a, b, [(64, 32), (32, 16), (16, 8)], mode, threads=2)
        for p1, p2 in zip(r1, r2):
            assert np.array_equal(p1["disp"], p2["disp"])
            assert np.array_equal(p1["peak"], p2["peak"])
            assert np.array_equal(p1["vec"], p2["vec"], equal_nan=True)
        ok = r1[-1]["peak"][:, 0] >= 0
        hit = np.all(r1[-1]["disp"][ok] == [9, -6], axis=1)
        assert hit.mean() > 0.9   # the shift, recovered at 16 px (edges wrap around)


def test_nearest_index_rule():
    from oracle import oracle as O
    c0, step, n = 16, 16, 5          # centres 16, 32, 48, 64, 80
    c = np.arange(0, 100)
    centres = c0 + step * np.arange(n)
    brute = np.array([np.argmin(np.abs(centres - x) + 1e-9 * np.arange(n)[::-1] * 0) for x in c])
    got = O.nearest_index(c, c0, step, n)
    # equidistant points (x = 24, 40, ...) go to the upper line: floor((d + 8) / 16)
    ties = (c - c0) % step == step // 2
    assert np.array_equal(got[~ties], brute[~ties])
    assert np.all(got[ties & (c < 80)] == ((c[ties & (c < 80)] - c0) // step) + 1)
