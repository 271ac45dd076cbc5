"""Adjoint d(u, v)/d(pixels): against an FP64 analytic gradient, FP64
central finite differences through the oracle, and Monte Carlo over pixel
noise (the config-5 float32 pair: 0.02 ppp, shift (0.40, 0.25))."""
import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth

pytestmark = pytest.mark.gpu
W = 32


def _torch():
    return pytest.importorskip("torch")


def forward(a, b, step, mode=og.CORR_COMPLEX):
    """Vectors and peak codes of the exact-parity path, device copies kept."""
    torch = _torch()
    h, w = a.shape
    plan = og.Plan(w, h, a.dtype, W, step, mode=mode)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    vec = torch.empty((plan.n, 5), dtype=torch.float32, device="cuda")
    pk = torch.empty(plan.n, dtype=torch.int32, device="cuda")
    plan.process_device(da.data_ptr(), db.data_ptr(), a.strides[0], vec.data_ptr(), pk.data_ptr(), 0)
    torch.cuda.synchronize()
    return plan, da, db, vec, pk


def reference_gradients(wa, wb, code):
    """FP64 du/da, du/db, dv/da, dv/db of one window (u = W/2 - px - fx)."""
    px, py = code % W, code // W
    lags = [(px - 16, py - 16), (px - 17, py - 16), (px - 15, py - 16), (px - 16, py - 17), (px - 16, py - 15)]
    R = [np.sum(wa * np.roll(wb, (-dy, -dx), axis=(0, 1))) for dx, dy in lags]
    c, l, r, u, d = R

    def partials(lo, hi):
        N = np.log(lo) - np.log(hi)
        D = 2 * (np.log(lo) + np.log(hi) - 2 * np.log(c))
        return -(D - 2 * N) / (lo * D * D), (D + 2 * N) / (hi * D * D), -4 * N / (c * D * D)

    gl, gr, gc = partials(l, r)
    gu, gd, gc2 = partials(u, d)
    gx = [gc, gl, gr, 0.0, 0.0]
    gy = [gc2, 0.0, 0.0, gu, gd]
    out = []
    for g in (gx, gy):
        da = sum(gv * np.roll(wb, (-dy, -dx), axis=(0, 1)) for gv, (dx, dy) in zip(g, lags))
        db = sum(gv * np.roll(wa, (dy, dx), axis=(0, 1)) for gv, (dx, dy) in zip(g, lags))
        out += [da, db]
    return out   # du/da, du/db, dv/da, dv/db


def sampled_windows(plan, stride):
    """Windows every `stride` grid steps in x and y: no two share a pixel."""
    grid = plan.grid()
    nx = len(np.unique(grid[:, 0]))
    idx = np.arange(len(grid)).reshape(-1, nx)[::stride, ::stride].ravel()
    return grid, idx


def piv_function(plan):
    """A test-only torch.autograd.Function: (frame a, frame b) -> (n, 2)
    displacements (u, v); backward through opiv_plan_adjoint."""
    torch = _torch()

    class PivVectors(torch.autograd.Function):
        @staticmethod
        def forward(ctx, a, b):
            a, b = a.contiguous(), b.contiguous()
            vec = torch.empty((plan.n, 5), dtype=torch.float32, device=a.device)
            pk = torch.empty(plan.n, dtype=torch.int32, device=a.device)
            plan.process_device(a.data_ptr(), b.data_ptr(), a.stride(0) * a.element_size(), vec.data_ptr(),
                                pk.data_ptr(), 0)
            ctx.save_for_backward(a, b, pk)
            return vec[:, 2:4].clone()

        @staticmethod
        def backward(ctx, grad_uv):
            a, b, pk = ctx.saved_tensors
            cot = grad_uv.contiguous().float()
            ga = torch.zeros_like(a)
            gb = torch.zeros_like(b)
            plan.adjoint_device(a.data_ptr(), b.data_ptr(), a.stride(0) * a.element_size(), pk.data_ptr(),
                                cot.data_ptr(), ga.data_ptr(), gb.data_ptr(), a.stride(0) * 4)
            return ga, gb

    return PivVectors.apply


def test_autograd_function_against_fp64_gradient():
    torch = _torch()
    a, b = synth.config5(size=512)
    plan, da, db, vec, pk = forward(a, b, 8)
    pk = pk.cpu().numpy()
    grid, idx = sampled_windows(plan, 4)
    idx = idx[pk[idx] >= 0]
    f = piv_function(plan)
    worst = 0.0
    for comp in (0, 1):                      # loss = sum of u (then v) over the sampled windows
        ta = torch.from_numpy(a).cuda().requires_grad_(True)
        tb = torch.from_numpy(b).cuda().requires_grad_(True)
        uv = f(ta, tb)
        sel = torch.zeros_like(uv)
        sel[torch.from_numpy(idx).cuda(), comp] = 1.0
        (uv * sel).sum().backward()
        ga, gb = ta.grad.cpu().numpy(), tb.grad.cpu().numpy()
        for w in idx:
            x, y = grid[w]
            ref = reference_gradients(a[y:y + W, x:x + W].astype(np.float64),
                                      b[y:y + W, x:x + W].astype(np.float64), int(pk[w]) & 0xFFFF)
            for got, want in ((ga[y:y + W, x:x + W], ref[2 * comp]), (gb[y:y + W, x:x + W], ref[2 * comp + 1])):
                scale = np.abs(want).max()
                if np.isfinite(scale) and scale > 0:
                    worst = max(worst, np.abs(got - want).max() / scale)
    assert worst < 2e-3, f"adjoint differs from the FP64 gradient by {worst:.2e} of its largest entry"


def test_adjoint_against_central_differences():
    """FP64 central differences (h = 1e-3) through the oracle on sampled
    windows, at the pixels with the largest adjoint entries."""
    from oracle import oracle as O
    orc = O.get("port")
    a, b = synth.config5(size=512)
    plan, da, db, vec, pk = forward(a, b, 8)
    pkn = pk.cpu().numpy()
    grid, idx = sampled_windows(plan, 4)
    idx = idx[pkn[idx] >= 0][:64]
    torch = _torch()
    ta = torch.from_numpy(a).cuda().requires_grad_(True)
    tb = torch.from_numpy(b).cuda()
    uv = piv_function(plan)(ta, tb)
    sel = torch.zeros_like(uv)
    sel[torch.from_numpy(idx).cuda(), 0] = 1.0
    (uv * sel).sum().backward()
    ga = ta.grad.cpu().numpy()
    h = 1e-3
    errs = []
    for w in idx:
        x, y = grid[w]
        wa = a[y:y + W, x:x + W].astype(np.float64)
        wb = b[y:y + W, x:x + W].astype(np.float64)
        u0 = orc.process_windows(wa, wb, np.array([[0, 0]], np.int32), W, og.CORR_COMPLEX)[0]
        if not np.isfinite(u0[0, 2]):
            continue
        g = ga[y:y + W, x:x + W]
        for flat in np.argsort(-np.abs(g).ravel())[:4]:
            py, px = divmod(int(flat), W)
            us = []
            for sgn in (1, -1):
                wp = wa.copy()
                wp[py, px] += sgn * h
                us.append(orc.process_windows(wp, wb, np.array([[0, 0]], np.int32), W, og.CORR_COMPLEX)[0][0, 2])
            fd = (us[0] - us[1]) / (2 * h)
            errs.append(abs(fd - g[py, px]) / max(abs(fd), 1e-3))
    assert len(errs) > 100
    assert np.median(errs) < 1e-3 and np.max(errs) < 2e-2, (np.median(errs), np.max(errs))


def test_propagated_sigma_against_monte_carlo():
    """Per-vector sigma_u, sigma_v from the adjoint (pixel noise sigma 0.02
    on both frames) against the spread of u, v over 200 noise seeds."""
    torch = _torch()
    a0, b0 = synth.config5(size=512, noise=0.0)
    sig = 0.02
    plan, da, db, vec, pk = forward(a0, b0, 16)
    dsig = torch.zeros((plan.n, 2), dtype=torch.float32, device="cuda")
    plan.adjoint_device(da.data_ptr(), db.data_ptr(), a0.strides[0], pk.data_ptr(), var_a=sig * sig,
                        var_b=sig * sig, d_sigma=dsig.data_ptr())
    torch.cuda.synchronize()
    pred = dsig.cpu().numpy()
    pk0 = pk.cpu().numpy()
    g = torch.Generator(device="cuda").manual_seed(20261203)
    us, same = [], np.ones(plan.n, bool)
    dvec = torch.empty_like(vec)
    dpk = torch.empty_like(pk)
    for _ in range(200):
        na = (da + sig * torch.randn(da.shape, generator=g, device="cuda")).contiguous()
        nb = (db + sig * torch.randn(db.shape, generator=g, device="cuda")).contiguous()
        plan.process_device(na.data_ptr(), nb.data_ptr(), a0.strides[0], dvec.data_ptr(), dpk.data_ptr(), 0)
        us.append(dvec[:, 2:4].cpu().numpy())
        same &= dpk.cpu().numpy() == pk0
    us = np.stack(us)
    mc = us.std(axis=0, ddof=1)
    ok = same & (pk0 >= 0) & np.isfinite(pred).all(1) & np.isfinite(mc).all(1) & (pred > 0).all(1)
    assert ok.sum() > 100
    ratio = mc[ok] / pred[ok]
    med = np.median(ratio, axis=0)
    assert np.all(np.abs(med - 1.0) < 0.1), f"median MC / propagated sigma = {med}"


# ---- REAL mode (FFT::cross_correlate_real) ------------------------------------
def project(win):
    """FP64 window with spectrum column k_x = 0 and rows k_y = 0, H/2 removed:
    what the reference's partial unpack leaves of it (fft.h:163-183)."""
    f = np.fft.fft2(win)
    f[:, 0] = 0
    f[0, :] = 0
    f[W // 2, :] = 0
    return np.fft.ifft2(f).real


def test_real_mode_adjoint_against_fp64_gradient():
    torch = _torch()
    a, b = synth.config5(size=512)
    plan, da, db, vec, pk = forward(a, b, 8, og.CORR_REAL)
    pkn, vecn = pk.cpu().numpy(), vec.cpu().numpy()
    grid, idx = sampled_windows(plan, 4)
    f = piv_function(plan)
    worst, n = 0.0, 0
    for comp in (0, 1):
        sel_w = [w for w in idx if pkn[w] >= 0 and np.isfinite(vecn[w, 2 + comp])]
        ta = torch.from_numpy(a).cuda().requires_grad_(True)
        tb = torch.from_numpy(b).cuda().requires_grad_(True)
        uv = f(ta, tb)
        sel = torch.zeros_like(uv)
        sel[torch.tensor(sel_w, device="cuda"), comp] = 1.0
        (uv.nan_to_num() * sel).sum().backward()
        ga, gb = ta.grad.cpu().numpy(), tb.grad.cpu().numpy()
        for w in sel_w:
            x, y = grid[w]
            ref = reference_gradients(project(a[y:y + W, x:x + W].astype(np.float64)),
                                      project(b[y:y + W, x:x + W].astype(np.float64)), int(pkn[w]) & 0xFFFF)
            for got, want in ((ga[y:y + W, x:x + W], ref[2 * comp]), (gb[y:y + W, x:x + W], ref[2 * comp + 1])):
                scale = np.abs(want).max()
                if np.isfinite(scale) and scale > 0:
                    worst = max(worst, np.abs(got - want).max() / scale)
                    n += 1
    assert n > 50
    assert worst < 5e-3, f"REAL-mode adjoint differs from the FP64 gradient by {worst:.2e} of its largest entry"


def test_real_mode_adjoint_against_central_differences():
    """FP64 central differences (h = 1e-3) through the oracle's REAL-mode
    chain (the reference's cross_correlate_real, peaks, fit)."""
    from oracle import oracle as O
    orc = O.get("port")
    a, b = synth.config5(size=512)
    plan, da, db, vec, pk = forward(a, b, 8, og.CORR_REAL)
    pkn, vecn = pk.cpu().numpy(), vec.cpu().numpy()
    grid, idx = sampled_windows(plan, 4)
    idx = [w for w in idx if pkn[w] >= 0 and np.isfinite(vecn[w, 2])][:64]
    torch = _torch()
    ta = torch.from_numpy(a).cuda().requires_grad_(True)
    tb = torch.from_numpy(b).cuda()
    uv = piv_function(plan)(ta, tb)
    sel = torch.zeros_like(uv)
    sel[torch.tensor(idx, device="cuda"), 0] = 1.0
    (uv.nan_to_num() * sel).sum().backward()
    ga = ta.grad.cpu().numpy()
    h = 1e-3
    errs = []
    for w in idx:
        x, y = grid[w]
        wa = a[y:y + W, x:x + W].astype(np.float64)
        wb = b[y:y + W, x:x + W].astype(np.float64)
        one = np.array([[0, 0]], np.int32)
        u0 = orc.process_windows(wa, wb, one, W, og.CORR_REAL)[0]
        if not np.isfinite(u0[0, 2]):
            continue
        g = ga[y:y + W, x:x + W]
        for flat in np.argsort(-np.abs(g).ravel())[:4]:
            py, px = divmod(int(flat), W)
            us = []
            for sgn in (1, -1):
                wp = wa.copy()
                wp[py, px] += sgn * h
                us.append(orc.process_windows(wp, wb, one, W, og.CORR_REAL)[0][0, 2])
            fd = (us[0] - us[1]) / (2 * h)
            errs.append(abs(fd - g[py, px]) / max(abs(fd), 1e-3))
    assert len(errs) > 40
    assert np.median(errs) < 1e-3 and np.max(errs) < 5e-2, (np.median(errs), np.max(errs))
