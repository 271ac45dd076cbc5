"""The identity the REAL-mode adjoint rests on, checked on the CPU: the
reference's cross_correlate_real plane (fft.h:208-227, with the partial
unpack of fft.h:163-183) is the circular correlation of the two windows
with spectrum column k_x = 0 and rows k_y = 0, H/2 removed, and that
projection is, in space, each row's mean and then each column's mean and
(-1)^y-weighted mean taken out (what csrc/piv_adjoint.cu computes)."""
import numpy as np

import opiv_gb300 as og

W = 32


def project(win):
    f = np.fft.fft2(win)
    f[:, 0] = 0
    f[0, :] = 0
    f[W // 2, :] = 0
    return np.fft.ifft2(f).real


def project_spatial(x):
    x = x - x.mean(1, keepdims=True)
    alt = ((-1.0) ** np.arange(W))[:, None]
    return x - x.mean(0)[None, :] - alt * (x * alt).mean(0)[None, :]


def test_real_mode_plane_is_the_projected_correlation(orc):
    """The REAL-mode plane equals the circular correlation of the projected
    windows (the identity the REAL-mode adjoint rests on), against the
    oracle's cross_correlate_real."""
    rng = np.random.default_rng(5)
    for _ in range(4):
        wa = rng.random((W, W))
        wb = np.roll(wa, (2, -3), (0, 1)) + 0.1 * rng.random((W, W))
        ac, bc = project(wa), project(wb)
        plane = np.array([[np.sum(ac * np.roll(bc, (-(y - 16), -(x - 16)), axis=(0, 1)))
                           for x in range(W)] for y in range(W)]) * (W * W)
        ref = orc.cross_correlate(wa, wb, og.CORR_REAL)
        assert np.abs(plane - ref).max() <= 1e-9 * np.abs(ref).max()




def test_spatial_projection_equals_spectral():
    rng = np.random.default_rng(6)
    for _ in range(4):
        x = rng.random((W, W)) * 4095
        assert np.abs(project_spatial(x) - project(x)).max() <= 1e-9 * np.abs(x).max()
