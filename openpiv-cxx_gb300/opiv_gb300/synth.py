"""Seeded synthetic PIV image pairs (particle images).

The reference names no public dataset; its workloads are described by
particle statistics, so inputs are generated here:
  * particles at `ppp` per pixel, positions uniform in [-4, W+4) x [-4, H+4)
    (no depletion at the edges);
  * each particle is a Gaussian spot I0 * exp(-8 r^2 / d^2), r measured from
    the pixel centre (x + 0.5, y + 0.5), d ~ N(2.5, 0.5) clipped to [1.5, 4];
  * frame B holds the same particles moved by the displacement field
    evaluated at each particle;
  * N(0, sigma) noise is added, then values are rounded half-to-even and
    clipped to the signal range of the pixel type (float frames are not
    rounded).
RNG: numpy PCG64, seed = 20261203 + 1000 * config + pair index.
"""
from __future__ import annotations

import math

import numpy as np

SEED_BASE = 20261203
STAMP = 6   # stamp half-width in pixels (exp(-8 r^2/d^2) * 4000 < 1e-5 beyond it)


def _render(h: int, w: int, px: np.ndarray, py: np.ndarray, d: np.ndarray, i0: np.ndarray,
            chunk: int = 1 << 16) -> np.ndarray:
    img = np.zeros(h * w, np.float64)
    offs = np.arange(-STAMP, STAMP + 1)
    for s in range(0, px.size, chunk):
        cx, cy = px[s:s + chunk], py[s:s + chunk]
        dd, ii = d[s:s + chunk], i0[s:s + chunk]
        ix = np.floor(cx).astype(np.int64)[:, None] + offs[None, :]     # (n, k)
        iy = np.floor(cy).astype(np.int64)[:, None] + offs[None, :]
        gx = np.exp(-8.0 * ((ix + 0.5) - cx[:, None]) ** 2 / (dd[:, None] ** 2))
        gy = np.exp(-8.0 * ((iy + 0.5) - cy[:, None]) ** 2 / (dd[:, None] ** 2))
        val = ii[:, None, None] * gy[:, :, None] * gx[:, None, :]       # (n, ky, kx)
        yy = np.broadcast_to(iy[:, :, None], val.shape)
        xx = np.broadcast_to(ix[:, None, :], val.shape)
        m = (xx >= 0) & (xx < w) & (yy >= 0) & (yy < h)
        img += np.bincount((yy[m] * w + xx[m]).ravel(), weights=val[m].ravel(), minlength=h * w)
    return img.reshape(h, w)


def particle_pair(h: int, w: int, *, ppp: float, i0_range: tuple[float, float], noise: float,
                  displacement, dtype, seed: int, full_scale: float | None = None,
                  d_mean: float = 2.5, d_std: float = 0.5):
    """Returns (frame_a, frame_b) of shape (h, w) and pixel type `dtype`.

    displacement(x, y) -> (u, v) in pixels, x to the right, y down (rows).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(round(ppp * w * h))
    x = rng.uniform(-4.0, w + 4.0, n)
    y = rng.uniform(-4.0, h + 4.0, n)
    d = np.clip(rng.normal(d_mean, d_std, n), 1.5, 4.0)
    i0 = rng.uniform(i0_range[0], i0_range[1], n)
    u, v = displacement(x, y)
    a = _render(h, w, x, y, d, i0)
    b = _render(h, w, x + u, y + v, d, i0)
    a += rng.normal(0.0, noise, a.shape)
    b += rng.normal(0.0, noise, b.shape)
    dt = np.dtype(dtype)
    if dt.kind == "u":
        hi = full_scale if full_scale is not None else float(np.iinfo(dt).max)
        a = np.clip(np.rint(a), 0, hi).astype(dt)
        b = np.clip(np.rint(b), 0, hi).astype(dt)
    else:
        lo, hi = (0.0, full_scale) if full_scale is not None else (-np.inf, np.inf)
        a = np.clip(a, lo, hi).astype(dt)
        b = np.clip(b, lo, hi).astype(dt)
    return a, b


# ---- the workloads -----------------------------------------------------------
def config1(pair: int = 0):
    """1024^2 uint8, ppp 0.02, I0 ~ U(150, 255), sigma 3, uniform (2.35, -1.70) px.
    Windows 32 x 32 at step fraction 0.5 (3969 windows)."""
    return particle_pair(1024, 1024, ppp=0.02, i0_range=(150, 255), noise=3.0,
                         displacement=lambda x, y: (np.full_like(x, 2.35), np.full_like(y, -1.70)),
                         dtype=np.uint8, seed=SEED_BASE + 1000 * 1 + pair)


def config2_field(x, y):
    return 3.0 * np.sin(2 * math.pi * y / 1024.0), 2.0 * np.cos(2 * math.pi * x / 768.0)


def config2(pair: int = 0, size: int = 4096):
    """4096^2 uint16 (12-bit signal), ppp 0.03, I0 ~ U(1500, 4000), sigma 20,
    u = 3 sin(2 pi y / 1024), v = 2 cos(2 pi x / 768).  Windows 32 x 32 at
    step 8 (509 x 509 = 259,081 windows)."""
    return particle_pair(size, size, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                         displacement=config2_field, dtype=np.uint16,
                         seed=SEED_BASE + 1000 * 2 + pair, full_scale=4095.0)


CONFIG3_SIZES = ((1024, 1024), (2048, 1536), (3072, 2048), (4096, 4096))   # (width, height)
LAMB_OSEEN_ALPHA = 1.25643   # r = rc is the radius of maximum swirl velocity


def lamb_oseen(cx: float, cy: float, rc: float = 150.0, vmax: float = 8.0,
               offset: tuple[float, float] = (0.0, 0.0)):
    """Lamb-Oseen vortex centred at (cx, cy): swirl velocity
    v(r) = vmax (1 + 1/(2 alpha)) (rc / r) (1 - exp(-alpha r^2 / rc^2)), which
    peaks at vmax for r = rc, plus a uniform offset."""
    k = vmax * (1.0 + 0.5 / LAMB_OSEEN_ALPHA) * rc

    def field(x, y):
        dx, dy = x - cx, y - cy
        r2 = dx * dx + dy * dy + 1e-12
        s = k * (1.0 - np.exp(-LAMB_OSEEN_ALPHA * r2 / (rc * rc))) / r2
        return -dy * s + offset[0], dx * s + offset[1]
    return field


def config3_layout(n_pairs: int = 48):
    """Per pair: (width, height) drawn from CONFIG3_SIZES and the uniform
    offset U(-2, 2)^2 px, by the config-3 seed."""
    rng = np.random.Generator(np.random.PCG64(SEED_BASE + 1000 * 3))
    idx = rng.integers(0, len(CONFIG3_SIZES), n_pairs)
    off = rng.uniform(-2.0, 2.0, (n_pairs, 2))
    return [(CONFIG3_SIZES[i], (float(o[0]), float(o[1]))) for i, o in zip(idx, off)]


def config3(pair: int, size: tuple[int, int], offset: tuple[float, float]):
    """One pair of the batched multi-pass workload: uint16 (12-bit signal) with
    config-2 particle statistics, Lamb-Oseen vortex (core radius 150 px, peak
    8 px) at the image centre plus the pair's uniform offset."""
    w, h = size
    return particle_pair(h, w, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                         displacement=lamb_oseen(w / 2.0, h / 2.0, offset=offset),
                         dtype=np.uint16, seed=SEED_BASE + 1000 * 3 + 1 + pair, full_scale=4095.0)


def config4(variant: str = "base", size: int = 4096):
    """The config-2 field for the precision sweep: "base" (config-2
    statistics), "sparse" (0.005 ppp) or "noisy" (sigma 80)."""
    ppp = 0.005 if variant == "sparse" else 0.03
    noise = 80.0 if variant == "noisy" else 20.0
    k = {"base": 0, "sparse": 1, "noisy": 2}[variant]
    return particle_pair(size, size, ppp=ppp, i0_range=(1500, 4000), noise=noise,
                         displacement=config2_field, dtype=np.uint16,
                         seed=SEED_BASE + 1000 * 4 + k, full_scale=4095.0)


def config5(pair: int = 0, size: int = 2048, noise: float = 0.02):
    """2048^2 float32 in [0, 1], ppp 0.02, I0 ~ U(0.6, 1), sigma 0.02, shift
    (0.40, 0.25).  noise = 0 gives the clean pair (Monte Carlo adds its own)."""
    return particle_pair(size, size, ppp=0.02, i0_range=(0.6, 1.0), noise=noise,
                         displacement=lambda x, y: (np.full_like(x, 0.40), np.full_like(y, 0.25)),
                         dtype=np.float32, seed=SEED_BASE + 1000 * 5 + pair, full_scale=1.0)
