"""ctypes front-end of the oracle -- TEST INFRASTRUCTURE ONLY.

Loads either the CPU restatement (``_build/liboracle*.so``, built from
``opiv_oracle.cpp``) or the reference compiled from its own sources
(``_ref/libopiv_ref*.so``, built from ``ref_harness.cpp``).  Both export the
same ``orc_*`` C functions, so every test can run against either.

Only tests, the smoke check and the CPU-baseline leg of ``bench.py`` import
this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

MODE_REAL = 0      # FFT::cross_correlate_real (reference spectrum unpack)
MODE_COMPLEX = 1   # FFT::cross_correlate (true circular correlation)

_LIBS = {
    ("port", False): os.path.join(HERE, "_build", "liboracle.so"),
    ("port", True): os.path.join(HERE, "_build", "liboracle_fast.so"),
    ("ref", False): os.path.join(HERE, "_ref", "libopiv_ref.so"),
    ("ref", True): os.path.join(HERE, "_ref", "libopiv_ref_fast.so"),
}
_cache: dict = {}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def build(ref: bool = False) -> None:
    """Compile the restatement (and, when ``ref``, the reference itself)."""
    targets = ["port"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def available(kind: str = "port", fast: bool = False) -> bool:
    return os.path.exists(_LIBS[(kind, fast)])


class Oracle:
    """One loaded oracle library (``kind`` = "port" or "ref")."""

    def __init__(self, kind: str = "port", fast: bool = False):
        path = _LIBS[(kind, fast)]
        if not os.path.exists(path):
            if kind == "port":
                build(ref=False)
            else:
                raise FileNotFoundError(path)
        self.kind = kind
        self.lib = L = C.CDLL(path)
        L.orc_grid.restype = C.c_int64
        L.orc_grid.argtypes = [C.c_uint32] * 4 + [C.c_double, _ip, C.c_int64]
        L.orc_grid_offsets.restype = C.c_int64
        L.orc_grid_offsets.argtypes = [C.c_uint32] * 6 + [_ip, C.c_int64]
        L.orc_transform.argtypes = [_dp, C.c_uint32, C.c_uint32, C.c_int]
        L.orc_transform_real.argtypes = [_dp, _dp, C.c_uint32, C.c_uint32, _dp, _dp]
        L.orc_cross_correlate.argtypes = [_dp, _dp, C.c_uint32, C.c_uint32, C.c_int, _dp]
        L.orc_swap_quadrants.argtypes = [_dp, C.c_uint32, C.c_uint32]
        L.orc_find_peaks.argtypes = [_dp, C.c_uint32, C.c_uint32, C.c_uint16, C.c_uint32, _ip, _dp]
        L.orc_fit_simple_gaussian.argtypes = [_dp, C.c_uint32, C.c_int32, C.c_int32, _dp]
        L.orc_correlate_windows.argtypes = [_dp, _dp, C.c_uint32, C.c_uint32, _ip, C.c_int64,
                                            C.c_uint32, C.c_int, _dp]
        L.orc_process_windows_ab.restype = C.c_double
        L.orc_process_windows_ab.argtypes = [_dp, _dp, C.c_uint32, C.c_uint32, _ip, _ip, C.c_int64,
                                             C.c_uint32, C.c_int, C.c_int, C.c_int, _dp, _ip]
        L.orc_process_windows.restype = C.c_double
        L.orc_process_windows.argtypes = [_dp, _dp, C.c_uint32, C.c_uint32, _ip, C.c_int64,
                                          C.c_uint32, C.c_int, C.c_int, C.c_int, _dp, _ip]

    # -- grid ---------------------------------------------------------------
    def grid(self, img_w, img_h, ia_w, ia_h, frac):
        n = self.lib.orc_grid(img_w, img_h, ia_w, ia_h, frac, None, 0)
        if n < 0:
            return int(n)
        out = np.zeros((n, 2), np.int32)
        self.lib.orc_grid(img_w, img_h, ia_w, ia_h, frac, out.ctypes.data_as(_ip), n)
        return out

    def grid_offsets(self, img_w, img_h, ia_w, ia_h, dx, dy):
        n = self.lib.orc_grid_offsets(img_w, img_h, ia_w, ia_h, dx, dy, None, 0)
        if n < 0:
            return int(n)
        out = np.zeros((n, 2), np.int32)
        self.lib.orc_grid_offsets(img_w, img_h, ia_w, ia_h, dx, dy, out.ctypes.data_as(_ip), n)
        return out

    # -- FFT ------------------------------------------------------------------
    def transform(self, z: np.ndarray, direction: int = -1) -> np.ndarray:
        h, w = z.shape
        buf = np.ascontiguousarray(z, np.complex128).copy()
        rc = self.lib.orc_transform(buf.ctypes.data_as(_dp), w, h, direction)
        if rc != 0:
            raise RuntimeError(f"orc_transform: {rc}")
        return buf

    def transform_real(self, a: np.ndarray, b: np.ndarray):
        h, w = a.shape
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        oa = np.zeros((h, w), np.complex128)
        ob = np.zeros((h, w), np.complex128)
        rc = self.lib.orc_transform_real(a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), w, h,
                                         oa.ctypes.data_as(_dp), ob.ctypes.data_as(_dp))
        if rc != 0:
            raise RuntimeError(f"orc_transform_real: {rc}")
        return oa, ob

    def cross_correlate(self, a: np.ndarray, b: np.ndarray, mode: int) -> np.ndarray:
        h, w = a.shape
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        out = np.zeros((h, w), np.float64)
        rc = self.lib.orc_cross_correlate(a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), w, h,
                                          mode, out.ctypes.data_as(_dp))
        if rc != 0:
            raise RuntimeError(f"orc_cross_correlate: {rc}")
        return out

    def swap_quadrants(self, im: np.ndarray) -> np.ndarray:
        h, w = im.shape
        buf = np.ascontiguousarray(im, np.float64).copy()
        self.lib.orc_swap_quadrants(buf.ctypes.data_as(_dp), w, h)
        return buf

    def find_peaks(self, im: np.ndarray, num: int, radius: int = 1):
        h, w = im.shape
        buf = np.ascontiguousarray(im, np.float64)
        xy = np.zeros((max(num, 1), 2), np.int32)
        v = np.zeros(max(num, 1), np.float64)
        n = self.lib.orc_find_peaks(buf.ctypes.data_as(_dp), w, h, num, radius,
                                    xy.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
        return xy[:n], v[:n]

    def fit_simple_gaussian(self, plane: np.ndarray, px: int, py: int):
        buf = np.ascontiguousarray(plane, np.float64)
        out = np.zeros(2, np.float64)
        self.lib.orc_fit_simple_gaussian(buf.ctypes.data_as(_dp), plane.shape[1], px, py,
                                         out.ctypes.data_as(_dp))
        return out

    # -- window batches -----------------------------------------------------
    def correlate_windows(self, img_a, img_b, win_xy, w, mode):
        img_a = np.ascontiguousarray(img_a, np.float64)
        img_b = np.ascontiguousarray(img_b, np.float64)
        win_xy = np.ascontiguousarray(win_xy, np.int32)
        n = win_xy.shape[0]
        planes = np.zeros((n, w, w), np.float64)
        rc = self.lib.orc_correlate_windows(img_a.ctypes.data_as(_dp), img_b.ctypes.data_as(_dp),
                                            img_a.shape[1], img_a.shape[0],
                                            win_xy.ctypes.data_as(_ip), n, w, mode,
                                            planes.ctypes.data_as(_dp))
        if rc != 0:
            raise RuntimeError(f"orc_correlate_windows: {rc}")
        return planes

    def process_windows(self, img_a, img_b, win_xy, w, mode, limit_search=False, threads=1):
        """Returns (vectors n x 5 {x, y, u, v, sn}, peaks n x 2, seconds)."""
        img_a = np.ascontiguousarray(img_a, np.float64)
        img_b = np.ascontiguousarray(img_b, np.float64)
        win_xy = np.ascontiguousarray(win_xy, np.int32)
        n = win_xy.shape[0]
        vec = np.zeros((n, 5), np.float64)
        pk = np.zeros((n, 2), np.int32)
        t = self.lib.orc_process_windows(img_a.ctypes.data_as(_dp), img_b.ctypes.data_as(_dp),
                                         img_a.shape[1], img_a.shape[0],
                                         win_xy.ctypes.data_as(_ip), n, w, mode,
                                         int(bool(limit_search)), int(threads),
                                         vec.ctypes.data_as(_dp), pk.ctypes.data_as(_ip))
        if t < 0:
            raise RuntimeError(f"orc_process_windows: {t}")
        return vec, pk, t


    def process_windows_ab(self, img_a, img_b, win_xy, win_b, w, mode, limit_search=False,
                           threads=1):
        """As process_windows, frame B's windows at their own corners."""
        img_a = np.ascontiguousarray(img_a, np.float64)
        img_b = np.ascontiguousarray(img_b, np.float64)
        win_xy = np.ascontiguousarray(win_xy, np.int32)
        win_b = np.ascontiguousarray(win_b, np.int32)
        n = win_xy.shape[0]
        vec = np.zeros((n, 5), np.float64)
        pk = np.zeros((n, 2), np.int32)
        t = self.lib.orc_process_windows_ab(img_a.ctypes.data_as(_dp), img_b.ctypes.data_as(_dp),
                                            img_a.shape[1], img_a.shape[0],
                                            win_xy.ctypes.data_as(_ip), win_b.ctypes.data_as(_ip),
                                            n, w, mode, int(bool(limit_search)), int(threads),
                                            vec.ctypes.data_as(_dp), pk.ctypes.data_as(_ip))
        if t < 0:
            raise RuntimeError(f"orc_process_windows_ab: {t}")
        return vec, pk, t


def nearest_index(c, c0, step, n):
    """Index of the grid line (origin c0, spacing step, n lines) nearest to c:
    floor((c - c0 + step/2) / step) clamped to [0, n - 1] (integer maths)."""
    c = np.asarray(c, np.int64)
    i = np.where(c < c0, 0, (c - c0 + step // 2) // step)
    return np.minimum(i, n - 1)


def multipass(orc, img_a, img_b, passes, mode, limit_search=False, threads=1):
    """The multi-pass window-offsetting chain composed from the reference's
    per-window steps.  passes: [(ia, step), ...].  Returns, per pass, a dict
    with the grid, the B corners, the vectors (total displacement, the
    reference's sign convention), the first-peak positions and the integer
    displacements handed to the next pass."""
    h, w = img_a.shape
    fa, fb = np.asarray(img_a, np.float64), np.asarray(img_b, np.float64)
    out, prev = [], None
    for ia, step in passes:
        grid = orc.grid_offsets(w, h, ia, ia, step, step)
        bx, by = grid[:, 0].astype(np.int64), grid[:, 1].astype(np.int64)
        ox = np.zeros(len(grid), np.int64)
        oy = np.zeros(len(grid), np.int64)
        if prev is not None:
            pg, pdisp, pia, pstep = prev
            pnx = len(np.unique(pg[:, 0]))
            pny = len(pg) // pnx
            ix = nearest_index(bx + ia // 2, pg[0, 0] + pia // 2, pstep, pnx)
            iy = nearest_index(by + ia // 2, pg[0, 1] + pia // 2, pstep, pny)
            d = pdisp[iy * pnx + ix]
            ox = np.clip(d[:, 0], -bx, w - ia - bx)
            oy = np.clip(d[:, 1], -by, h - ia - by)
        bxy = np.stack([bx + ox, by + oy], 1).astype(np.int32)
        vec, pk, _ = orc.process_windows_ab(fa, fb, grid, bxy, ia, mode, limit_search, threads)
        found = pk[:, 0] >= 0
        vec[found, 2] -= ox[found]
        vec[found, 3] -= oy[found]
        disp = np.stack([np.where(found, pk[:, 0] - ia // 2 + ox, ox),
                         np.where(found, pk[:, 1] - ia // 2 + oy, oy)], 1)
        out.append({"grid": grid, "b_xy": bxy, "vec": vec, "peak": pk, "disp": disp})
        prev = (grid, disp, ia, step)
    return out


def get(kind: str = "port", fast: bool = False) -> Oracle:
    key = (kind, fast)
    if key not in _cache:
        _cache[key] = Oracle(kind, fast)
    return _cache[key]
