"""Python binding of the GB300 PIV path -- a thin ctypes layer over the C ABI
declared in include/openpiv_gb300.h (libopenpiv_gb300.so, built in-tree by
openpiv-cxx_gb300/build.py).

There is no fallback: if the shared library is missing, importing the
functions below raises.  Errors of the C ABI become ``OpivError`` carrying
the status code and the library's message (which starts with the text of
the exception the reference throws for the same condition).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libopenpiv_gb300.so")

U8, U16, F32 = 0, 1, 2
CORR_REAL, CORR_COMPLEX, CORR_POCKET, CORR_POCKET_REAL = 0, 1, 2, 3
PEAK_EXACT = 0x40000000
PEAK_MASK = 0x0000FFFF

OK = 0
ERR_OFFSET_RANGE = -1
ERR_IMAGE_EMPTY = -2
ERR_IA_EMPTY = -3
ERR_OFFSET_ZERO = -4
ERR_IA_TOO_BIG = -5
ERR_NOT_POW2 = -6
ERR_CAPACITY = -7
ERR_RECT_OUTSIDE = -8
ERR_ARG = -9
ERR_SIZE_MISMATCH = -10
ERR_UNSUPPORTED = -11
ERR_CUDA = -12
ERR_NO_DEVICE = -13
ERR_TIMEOUT = -14
PREC_FP32, PREC_TC_SPLIT_BF16, PREC_TC_BF16, PREC_FP64 = 0, 1, 2, 3
PREC_TC_SPLIT_FP16, PREC_TC_FP16, PREC_TC_SPLIT2_FP16 = 4, 5, 6

DTYPES = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32}
SYMBOLS = [
    "opiv_last_error", "opiv_status_string", "opiv_version", "opiv_kernel_launch_count",
    "opiv_grid", "opiv_grid_offsets", "opiv_plan_create", "opiv_plan_destroy",
    "opiv_plan_window_count", "opiv_plan_grid", "opiv_process_pair",
    "opiv_process_pair_device", "opiv_plan_exact_count", "opiv_plan_set_timing",
    "opiv_plan_last_timing", "opiv_cross_correlate_batch",
    "opiv_find_peaks", "opiv_fit_simple_gaussian", "opiv_process_pair_device_noalloc",
    "opiv_transform_batch", "opiv_transform_real_batch", "opiv_auto_correlate_batch",
    "opiv_gaussian_offsets",
    "opiv_image_info", "opiv_image_load", "opiv_vectors_write",
    "opiv_multipass_create", "opiv_multipass_destroy", "opiv_multipass_window_count",
    "opiv_multipass_grid", "opiv_multipass_process", "opiv_multipass_process_device",
    "opiv_multipass_results", "opiv_batch_create", "opiv_batch_destroy", "opiv_batch_frames",
    "opiv_batch_upload", "opiv_batch_run", "opiv_batch_window_count", "opiv_batch_results",
    "opiv_plan_set_precision", "opiv_plan_status", "opiv_plan_set_plane_output",
    "opiv_process_pairs", "opiv_plan_adjoint", "opiv_batch_process", "opiv_plan_create_tc",
    "opiv_batch_set_schedule", "opiv_batch_set_tuning", "opiv_batch_get_tuning",
    "opiv_batch_autotune", "opiv_batch_set_lanes", "opiv_batch_get_lanes",
    "opiv_plan_set_tile", "opiv_plan_get_tile", "opiv_plan_autotune",
    "opiv_plan_test_mma_timeout",
]
TILE_AUTO, TILE_VERTICAL, TILE_HORIZONTAL = 0, 1, 2
BATCH_STREAMS, BATCH_QUEUE = 0, 1

VECTOR_DTYPE = np.dtype([("x", np.float32), ("y", np.float32), ("u", np.float32),
                         ("v", np.float32), ("sn", np.float32)])


class OpivError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


_lib = None
_ip = C.POINTER(C.c_int32)
_dp = C.POINTER(C.c_double)


def lib_path() -> str:
    return LIB_PATH


def load(path: str | None = None) -> C.CDLL:
    """Loads the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run build() (the GPU path has no fallback)")
    L = C.CDLL(path)
    L.opiv_last_error.restype = C.c_char_p
    L.opiv_status_string.restype = C.c_char_p
    L.opiv_status_string.argtypes = [C.c_int]
    L.opiv_kernel_launch_count.restype = C.c_int64
    L.opiv_grid.restype = C.c_int64
    L.opiv_grid.argtypes = [C.c_uint32] * 4 + [C.c_double, _ip, C.c_int64]
    L.opiv_grid_offsets.restype = C.c_int64
    L.opiv_grid_offsets.argtypes = [C.c_uint32] * 6 + [_ip, C.c_int64]
    L.opiv_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_int,
                                   C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_int]
    L.opiv_plan_create_tc.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_int,
                                      C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_int,
                                      C.c_int]
    L.opiv_plan_destroy.argtypes = [C.c_void_p]
    L.opiv_plan_window_count.restype = C.c_int64
    L.opiv_plan_window_count.argtypes = [C.c_void_p]
    L.opiv_plan_grid.argtypes = [C.c_void_p, _ip, C.c_int64]
    L.opiv_process_pair.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                    C.c_void_p]
    L.opiv_process_pair_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                           C.c_void_p, C.c_void_p, C.c_void_p]
    L.opiv_plan_exact_count.restype = C.c_int64
    L.opiv_plan_exact_count.argtypes = [C.c_void_p]
    L.opiv_plan_set_timing.argtypes = [C.c_void_p, C.c_int]
    L.opiv_plan_set_precision.argtypes = [C.c_void_p, C.c_int]
    L.opiv_plan_set_tile.argtypes = [C.c_void_p, C.c_int]
    L.opiv_plan_test_mma_timeout.argtypes = [C.c_void_p, C.c_int]
    L.opiv_plan_get_tile.argtypes = [C.c_void_p]
    L.opiv_plan_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    L.opiv_plan_adjoint.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_float,
                                    C.c_float, C.c_void_p, C.c_void_p]
    L.opiv_process_pairs.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_void_p), C.c_size_t, C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_void_p)]
    L.opiv_plan_status.argtypes = [C.c_void_p]
    L.opiv_plan_set_plane_output.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.opiv_plan_last_timing.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.opiv_cross_correlate_batch.argtypes = [_dp, _dp, C.c_uint32, C.c_int64, C.c_int, C.c_int,
                                             _dp, C.c_int]
    L.opiv_process_pair_device_noalloc.argtypes = [
        C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32,
        C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.opiv_image_info.argtypes = [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_int)]
    L.opiv_image_load.argtypes = [C.c_char_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32,
                                  C.c_int]
    L.opiv_vectors_write.argtypes = [C.c_char_p, C.c_void_p, C.c_int64]
    L.opiv_multipass_create.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_int,
                                        C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.c_int, C.c_int, C.c_int]
    L.opiv_multipass_destroy.argtypes = [C.c_void_p]
    L.opiv_multipass_window_count.restype = C.c_int64
    L.opiv_multipass_window_count.argtypes = [C.c_void_p, C.c_int]
    L.opiv_multipass_grid.argtypes = [C.c_void_p, C.c_int, _ip, C.c_int64]
    L.opiv_multipass_process.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
    L.opiv_multipass_process_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                                C.c_void_p]
    L.opiv_multipass_results.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.opiv_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32), C.c_int, C.c_int,
                                    C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_int, C.c_int,
                                    C.c_int]
    L.opiv_batch_destroy.argtypes = [C.c_void_p]
    L.opiv_batch_frames.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
    L.opiv_batch_upload.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t,
                                    C.c_void_p]
    L.opiv_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.opiv_batch_window_count.restype = C.c_int64
    L.opiv_batch_window_count.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.opiv_batch_results.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p]
    L.opiv_batch_process.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_size_t), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.opiv_batch_set_schedule.argtypes = [C.c_void_p, C.c_int]
    L.opiv_batch_set_tuning.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.opiv_batch_get_tuning.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _ip, C.POINTER(C.c_float)]
    L.opiv_batch_autotune.argtypes = [C.c_void_p, C.c_void_p]
    L.opiv_batch_set_lanes.argtypes = [C.c_void_p, C.c_int]
    L.opiv_batch_get_lanes.argtypes = [C.c_void_p]
    L.opiv_find_peaks.argtypes = [_dp, C.c_uint32, C.c_uint32, C.c_uint16, C.c_uint32, _ip, _dp]
    L.opiv_fit_simple_gaussian.argtypes = [_dp, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, _dp]
    L.opiv_transform_batch.argtypes = [_dp, C.c_uint32, C.c_int64, C.c_int, _dp, C.c_int]
    L.opiv_transform_real_batch.argtypes = [_dp, _dp, C.c_uint32, C.c_int64, C.c_int, _dp, _dp, C.c_int]
    L.opiv_auto_correlate_batch.argtypes = [_dp, C.c_uint32, C.c_int64, _dp, C.c_int]
    L.opiv_gaussian_offsets.argtypes = [_dp, _dp]
    _lib = L
    return L


def _check(status: int) -> int:
    if status < 0:
        raise OpivError(int(status), load().opiv_last_error().decode())
    return status


def last_error() -> str:
    return load().opiv_last_error().decode()


def kernel_launch_count() -> int:
    return int(load().opiv_kernel_launch_count())


# ---- grid ------------------------------------------------------------------
def grid(img_w: int, img_h: int, ia_w: int, ia_h: int, step_fraction: float) -> np.ndarray:
    """core::generate_cartesian_grid(size, size, double): (n, 2) int32 corners."""
    L = load()
    n = _check(L.opiv_grid(img_w, img_h, ia_w, ia_h, step_fraction, None, 0))
    out = np.zeros((n, 2), np.int32)
    _check(L.opiv_grid(img_w, img_h, ia_w, ia_h, step_fraction, out.ctypes.data_as(_ip), n))
    return out


def grid_offsets(img_w: int, img_h: int, ia_w: int, ia_h: int, dx: int, dy: int) -> np.ndarray:
    L = load()
    n = _check(L.opiv_grid_offsets(img_w, img_h, ia_w, ia_h, dx, dy, None, 0))
    out = np.zeros((n, 2), np.int32)
    _check(L.opiv_grid_offsets(img_w, img_h, ia_w, ia_h, dx, dy, out.ctypes.data_as(_ip), n))
    return out


# ---- plans -----------------------------------------------------------------
class Plan:
    """One image geometry + window size + grid step + correlation mode."""

    def __init__(self, img_w: int, img_h: int, dtype, ia: int, dx: int, dy: int | None = None,
                 mode: int = CORR_COMPLEX, limit_search: bool = False, device: int = 0,
                 tensor_core: int | None = None):
        """tensor_core: one of the PREC_TC_* precisions for a plan of the
        tensor-core path alone (opiv_plan_create_tc: 16, 32, 48 or 64 px
        windows, 48 included)."""
        L = load()
        dy = dx if dy is None else dy
        self.dtype = np.dtype(dtype)
        if self.dtype not in DTYPES:
            raise OpivError(ERR_ARG, f"unsupported pixel type {self.dtype}")
        h = C.c_void_p()
        if tensor_core is not None:
            _check(L.opiv_plan_create_tc(C.byref(h), img_w, img_h, DTYPES[self.dtype], ia, dx, dy, mode,
                                         int(bool(limit_search)), tensor_core, device))
        else:
            _check(L.opiv_plan_create(C.byref(h), img_w, img_h, DTYPES[self.dtype], ia, dx, dy, mode,
                                      int(bool(limit_search)), device))
        self._h = h
        self.img_w, self.img_h, self.ia, self.dx, self.dy = img_w, img_h, ia, dx, dy
        self.mode, self.limit_search = mode, bool(limit_search)
        self.n = int(L.opiv_plan_window_count(h))

    @property
    def handle(self) -> int:
        return self._h.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().opiv_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.int32)
        _check(load().opiv_plan_grid(self._h, out.ctypes.data_as(_ip), self.n))
        return out

    def process(self, frame_a: np.ndarray, frame_b: np.ndarray, with_peaks: bool = True):
        """Host arrays in, (vectors (n, 5) float32, peak codes (n,) int32) out."""
        for f in (frame_a, frame_b):
            if f.dtype != self.dtype or f.shape != (self.img_h, self.img_w):
                raise OpivError(ERR_SIZE_MISMATCH,
                                f"image size is different from expected: {f.shape} {f.dtype}")
        fa = np.ascontiguousarray(frame_a)
        fb = np.ascontiguousarray(frame_b)
        vec = np.zeros((self.n, 5), np.float32)
        pk = np.zeros(self.n, np.int32) if with_peaks else None
        _check(load().opiv_process_pair(self._h, fa.ctypes.data, fb.ctypes.data, fa.strides[0],
                                        vec.ctypes.data, pk.ctypes.data if with_peaks else None))
        return vec, pk

    def process_into(self, pa: int, pb: int, pitch: int, out_vec: int, out_peak: int | None):
        """Host pointers (e.g. pinned buffers) in and out; synchronous."""
        _check(load().opiv_process_pair(self._h, pa, pb, pitch, out_vec, out_peak))

    def process_device(self, d_a: int, d_b: int, pitch: int, d_vec: int, d_peak: int | None,
                       stream: int = 0):
        """Device pointers; asynchronous on `stream` (a cudaStream_t value)."""
        _check(load().opiv_process_pair_device(self._h, d_a, d_b, pitch, d_vec, d_peak,
                                               stream or None))

    def exact_count(self) -> int:
        return int(load().opiv_plan_exact_count(self._h))

    def process_pairs_into(self, ptrs_a, ptrs_b, pitch: int, ptrs_vec, ptrs_peak=None):
        """Host pointers (pinned for overlap), one per pair: pipelined passes."""
        n = len(ptrs_a)
        arr = lambda xs: (C.c_void_p * n)(*xs)
        _check(load().opiv_process_pairs(self._h, n, arr(ptrs_a), arr(ptrs_b), pitch, arr(ptrs_vec),
                                         arr(ptrs_peak) if ptrs_peak is not None else None))

    def process_pairs(self, pairs):
        """[(frame_a, frame_b), ...] numpy frames -> [(vectors, peaks), ...]."""
        fr = [(np.ascontiguousarray(a, self.dtype), np.ascontiguousarray(b, self.dtype)) for a, b in pairs]
        for a, b in fr:
            if a.shape != (self.img_h, self.img_w) or b.shape != (self.img_h, self.img_w):
                raise OpivError(ERR_SIZE_MISMATCH, f"image size is different from expected: {a.shape}")
        outs = [(np.zeros((self.n, 5), np.float32), np.zeros(self.n, np.int32)) for _ in fr]
        self.process_pairs_into([a.ctypes.data for a, _ in fr], [b.ctypes.data for _, b in fr],
                                fr[0][0].strides[0] if fr else 0,
                                [v.ctypes.data for v, _ in outs], [p.ctypes.data for _, p in outs])
        return outs

    def adjoint_device(self, d_a: int, d_b: int, pitch: int, d_peak: int, d_cot: int = 0,
                       d_grad_a: int = 0, d_grad_b: int = 0, grad_pitch: int = 0,
                       var_a: float = 0.0, var_b: float = 0.0, d_sigma: int = 0, stream: int = 0):
        """Device pointers: see opiv_plan_adjoint."""
        _check(load().opiv_plan_adjoint(self._h, d_a, d_b, pitch, d_peak, d_cot or None,
                                        d_grad_a or None, d_grad_b or None, grad_pitch, var_a, var_b,
                                        d_sigma or None, stream or None))

    def test_mma_timeout(self, on: bool):
        """Failure-path test: the 32 px tensor-core kernel issues no MMAs, its
        bounded waits run out and the pass raises ERR_TIMEOUT."""
        _check(load().opiv_plan_test_mma_timeout(self._h, int(bool(on))))

    def set_tile(self, tile: int):
        """32 px tensor-core tile shape: TILE_AUTO, TILE_VERTICAL or TILE_HORIZONTAL."""
        _check(load().opiv_plan_set_tile(self._h, tile))

    def tile(self) -> int:
        return _check(load().opiv_plan_get_tile(self._h))

    def autotune(self, d_a: int, d_b: int, pitch: int, stream: int = 0) -> int:
        """Times the tile shapes on device frames, keeps the faster; returns it."""
        _check(load().opiv_plan_autotune(self._h, d_a, d_b, pitch, stream or None))
        return self.tile()

    def set_precision(self, precision: int):
        """PREC_FP32 (default, reference-exact peaks), PREC_TC_SPLIT_BF16,
        PREC_TC_BF16, PREC_TC_SPLIT_FP16, PREC_TC_FP16 (tensor cores, 32 x 32
        windows) or PREC_FP64 (every window through the exact kernel)."""
        _check(load().opiv_plan_set_precision(self._h, precision))

    def status(self):
        _check(load().opiv_plan_status(self._h))

    def set_plane_output(self, d_planes: int, d_pedestals: int):
        _check(load().opiv_plan_set_plane_output(self._h, d_planes or None, d_pedestals or None))

    def set_timing(self, enable: bool = True):
        _check(load().opiv_plan_set_timing(self._h, int(bool(enable))))

    def last_timing(self) -> tuple[float, float]:
        """(FP32 kernel ms, exact pass ms) of the last pass."""
        a, b = C.c_float(), C.c_float()
        _check(load().opiv_plan_last_timing(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value


# ---- multi-pass window offsetting ------------------------------------------
def unpack_disp(d: np.ndarray) -> np.ndarray:
    """(n,) packed (dy << 16) | (dx & 0xffff) -> (n, 2) int (dx, dy)."""
    d = np.asarray(d, np.int32)
    return np.stack([(d & 0xFFFF).astype(np.uint16).astype(np.int16).astype(np.int64),
                     (d >> 16).astype(np.int64)], 1)


class MultiPass:
    """A chain of passes (window sizes / steps) over one image pair; pass k's
    frame-B windows are offset by pass k-1's integer displacements."""

    def __init__(self, img_w: int, img_h: int, dtype, passes, mode: int = CORR_COMPLEX,
                 limit_search: bool = False, device: int = 0):
        L = load()
        self.dtype = np.dtype(dtype)
        if self.dtype not in DTYPES:
            raise OpivError(ERR_ARG, f"unsupported pixel type {self.dtype}")
        ia = (C.c_uint32 * len(passes))(*[p[0] for p in passes])
        st = (C.c_uint32 * len(passes))(*[p[1] for p in passes])
        h = C.c_void_p()
        _check(L.opiv_multipass_create(C.byref(h), img_w, img_h, DTYPES[self.dtype], len(passes),
                                       ia, st, mode, int(bool(limit_search)), device))
        self._h = h
        self.passes = list(passes)
        self.img_w, self.img_h = img_w, img_h
        self.counts = [int(L.opiv_multipass_window_count(h, k)) for k in range(len(passes))]

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().opiv_multipass_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self, k: int) -> np.ndarray:
        out = np.zeros((self.counts[k], 2), np.int32)
        _check(load().opiv_multipass_grid(self._h, k, out.ctypes.data_as(_ip), self.counts[k]))
        return out

    def process(self, frame_a: np.ndarray, frame_b: np.ndarray):
        """Runs every pass; returns the last pass's (vectors, peak codes, displacements)."""
        fa = np.ascontiguousarray(frame_a, self.dtype)
        fb = np.ascontiguousarray(frame_b, self.dtype)
        n = self.counts[-1]
        vec = np.zeros((n, 5), np.float32)
        pk = np.zeros(n, np.int32)
        disp = np.zeros(n, np.int32)
        _check(load().opiv_multipass_process(self._h, fa.ctypes.data, fb.ctypes.data, fa.strides[0],
                                             vec.ctypes.data, pk.ctypes.data, disp.ctypes.data))
        return vec, pk, unpack_disp(disp)

    def results(self, k: int):
        n = self.counts[k]
        vec = np.zeros((n, 5), np.float32)
        pk = np.zeros(n, np.int32)
        disp = np.zeros(n, np.int32)
        _check(load().opiv_multipass_results(self._h, k, vec.ctypes.data, pk.ctypes.data,
                                             disp.ctypes.data))
        return vec, pk, unpack_disp(disp)


class Batch:
    """Many image pairs (sizes may differ) through one multi-pass schedule,
    submitted together (optionally as one replayed CUDA graph)."""

    def __init__(self, sizes, dtype, passes, mode: int = CORR_COMPLEX,
                 limit_search: bool = False, device: int = 0):
        L = load()
        self.dtype = np.dtype(dtype)
        n = len(sizes)
        ws = (C.c_uint32 * n)(*[s[0] for s in sizes])
        hs = (C.c_uint32 * n)(*[s[1] for s in sizes])
        ia = (C.c_uint32 * len(passes))(*[p[0] for p in passes])
        st = (C.c_uint32 * len(passes))(*[p[1] for p in passes])
        h = C.c_void_p()
        _check(L.opiv_batch_create(C.byref(h), n, ws, hs, DTYPES[self.dtype], len(passes), ia, st,
                                   mode, int(bool(limit_search)), device))
        self._h = h
        self.sizes, self.passes = list(sizes), list(passes)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().opiv_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, pair: int, frame_a: np.ndarray, frame_b: np.ndarray, stream: int = 0):
        fa = np.ascontiguousarray(frame_a, self.dtype)
        fb = np.ascontiguousarray(frame_b, self.dtype)
        _check(load().opiv_batch_upload(self._h, pair, fa.ctypes.data, fb.ctypes.data,
                                        fa.strides[0], stream or None))

    def run(self, use_graph: bool = True, stream: int = 0):
        _check(load().opiv_batch_run(self._h, int(bool(use_graph)), stream or None))

    def set_schedule(self, schedule: int):
        """BATCH_STREAMS (per-pair pass chains on fork streams) or BATCH_QUEUE
        (per pass one persistent kernel over a device work queue of all pairs)."""
        _check(load().opiv_batch_set_schedule(self._h, schedule))

    def set_tuning(self, k: int, ctas_per_sm: int, chunk: int):
        _check(load().opiv_batch_set_tuning(self._h, k, ctas_per_sm, chunk))

    def tuning(self, k: int):
        """(CTAs per SM, tasks per warp and dequeue, resident CTA limit, the
        autotuner's fastest pass time in ms or 0) of pass k's queue."""
        c, ch, mx, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_float()
        _check(load().opiv_batch_get_tuning(self._h, k, C.byref(c), C.byref(ch), C.byref(mx), C.byref(ms)))
        return c.value, ch.value, mx.value, ms.value

    def set_lanes(self, lanes: int):
        """Queue schedule: the pairs split into `lanes` chains on fork streams."""
        _check(load().opiv_batch_set_lanes(self._h, lanes))

    def lanes(self) -> int:
        return _check(load().opiv_batch_get_lanes(self._h))

    def autotune(self, stream: int = 0):
        """Queue schedule; each pass's grid and chunk timed on the frames held now."""
        _check(load().opiv_batch_autotune(self._h, stream or None))

    def process_into(self, ptrs_a, ptrs_b, pitches, ptrs_vec, ptrs_peak=None):
        """Host pointers, one per pair (pinned for overlap): every pair's
        upload, passes and final-pass download, pipelined (opiv_batch_process)."""
        n = len(self.sizes)
        arr = lambda xs: (C.c_void_p * n)(*xs)
        _check(load().opiv_batch_process(self._h, arr(ptrs_a), arr(ptrs_b), (C.c_size_t * n)(*pitches),
                                         arr(ptrs_vec), arr(ptrs_peak) if ptrs_peak is not None else None))

    def process(self, frames):
        """[(frame_a, frame_b), ...] numpy frames, one per pair -> [(final-pass
        vectors, peak codes), ...]."""
        if len(frames) != len(self.sizes):
            raise OpivError(ERR_ARG, f"{len(frames)} pairs for a batch of {len(self.sizes)}")
        fr = [(np.ascontiguousarray(a, self.dtype), np.ascontiguousarray(b, self.dtype)) for a, b in frames]
        for (a, b), (w, h) in zip(fr, self.sizes):
            if a.shape != (h, w) or b.shape != (h, w):
                raise OpivError(ERR_SIZE_MISMATCH, f"image size is different from expected: {a.shape}")
        last = len(self.passes) - 1
        outs = [(np.zeros((self.window_count(i, last), 5), np.float32),
                 np.zeros(self.window_count(i, last), np.int32)) for i in range(len(fr))]
        self.process_into([a.ctypes.data for a, _ in fr], [b.ctypes.data for _, b in fr],
                          [a.strides[0] for a, _ in fr], [v.ctypes.data for v, _ in outs],
                          [p.ctypes.data for _, p in outs])
        return outs

    def window_count(self, pair: int, k: int) -> int:
        return int(load().opiv_batch_window_count(self._h, pair, k))

    def results(self, pair: int, k: int):
        n = self.window_count(pair, k)
        vec = np.zeros((n, 5), np.float32)
        pk = np.zeros(n, np.int32)
        disp = np.zeros(n, np.int32)
        _check(load().opiv_batch_results(self._h, pair, k, vec.ctypes.data, pk.ctypes.data,
                                         disp.ctypes.data))
        return vec, pk, unpack_disp(disp)


# ---- allocation-free pass --------------------------------------------------
def process_pair_device_noalloc(d_a: int, d_b: int, pitch: int, img_w: int, img_h: int, dtype,
                                ia: int, dx: int, dy: int, mode: int, limit_search: bool,
                                d_vec: int, d_peak: int | None, stream: int = 0):
    """The pass without a plan and without any device allocation (current
    device, asynchronous on `stream`).  See opiv_process_pair_device_noalloc."""
    _check(load().opiv_process_pair_device_noalloc(
        d_a, d_b, pitch, img_w, img_h, DTYPES[np.dtype(dtype)], ia, dx, dy, mode,
        int(bool(limit_search)), d_vec, d_peak, stream or None))


# ---- per-window API --------------------------------------------------------
def cross_correlate_batch(a: np.ndarray, b: np.ndarray, mode: int, exact: bool = False,
                          device: int = 0) -> np.ndarray:
    """FFT::cross_correlate[_real] on (n, w, w) window stacks -> (n, w, w) planes."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    if a.ndim == 2:
        a, b = a[None], b[None]
    if a.shape != b.shape:
        raise OpivError(ERR_SIZE_MISMATCH, f"image size is different from expected: {a.shape}")
    n, h, w = a.shape
    if h != w:
        raise OpivError(ERR_UNSUPPORTED, f"no kernel for {w}x{h} windows")
    out = np.zeros((n, w, w), np.float64)
    _check(load().opiv_cross_correlate_batch(a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), w, n,
                                             mode, int(bool(exact)), out.ctypes.data_as(_dp),
                                             device))
    return out


FORWARD, REVERSE = 0, 1   # algos::direction


def _stack(z, dtype):
    z = np.ascontiguousarray(z, dtype)
    return z[None] if z.ndim == 2 else z


def transform_batch(z: np.ndarray, direction: int = FORWARD, device: int = 0) -> np.ndarray:
    """FFT::transform (fft.h:87-119) of (n, w, w) or (w, w) complex windows,
    on the GPU in the reference's double arithmetic."""
    z = _stack(z, np.complex128)
    out = np.zeros_like(z)
    _check(load().opiv_transform_batch(z.ctypes.data_as(_dp), z.shape[-1], z.shape[0], direction,
                                       out.ctypes.data_as(_dp), device))
    return out


def transform_real_batch(a: np.ndarray, b: np.ndarray, direction: int = FORWARD, device: int = 0):
    """FFT::transform_real (fft.h:123-186): the two spectra of real windows a, b."""
    a, b = _stack(a, np.float64), _stack(b, np.float64)
    if a.shape != b.shape:
        raise OpivError(ERR_SIZE_MISMATCH, f"image size is different from expected: {a.shape}")
    oa = np.zeros(a.shape, np.complex128)
    ob = np.zeros(a.shape, np.complex128)
    _check(load().opiv_transform_real_batch(a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), a.shape[-1],
                                            a.shape[0], direction, oa.ctypes.data_as(_dp),
                                            ob.ctypes.data_as(_dp), device))
    return oa, ob


def auto_correlate_batch(z: np.ndarray, device: int = 0) -> np.ndarray:
    """FFT::auto_correlate (fft.h:229-242): complex planes, zero imaginary parts."""
    z = _stack(z, np.complex128)
    out = np.zeros_like(z)
    _check(load().opiv_auto_correlate_batch(z.ctypes.data_as(_dp), z.shape[-1], z.shape[0],
                                            out.ctypes.data_as(_dp), device))
    return out


def find_peaks(im: np.ndarray, num_peaks: int, radius: int = 1):
    im = np.ascontiguousarray(im, np.float64)
    h, w = im.shape
    xy = np.zeros((max(num_peaks, 1), 2), np.int32)
    v = np.zeros(max(num_peaks, 1), np.float64)
    n = _check(load().opiv_find_peaks(im.ctypes.data_as(_dp), w, h, num_peaks, radius,
                                      xy.ctypes.data_as(_ip), v.ctypes.data_as(_dp)))
    return xy[:n], v[:n]


def fit_simple_gaussian(plane: np.ndarray, px: int, py: int) -> np.ndarray:
    plane = np.ascontiguousarray(plane, np.float64)
    out = np.zeros(2, np.float64)
    _check(load().opiv_fit_simple_gaussian(plane.ctypes.data_as(_dp), plane.shape[1],
                                           plane.shape[0], px, py, out.ctypes.data_as(_dp)))
    return out


# ---- image ingest and vector output ---------------------------------------
def load_image(path: str) -> np.ndarray:
    """PNM (P5/P6) or uncompressed TIFF -> (h, w) uint8 or uint16 grey samples."""
    L = load()
    w, h, dt = C.c_uint32(), C.c_uint32(), C.c_int()
    _check(L.opiv_image_info(path.encode(), C.byref(w), C.byref(h), C.byref(dt)))
    out = np.zeros((h.value, w.value), np.uint16 if dt.value == U16 else np.uint8)
    _check(L.opiv_image_load(path.encode(), out.ctypes.data, out.strides[0], w.value, h.value,
                             dt.value))
    return out


def write_vectors(path: str, vectors: np.ndarray) -> None:
    """The reference app's text output: one "x, y, u, v, sn" line per window."""
    v = np.ascontiguousarray(vectors, np.float32)
    _check(load().opiv_vectors_write(path.encode(), v.ctypes.data, v.shape[0]))
