"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-side parts (grids, argument validation, the
host find_peaks / fit_simple_gaussian) agree with the oracle."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import opiv_gb300 as og

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "openpiv_gb300.h")
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(opiv_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 16
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
    assert set(names) == set(og.SYMBOLS)


def test_status_strings(lib):
    assert og.load().opiv_status_string(og.ERR_NOT_POW2).decode() == "dimensions must be power of 2"
    assert og.load().opiv_status_string(og.ERR_OFFSET_ZERO).decode() == "offsets must be non-zero"


@pytest.mark.parametrize("case", json.load(open(os.path.join(GOLDEN, "reference_kats.json")))["grid"],
                         ids=lambda c: c["cite"])
def test_grid_kats(lib, case):
    (iw, ih), (aw, ah) = case["image"], case["ia"]
    if "frac" in case:
        g = og.grid(iw, ih, aw, ah, case["frac"])
    else:
        g = og.grid_offsets(iw, ih, aw, ah, *case["offsets"])
    assert sorted(map(tuple, g.tolist())) == sorted(map(tuple, case["origins"]))


@pytest.mark.parametrize("args", [(1024, 1024, 32, 32, 0.5), (4096, 4096, 32, 32, 0.25),
                                  (1000, 700, 16, 16, 0.5), (517, 333, 64, 64, 0.75),
                                  (2048, 1536, 64, 64, 0.5), (33, 32, 32, 32, 1.0)])
def test_grid_matches_oracle(lib, orc, args):
    assert np.array_equal(og.grid(*args), orc.grid(*args))


@pytest.mark.parametrize("args,status,msg", [
    ((100, 100, 32, 32, 1.5), og.ERR_OFFSET_RANGE, "offsets must be between 0.0 and 1.0"),
    ((0, 100, 32, 32, 0.5), og.ERR_IMAGE_EMPTY, "image size must be non-zero"),
    ((100, 100, 0, 32, 0.5), og.ERR_IA_EMPTY, "interrogation size must be non-zero"),
    ((100, 100, 32, 32, 0.01), og.ERR_OFFSET_ZERO, "offsets must be non-zero"),
    ((16, 100, 32, 32, 0.5), og.ERR_IA_TOO_BIG, "interrogation size is bigger than image"),
])
def test_grid_errors(lib, args, status, msg):
    with pytest.raises(og.OpivError) as e:
        og.grid(*args)
    assert e.value.status == status
    assert e.value.message.startswith(msg)


def test_plan_validation_precedes_device(lib):
    """Argument errors are reported before any device is touched, in the
    reference's order (grid checks, then the FFT's power-of-two check)."""
    with pytest.raises(og.OpivError) as e:
        og.Plan(100, 100, np.uint8, 24, 8)
    assert e.value.status == og.ERR_NOT_POW2
    assert "power of 2" in e.value.message
    with pytest.raises(og.OpivError) as e:
        og.Plan(100, 100, np.uint8, 128, 8)
    assert e.value.status == og.ERR_IA_TOO_BIG
    with pytest.raises(og.OpivError) as e:
        og.Plan(100, 100, np.uint8, 32, 0)
    assert e.value.status == og.ERR_OFFSET_ZERO
    with pytest.raises(og.OpivError) as e:
        og.Plan(100, 100, np.int32, 32, 8)
    assert e.value.status == og.ERR_ARG
    # 65,521^2 windows: past the 2^31 - 1 a pass indexes (both creators)
    with pytest.raises(og.OpivError) as e:
        og.Plan(65536, 65536, np.uint8, 16, 1)
    assert e.value.status == og.ERR_CAPACITY and "2^31" in e.value.message
    with pytest.raises(og.OpivError) as e:
        og.Plan(65536, 65536, np.uint8, 16, 1, tensor_core=og.PREC_TC_SPLIT_BF16)
    assert e.value.status == og.ERR_CAPACITY


def test_tensor_core_plan_validation_precedes_device(lib):
    """opiv_plan_create_tc: a tensor-core precision, then the grid checks,
    then the window sizes that path takes (16, 32, 48, 64 px of u8/u16
    frames; 48 px, which the FFT path rejects, included) -- all before any
    device is touched."""
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 48, 12, tensor_core=og.PREC_FP32)
    assert e.value.status == og.ERR_ARG
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 48, 12, tensor_core=9)
    assert e.value.status == og.ERR_ARG
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 40, 8, tensor_core=og.PREC_TC_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.float32, 48, 12, tensor_core=og.PREC_TC_BF16)
    assert e.value.status == og.ERR_UNSUPPORTED
    with pytest.raises(og.OpivError) as e:
        og.Plan(40, 256, np.uint16, 48, 12, tensor_core=og.PREC_TC_BF16)
    assert e.value.status == og.ERR_IA_TOO_BIG
    with pytest.raises(og.OpivError) as e:
        og.Plan(256, 256, np.uint16, 48, 12)
    assert e.value.status == og.ERR_NOT_POW2


def test_host_find_peaks_and_fit(lib, orc):
    rng = np.random.default_rng(1)
    for _ in range(20):
        im = rng.normal(size=(32, 32))
        xy1, v1 = og.find_peaks(im, 5, 1)
        xy2, v2 = orc.find_peaks(im, 5, 1)
        assert np.array_equal(xy1, xy2) and np.array_equal(v1, v2)
        plane = np.abs(im) + 1.0
        px, py = int(rng.integers(1, 31)), int(rng.integers(1, 31))
        assert np.array_equal(og.fit_simple_gaussian(plane, px, py),
                              orc.fit_simple_gaussian(plane, px, py))
    with pytest.raises(og.OpivError):
        og.fit_simple_gaussian(np.ones((32, 32)), 0, 5)


def test_batch_schedule_calls_check_arguments(lib):
    """The queue-schedule calls of a batch and the tile calls of a plan
    reject a null handle before they touch a device."""
    L = og.load()
    a, b, m = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    assert L.opiv_batch_set_schedule(None, og.BATCH_QUEUE) == og.ERR_ARG
    assert L.opiv_batch_set_tuning(None, 0, 1, 1) == og.ERR_ARG
    assert L.opiv_batch_get_tuning(None, 0, ctypes.byref(a), ctypes.byref(b), ctypes.byref(m), None) == og.ERR_ARG
    assert L.opiv_batch_autotune(None, None) == og.ERR_ARG
    assert L.opiv_batch_set_lanes(None, 2) == og.ERR_ARG
    assert L.opiv_batch_get_lanes(None) == og.ERR_ARG
    assert L.opiv_plan_set_tile(None, og.TILE_VERTICAL) == og.ERR_ARG
    assert L.opiv_plan_get_tile(None) == og.ERR_ARG
    assert L.opiv_plan_autotune(None, None, None, 0, None) == og.ERR_ARG
    assert L.opiv_plan_test_mma_timeout(None, 1) == og.ERR_ARG
    assert "null" in L.opiv_last_error().decode()


def test_batch_correlation_window_limit(lib):
    """opiv_cross_correlate_batch stacks its windows as the rows of one
    frame indexed in 32 bits: a count past (2^31 - 1) / w is refused before
    any buffer or device is touched."""
    import ctypes as C

    buf = np.zeros(16, np.float64)
    p = buf.ctypes.data_as(C.POINTER(C.c_double))
    st = lib.opiv_cross_correlate_batch(p, p, 16, (2 ** 31) // 16 + 1, og.CORR_COMPLEX, 0, p, 0)
    assert st == og.ERR_CAPACITY
