"""The allocation-free entry point, opiv_process_pair_device_noalloc.

It is for callers that cannot allocate device memory once they are running
(a fixed-budget acquisition loop, a host that owns the device allocator):
the pass keeps its scratch in one fixed device array instead of a plan.
These checks call it through the C ABI and compare its output with the
plan-based device call (opiv_process_pair_device) on the same frames, on two
calls in a row (the shared scratch must be reset between calls), over both
window sizes it takes (16 and 32 px), 8- and 16-bit frames and the limited
search; they also check that a grid larger than the fixed scratch and a
64 px window are refused.  This file is named so that pytest collects it
last."""
import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth

pytestmark = pytest.mark.gpu

UV_TOL = 1e-4


def _frames(torch, dtype):
    a, b = synth.config2(size=1024)
    if dtype == np.uint8:
        a, b = (a >> 4).astype(np.uint8), (b >> 4).astype(np.uint8)
        return a, b, torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    # uploaded through an int16 view: same bytes, a dtype every torch build copies
    return (a, b, torch.from_numpy(a.view(np.int16)).cuda(),
            torch.from_numpy(b.view(np.int16)).cuda())


CASES = [
    (32, 8, np.uint16, og.CORR_COMPLEX, False),
    (32, 8, np.uint16, og.CORR_REAL, False),
    (16, 4, np.uint16, og.CORR_COMPLEX, False),
    (16, 8, np.uint8, og.CORR_REAL, True),
    (32, 16, np.uint8, og.CORR_POCKET, True),
]


@pytest.mark.parametrize("ia,step,dtype,mode,limit", CASES)
def test_noalloc_matches_plan_call_twice(ia, step, dtype, mode, limit):
    torch = pytest.importorskip("torch")
    a, b, da, db = _frames(torch, dtype)
    h, w = a.shape
    pitch = w * np.dtype(dtype).itemsize
    s = torch.cuda.Stream()
    # the frames were copied on torch's current stream: order the passes after them
    s.wait_stream(torch.cuda.current_stream())
    plan = og.Plan(w, h, dtype, ia, step, mode=mode, limit_search=limit)
    with torch.cuda.stream(s):
        ref_vec = torch.zeros((plan.n, 5), dtype=torch.float32, device="cuda")
        ref_pk = torch.zeros(plan.n, dtype=torch.int32, device="cuda")
    plan.process_device(da.data_ptr(), db.data_ptr(), pitch, ref_vec.data_ptr(),
                        ref_pk.data_ptr(), s.cuda_stream)
    s.synchronize()
    ref_vec, ref_pk = ref_vec.cpu().numpy(), ref_pk.cpu().numpy()
    for call in range(2):
        with torch.cuda.stream(s):
            vec = torch.full((plan.n, 5), -7.0, dtype=torch.float32, device="cuda")
            pk = torch.full((plan.n,), -7, dtype=torch.int32, device="cuda")
        og.process_pair_device_noalloc(da.data_ptr(), db.data_ptr(), pitch, w, h, dtype, ia, step,
                                       step, mode, limit, vec.data_ptr(), pk.data_ptr(),
                                       s.cuda_stream)
        s.synchronize()
        vec, pk = vec.cpu().numpy(), pk.cpu().numpy()
        assert np.array_equal(pk, ref_pk), f"call {call}: peaks differ"
        assert np.array_equal(np.isnan(vec), np.isnan(ref_vec)), f"call {call}: NaN pattern"
        d = np.nan_to_num(np.abs(vec[:, 2:4] - ref_vec[:, 2:4]))
        assert d.max() <= UV_TOL, f"call {call}: displacements differ by {d.max()}"
        assert np.array_equal(vec[:, :2], ref_vec[:, :2])
        sn_ok = np.isclose(vec[:, 4], ref_vec[:, 4], rtol=1e-5, atol=0.0) | \
            (np.isnan(vec[:, 4]) & np.isnan(ref_vec[:, 4]))
        assert sn_ok.all(), f"call {call}: sn differs"
    plan.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    side = 8192   # 16 x 16 windows at step 4: 2045^2 = 4,182,025 windows > 1,048,576
    da = torch.empty((side, side), dtype=torch.int16, device="cuda")
    vec = torch.empty((16, 5), dtype=torch.float32, device="cuda")
    with pytest.raises(og.OpivError) as e:
        og.process_pair_device_noalloc(da.data_ptr(), da.data_ptr(), side * 2, side, side,
                                       np.uint16, 16, 4, 4, og.CORR_COMPLEX, False,
                                       vec.data_ptr(), None, 0)
    assert e.value.status == og.ERR_CAPACITY
    assert "exceed the fixed scratch" in e.value.message
    # 64 px windows: the fixed twiddle tables cover 16 and 32 px only
    with pytest.raises(og.OpivError) as e:
        og.process_pair_device_noalloc(da.data_ptr(), da.data_ptr(), side * 2, 1024, 1024,
                                       np.uint16, 64, 32, 32, og.CORR_COMPLEX, False,
                                       vec.data_ptr(), None, 0)
    assert e.value.status == og.ERR_UNSUPPORTED
