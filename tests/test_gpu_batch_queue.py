"""GPU: the queue schedule of a batch (per pass one persistent kernel over a
device work queue of every pair's windows, then one exact re-decision launch
over all pairs' flagged windows) against per-pair MultiPass runs of the same
frames.  Every window is computed by the same arithmetic whichever warp or
CTA takes it, so results must be identical (vectors, peak codes,
displacements, every pass), for every tuning, eager or replayed as a graph,
and after the autotuner.
"""
import numpy as np
import pytest

import opiv_gb300 as og
from opiv_gb300 import synth

pytestmark = pytest.mark.gpu

# (780, 520): rows of 1,560 bytes and a 16 px grid starting at x = 2, so the
# 16 px pass takes the element-load form of the kernel; (256, 256): a
# periodic pair whose tied peaks go to the exact pass
SIZES = [(512, 384), (780, 520), (1024, 1024), (256, 256)]
PASSES = [(64, 32), (32, 16), (16, 8)]


def make_frames(j):
    out = []
    for i, (w, h) in enumerate(SIZES[:3]):
        out.append(synth.particle_pair(
            h, w, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
            displacement=synth.lamb_oseen(w / 2.0, h / 2.0, offset=(1.1 - i, 0.4 + j)),
            dtype=np.uint16, seed=synth.SEED_BASE + 4100 + 10 * i + j, full_scale=4095.0))
    rng = np.random.default_rng(77 + j)
    a = np.tile(rng.integers(0, 4096, (8, 8)).astype(np.uint16), (32, 32))
    out.append((a, np.roll(a, (2, 3), (0, 1))))
    return out


@pytest.fixture(scope="module")
def data():
    frames = [make_frames(0), make_frames(1)]
    expect = []
    for j in range(2):
        per = []
        for i, (w, h) in enumerate(SIZES):
            mp = og.MultiPass(w, h, np.uint16, PASSES)
            mp.process(*frames[j][i])
            per.append([mp.results(k) for k in range(len(PASSES))])
            mp.close()
        expect.append(per)
    # the periodic pair makes the exact queue kernel do real work
    assert any(np.any(expect[0][3][k][1] & og.PEAK_EXACT) for k in range(len(PASSES)))
    return frames, expect


def check(batch, expect, label):
    for i in range(len(SIZES)):
        for k in range(len(PASSES)):
            got = batch.results(i, k)
            for g, r, name in zip(got, expect[i][k], ("vectors", "peaks", "displacements")):
                assert np.array_equal(g, r), f"{label}: pair {i} pass {k} {name} differ"


def upload(batch, frames):
    for i in range(len(SIZES)):
        batch.upload(i, *frames[i])


def test_queue_schedule_matches_per_pair_multipass(data):
    frames, expect = data
    batch = og.Batch(SIZES, np.uint16, PASSES)
    batch.set_schedule(og.BATCH_QUEUE)
    upload(batch, frames[0])
    assert batch.lanes() == 2
    n0 = og.kernel_launch_count()
    batch.run(use_graph=False)
    assert og.kernel_launch_count() - n0 == 2 * 2 * len(PASSES)   # two lanes of one group each
    check(batch, expect[0], "queue, default tuning")
    for lanes in (1, 3, 4, 2):
        batch.set_lanes(lanes)
        n0 = og.kernel_launch_count()
        batch.run(use_graph=False)
        assert og.kernel_launch_count() - n0 == 2 * lanes * len(PASSES)
        check(batch, expect[0], f"queue, {lanes} lanes")
    for k in range(len(PASSES)):
        c, ch, mx, ms = batch.tuning(k)
        assert mx >= 1 and c == mx and ch == 1 and ms == 0
    # every tuning gives the same windows; 9 CTAs per SM exceeds the resident
    # limit (the extra CTAs run later), chunk 3 leaves a partial last chunk
    for c, ch in [(1, 1), (2, 3), (4, 8), (9, 1), (3, 1024), (0, 1)]:
        for k in range(len(PASSES)):
            batch.set_tuning(k, c, ch)
        batch.run(use_graph=False)
        check(batch, expect[0], f"queue, {c} CTAs/SM, chunk {ch}")
    # graph: eager run + capture, then replays after new frames
    batch.run(use_graph=True)
    check(batch, expect[0], "queue, first graph call")
    for j in (1, 0, 1):
        upload(batch, frames[j])
        n0 = og.kernel_launch_count()
        batch.run(use_graph=True)
        assert og.kernel_launch_count() - n0 == 2 * 2 * len(PASSES)
        check(batch, expect[j], f"queue, replay {j}")
    # back to the streams schedule: same results
    batch.set_schedule(og.BATCH_STREAMS)
    upload(batch, frames[0])
    batch.run(use_graph=True)
    check(batch, expect[0], "streams after queue")
    batch.close()


def test_autotune_and_host_call(data):
    frames, expect = data
    batch = og.Batch(SIZES, np.uint16, PASSES)
    upload(batch, frames[1])
    batch.autotune()
    check(batch, expect[1], "after autotune")
    for k in range(len(PASSES)):
        c, ch, mx, ms = batch.tuning(k)
        assert 0 <= c <= min(mx, 4) and ch in (1, 2, 4, 8) and ms > 0
    assert batch.lanes() in (1, 2)
    upload(batch, frames[0])
    batch.run(use_graph=True)
    batch.run(use_graph=True)
    check(batch, expect[0], "autotuned graph")
    # host frames in, final vectors out, under the queue schedule
    last = len(PASSES) - 1
    for j in (1, 0):
        n0 = og.kernel_launch_count()
        outs = batch.process(frames[j])
        assert og.kernel_launch_count() - n0 == 2 * batch.lanes() * len(PASSES)
        for i, (vec, pk) in enumerate(outs):
            assert np.array_equal(vec, expect[j][i][last][0]), f"process {j}: pair {i} vectors differ"
            assert np.array_equal(pk, expect[j][i][last][1]), f"process {j}: pair {i} peaks differ"
    with pytest.raises(og.OpivError):
        batch.set_tuning(0, -1, 1)
    with pytest.raises(og.OpivError):
        batch.set_tuning(len(PASSES), 1, 1)
    with pytest.raises(og.OpivError):
        batch.set_schedule(7)
    with pytest.raises(og.OpivError):
        batch.set_lanes(0)
    batch.close()



def test_queue_groups_of_many_pairs():
    """More pairs than one queue holds (64): the pass runs as several queues
    (two launches each); results equal the streams schedule's."""
    n = 70
    sizes = [(128 + 16 * (i % 3), 128 + 8 * (i % 5)) for i in range(n)]
    passes = [(32, 16), (16, 8)]
    frames = []
    for i, (w, h) in enumerate(sizes):
        a = synth.particle_pair(h, w, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                                displacement=synth.lamb_oseen(w / 2.0, h / 2.0, offset=(0.3, -0.7)),
                                dtype=np.uint16, seed=synth.SEED_BASE + 4300 + i, full_scale=4095.0)
        frames.append(a)
    batch = og.Batch(sizes, np.uint16, passes)
    for i in range(n):
        batch.upload(i, *frames[i])
    batch.run(use_graph=False)
    ref = [[batch.results(i, k) for k in range(len(passes))] for i in range(n)]
    batch.set_schedule(og.BATCH_QUEUE)
    batch.set_lanes(1)                    # one lane: groups of 64 and 6 pairs
    n0 = og.kernel_launch_count()
    batch.run(use_graph=False)
    assert og.kernel_launch_count() - n0 == 2 * 2 * len(passes)
    for i in range(n):
        for k in range(len(passes)):
            for g, r in zip(batch.results(i, k), ref[i][k]):
                assert np.array_equal(g, r), f"pair {i} pass {k} differs"
    batch.close()


@pytest.mark.parametrize("mode,limit,dtype", [(og.CORR_REAL, True, np.uint8),
                                              (og.CORR_COMPLEX, True, np.float32),
                                              (og.CORR_POCKET_REAL, False, np.uint8)])
def test_queue_other_modes_and_pixel_types(mode, limit, dtype):
    """REAL and pocket modes, limited peak search, 8-bit and float frames:
    the queue schedule's windows equal the streams schedule's."""
    sizes = [(384, 256), (512, 512), (264, 200)]
    passes = [(64, 32), (32, 16), (16, 8)]
    batch = og.Batch(sizes, dtype, passes, mode=mode, limit_search=limit)
    for i, (w, h) in enumerate(sizes):
        if dtype == np.uint8:
            a, b = synth.particle_pair(h, w, ppp=0.02, i0_range=(150, 255), noise=3.0,
                                       displacement=synth.lamb_oseen(w / 2.0, h / 2.0, offset=(0.7, -1.2)),
                                       dtype=np.uint8, seed=synth.SEED_BASE + 4500 + i, full_scale=255.0)
        else:
            a, b = synth.particle_pair(h, w, ppp=0.02, i0_range=(0.6, 1.0), noise=0.02,
                                       displacement=synth.lamb_oseen(w / 2.0, h / 2.0, offset=(0.7, -1.2)),
                                       dtype=np.float32, seed=synth.SEED_BASE + 4600 + i, full_scale=None)
        batch.upload(i, a, b)
    batch.run(use_graph=False)
    ref = [[batch.results(i, k) for k in range(len(passes))] for i in range(len(sizes))]
    batch.set_schedule(og.BATCH_QUEUE)
    for tuning in ((0, 1), (2, 2)):
        for k in range(len(passes)):
            batch.set_tuning(k, *tuning)
        batch.run(use_graph=False)
        for i in range(len(sizes)):
            for k in range(len(passes)):
                for g, r, name in zip(batch.results(i, k), ref[i][k], ("vectors", "peaks", "displacements")):
                    assert np.array_equal(g, r, equal_nan=True), f"{tuning}: pair {i} pass {k} {name} differ"
    batch.close()
