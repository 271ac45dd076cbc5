"""Generates the golden fixtures under tests/golden/.

* reference_kats.json -- the known answers the reference's own tests assert
  for this path, transcribed with their file:line (grid origins, peak order,
  swap_quadrants sums, FFT spike positions, error messages).
* ref_outputs.npz -- outputs of the reference itself (compiled from its own
  sources by oracle/Makefile, target "ref") on small seeded inputs: grids,
  correlation planes, and whole-pass vectors / peaks for both correlation
  modes, with and without the limited peak search.

Run on a machine that has the reference sources (they do not travel to the
GPU host; the fixtures do):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "openpiv-cxx_gb300"))

from oracle import oracle  # noqa: E402
from opiv_gb300 import synth  # noqa: E402

KATS = {
    "source": "openpiv-cxx tests (Catch2 suites); values transcribed, lines cited",
    "grid": [
        # tests/grid_test.cpp:57-71  generate_cartesian_grid({100, 50}, {32, 32}, 0.5)
        {"cite": "tests/grid_test.cpp:57-71", "image": [100, 50], "ia": [32, 32], "frac": 0.5,
         "origins": [[2, 1], [18, 1], [34, 1], [50, 1], [66, 1],
                     [2, 17], [18, 17], [34, 17], [50, 17], [66, 17]]},
        {"cite": "tests/grid_test.cpp:73-83", "image": [32, 32], "ia": [32, 32], "frac": 0.5,
         "origins": [[0, 0]]},
        {"cite": "tests/grid_test.cpp:85-100", "image": [64, 64], "ia": [32, 32], "frac": 0.5,
         "origins": [[0, 0], [16, 0], [32, 0], [0, 16], [16, 16], [32, 16],
                     [0, 32], [16, 32], [32, 32]]},
        {"cite": "tests/grid_test.cpp:102-119", "image": [64, 64], "ia": [32, 32], "frac": 0.25,
         "origins": [[x, y] for y in (0, 8, 16, 24, 32) for x in (0, 8, 16, 24, 32)]},
        {"cite": "tests/grid_test.cpp:121-136", "image": [65, 65], "ia": [32, 32], "frac": 0.5,
         "origins": [[0, 0], [16, 0], [32, 0], [0, 16], [16, 16], [32, 16],
                     [0, 32], [16, 32], [32, 32]]},
        {"cite": "tests/grid_test.cpp:138-153", "image": [66, 66], "ia": [32, 32], "frac": 0.5,
         "origins": [[1, 1], [17, 1], [33, 1], [1, 17], [17, 17], [33, 17],
                     [1, 33], [17, 33], [33, 33]]},
        {"cite": "tests/grid_test.cpp:155-170", "image": [64, 64], "ia": [32, 32], "offsets": [16, 16],
         "origins": [[0, 0], [16, 0], [32, 0], [0, 16], [16, 16], [32, 16],
                     [0, 32], [16, 32], [32, 32]]},
        {"cite": "tests/grid_test.cpp:172-189", "image": [64, 64], "ia": [32, 32], "offsets": [16, 8],
         "origins": [[x, y] for y in (0, 8, 16, 24, 32) for x in (0, 16, 32)]},
        {"cite": "tests/grid_test.cpp:191-216", "image": [64, 64], "ia": [32, 16], "offsets": [16, 8],
         "origins": [[x, y] for y in (0, 8, 16, 24, 32, 40, 48) for x in (0, 16, 32)]},
    ],
    "peaks": [
        # tests/image_utils_test.cpp:246-267: 100x100 zeros with spikes; top 3
        {"cite": "tests/image_utils_test.cpp:246-267", "size": [100, 100],
         "spikes": [[20, 20, 20.0], [30, 30, 30.0], [40, 40, 40.0], [50, 50, 50.0]],
         "num": 3, "centres": [[50, 50], [40, 40], [30, 30]], "values": [50.0, 40.0, 30.0]},
        # tests/image_utils_test.cpp:307-314: zero image -> no peaks
        {"cite": "tests/image_utils_test.cpp:307-314", "size": [100, 100], "spikes": [],
         "num": 3, "centres": [], "values": []},
    ],
    "swap_quadrants": {
        # tests/image_utils_test.cpp:208-244: quadrant sums 1,2,4,8 -> 8,4,2,1
        "cite": "tests/image_utils_test.cpp:208-244", "size": [100, 100],
        "before": [1, 2, 4, 8], "after": [8, 4, 2, 1]},
    "fft": {
        # tests/image_algos_test.cpp:23-62: 256^2, 128 sin(2 pi w/8 + 2 pi h/8);
        # spectrum non-zero only at (32,32) and (224,224), |X|^2 < 1e-9 elsewhere
        "cite_transform": "tests/image_algos_test.cpp:23-62",
        "size": 256, "spikes": [[32, 32], [224, 224]], "tol_abs_sqr": 1e-9,
        # tests/image_algos_test.cpp:64-109: transform_real of a (as above) and
        # b = 128 sin(2 pi (W-w)/8 + 2 pi h/8)
        "cite_transform_real": "tests/image_algos_test.cpp:64-109",
        "spikes_a": [[32, 32], [224, 224]], "spikes_b": [[32, 224], [224, 32]],
    },
    "errors": [
        {"cite": "tests/image_algos_test.cpp:111-120", "what": "size mismatch",
         "message": "image size is different"},
        {"cite": "tests/image_algos_test.cpp:122-130", "what": "non-power-of-two FFT",
         "sizes": [[512, 400], [400, 512]], "message": "power of 2"},
    ],
}


def fixture_pairs():
    """Small seeded pairs: (name, frame_a, frame_b, ia, step)."""
    out = []
    a, b = synth.particle_pair(96, 128, ppp=0.02, i0_range=(150, 255), noise=3.0,
                               displacement=lambda x, y: (np.full_like(x, 2.35), np.full_like(y, -1.70)),
                               dtype=np.uint8, seed=synth.SEED_BASE + 1000 * 1 + 99)
    out.append(("u8_w32", a, b, 32, 16))
    a, b = synth.particle_pair(112, 104, ppp=0.03, i0_range=(1500, 4000), noise=20.0,
                               displacement=synth.config2_field, dtype=np.uint16,
                               seed=synth.SEED_BASE + 1000 * 2 + 99, full_scale=4095.0)
    out.append(("u16_w32", a, b, 32, 8))
    out.append(("u16_w16", a, b, 16, 4))
    return out


def main() -> None:
    ref = oracle.get("ref")
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(KATS, f, indent=1)
    arrays = {}
    for name, a, b, ia, step in fixture_pairs():
        h, w = a.shape
        grid = ref.grid_offsets(w, h, ia, ia, step, step)
        arrays[f"{name}/a"] = a
        arrays[f"{name}/b"] = b
        arrays[f"{name}/grid"] = grid
        arrays[f"{name}/meta"] = np.array([ia, step], np.int32)
        fa, fb = a.astype(np.float64), b.astype(np.float64)
        sel = np.linspace(0, len(grid) - 1, 6).astype(int)
        for mode, mname in ((0, "real"), (1, "complex")):
            arrays[f"{name}/planes_{mname}"] = ref.correlate_windows(fa, fb, grid[sel], ia, mode)
            arrays[f"{name}/planes_sel"] = sel
            for limit in (0, 1):
                vec, pk, _ = ref.process_windows(fa, fb, grid, ia, mode, limit, 1)
                arrays[f"{name}/vec_{mname}_{limit}"] = vec
                arrays[f"{name}/peak_{mname}_{limit}"] = pk
    np.savez_compressed(os.path.join(HERE, "ref_outputs.npz"), **arrays)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
