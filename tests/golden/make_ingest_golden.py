"""Generates the ingest fixtures: tests/golden/ingest/*.pnm (seeded images
written here) and tests/golden/ingest_ref.npz (those files decoded by the
reference's own PNM loader, loaders/pnm_image_loader.cpp:199-226, compiled
from its sources with ref_pnm_decode.cpp).

The files cover what the reference's loader reads: P5 8- and 16-bit
(16-bit samples big-endian; a maxval below 65535 is kept as is), P6 RGB
8- and 16-bit (grey = (218 r + 732 g + 74 b) >> 10, pixel_types.h:390-400),
comment lines after the magic number (the only place its header parser
skips them).  8-bit RGB samples stay below 128: the reference copies them
through `char`, whose signedness is the platform's (negative on x86-64 for
samples >= 128); the loader here reads them as unsigned bytes.

The reference's TIFF loader needs libtiff, which is not installed here, so
there is no reference-decoded TIFF fixture.

Run on a machine with the reference sources:  python tests/golden/make_ingest_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("OPENPIV_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "ingest")


def write_pnm(path, img, magic, maxval, comment="seeded test image"):
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(f"{magic}\n# {comment}\n{w} {h}\n{maxval}\n".encode())
        if maxval > 255:
            f.write(img.astype(">u2").tobytes())
        else:
            f.write(img.astype(np.uint8).tobytes())


def cases():
    rng = np.random.default_rng(20261204)
    yield "p5_u8", "P5", 255, rng.integers(0, 256, (23, 37))
    yield "p5_u16", "P5", 65535, rng.integers(0, 65536, (17, 29))
    yield "p5_u12", "P5", 4095, rng.integers(0, 4096, (16, 16))
    yield "p6_u16", "P6", 65535, rng.integers(0, 65536, (13, 21, 3))
    yield "p6_u8", "P6", 255, rng.integers(0, 128, (11, 19, 3))


def build_decoder(tmp):
    import torch

    ref = os.path.join(REFERENCE, "openpiv")
    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")   # fmt, header-only
    srcs = [os.path.join(HERE, "ref_pnm_decode.cpp")] + \
        [os.path.join(ref, "core", f) for f in ("size.cpp", "rect.cpp", "util.cpp")] + \
        [os.path.join(ref, "loaders", f) for f in ("image_loader.cpp", "pnm_image_loader.cpp")]
    exe = os.path.join(tmp, "ref_pnm_decode")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", ref, "-idirafter", torch_inc, "-DFMT_HEADER_ONLY",
                    "-D_USE_MATH_DEFINES", "-include", "cstring", *srcs, "-pthread", "-o", exe], check=True)
    return exe


def main() -> None:
    if not os.path.isdir(os.path.join(REFERENCE, "openpiv")):
        sys.exit("reference sources not found (set OPENPIV_REFERENCE)")
    os.makedirs(OUT_DIR, exist_ok=True)
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        exe = build_decoder(tmp)
        for name, magic, maxval, img in cases():
            path = os.path.join(OUT_DIR, f"{name}.pnm")
            write_pnm(path, img, magic, maxval)
            raw = os.path.join(tmp, name + ".raw")
            subprocess.run([exe, path, raw], check=True)
            data = np.fromfile(raw, np.uint8)
            w, h = np.frombuffer(data[:8].tobytes(), "<u4")
            arrays[name] = np.frombuffer(data[8:].tobytes(), "<u2").reshape(h, w)
    np.savez_compressed(os.path.join(HERE, "ingest_ref.npz"), **arrays)
    print("wrote", ", ".join(sorted(arrays)))


if __name__ == "__main__":
    main()
