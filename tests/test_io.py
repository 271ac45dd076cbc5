"""Image ingest (PNM / uncompressed TIFF, as the reference's loaders read them)
and the "x, y, u, v, sn" vector output, host-only."""
import os
import struct

import numpy as np
import pytest

import opiv_gb300 as og

REF_DATA = os.path.join(os.environ.get("OPENPIV_REFERENCE", "/root/reference"), "examples")


def write_pnm(path, img, rgb=False):
    h, w = img.shape[:2]
    maxval = 65535 if img.dtype == np.uint16 else 255
    with open(path, "wb") as f:
        f.write(f"P{6 if rgb else 5}\n# written by the test\n{w} {h}\n{maxval}\n".encode())
        f.write(img.astype(">u2" if maxval > 255 else np.uint8).tobytes())


def write_tiff(path, img, big_endian=False, rows_per_strip=None, compression=1):
    """Minimal baseline TIFF writer (chunky, uncompressed unless told)."""
    e = ">" if big_endian else "<"
    h, w = img.shape[:2]
    spp = 1 if img.ndim == 2 else img.shape[2]
    bps = 16 if img.dtype == np.uint16 else 8
    data = img.astype(e + ("u2" if bps == 16 else "u1")).tobytes()
    rps = rows_per_strip or h
    row_bytes = w * spp * bps // 8
    strips = [data[y * row_bytes:min(h, y + rps) * row_bytes] for y in range(0, h, rps)]
    offsets, pos = [], 8
    for s in strips:
        offsets.append(pos)
        pos += len(s)
    extra = b""
    entries = []

    def entry(tag, typ, vals):
        nonlocal extra
        size = 2 if typ == 3 else 4
        fmt = e + ("H" if typ == 3 else "I") * len(vals)
        raw = struct.pack(fmt, *vals)
        if len(raw) <= 4:
            entries.append(struct.pack(e + "HHI", tag, typ, len(vals)) + raw.ljust(4, b"\0"))
        else:
            off = pos_extra[0] + len(extra)
            extra += raw
            entries.append(struct.pack(e + "HHII", tag, typ, len(vals), off))

    ifd_pos = pos
    n_tags = 10
    pos_extra = [ifd_pos + 2 + 12 * n_tags + 4]
    entry(256, 4, [w])
    entry(257, 4, [h])
    entry(258, 3, [bps] * spp)
    entry(259, 3, [compression])
    entry(262, 3, [2 if spp == 3 else 1])
    entry(273, 4, offsets)
    entry(277, 3, [spp])
    entry(278, 4, [rps])
    entry(279, 4, [len(s) for s in strips])
    entry(284, 3, [1])
    with open(path, "wb") as f:
        f.write((b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, ifd_pos))
        for s in strips:
            f.write(s)
        f.write(struct.pack(e + "H", n_tags) + b"".join(entries) + struct.pack(e + "I", 0) + extra)


def grey(rgb):
    r, g, b = (rgb[..., c].astype(np.uint64) for c in range(3))
    return ((r * 218 + g * 732 + b * 74) >> 10)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_pgm_roundtrip(lib, tmp_path, dtype):
    rng = np.random.default_rng(1)
    img = rng.integers(0, np.iinfo(dtype).max + 1, (37, 53)).astype(dtype)
    p = str(tmp_path / "a.pgm")
    write_pnm(p, img)
    got = og.load_image(p)
    assert got.dtype == dtype and np.array_equal(got, img)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_ppm_rgb_to_grey(lib, tmp_path, dtype):
    rng = np.random.default_rng(2)
    img = rng.integers(0, np.iinfo(dtype).max + 1, (9, 11, 3)).astype(dtype)
    p = str(tmp_path / "a.ppm")
    write_pnm(p, img, rgb=True)
    assert np.array_equal(og.load_image(p), grey(img).astype(dtype))


@pytest.mark.parametrize("big_endian", [False, True])
@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("rps", [None, 7])
def test_tiff_roundtrip(lib, tmp_path, big_endian, dtype, rps):
    rng = np.random.default_rng(3)
    img = rng.integers(0, np.iinfo(dtype).max + 1, (29, 41)).astype(dtype)
    p = str(tmp_path / "a.tif")
    write_tiff(p, img, big_endian=big_endian, rows_per_strip=rps)
    got = og.load_image(p)
    assert got.dtype == dtype and np.array_equal(got, img)


def test_tiff_rgb_and_errors(lib, tmp_path):
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (8, 10, 3)).astype(np.uint8)
    p = str(tmp_path / "rgb.tif")
    write_tiff(p, img)
    assert np.array_equal(og.load_image(p), grey(img).astype(np.uint8))
    q = str(tmp_path / "deflate.tif")
    write_tiff(q, img[..., 0], compression=8)
    with pytest.raises(og.OpivError) as e:
        og.load_image(q)
    assert e.value.status == og.ERR_UNSUPPORTED and "compression" in e.value.message
    with pytest.raises(og.OpivError) as e:
        og.load_image(str(tmp_path / "missing.pgm"))
    assert "failed to open" in e.value.message


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="reference data not on this machine")
def test_reference_example_images(lib):
    a = og.load_image(os.path.join(REF_DATA, "process", "piv1.pgm"))
    assert a.shape == (1024, 1024) and a.dtype == np.uint8
    t = og.load_image(os.path.join(REF_DATA, "data", "test1", "exp1_001_a.tiff"))
    assert t.ndim == 2 and t.size > 0 and t.max() > 0


def test_vectors_write_format(lib, tmp_path):
    v = np.array([[16, 1008, -2.3512345, 1.7, 1.2345678],
                  [0, 0, 0, 0, 0],
                  [48, 1008, np.nan, -0.25, 10.5]], np.float32)
    p = str(tmp_path / "v.txt")
    og.write_vectors(p, v)
    lines = open(p).read().splitlines()
    assert lines[0] == "16, 1008, -2.35123, 1.7, 1.23457"
    assert lines[1] == "0, 0, 0, 0, 0"
    assert lines[2] == "48, 1008, nan, -0.25, 10.5"


INGEST = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ingest")


@pytest.mark.parametrize("name", ["p5_u8", "p5_u16", "p5_u12", "p6_u16", "p6_u8"])
def test_pnm_equals_reference_loader(lib, name):
    """opiv_image_load on seeded PNM files against the same files decoded by
    the reference's own loader (loaders/pnm_image_loader.cpp:199-226,
    compiled from its sources by tests/golden/make_ingest_golden.py): the
    16-bit grey samples it hands to the app, value for value."""
    ref = np.load(os.path.join(os.path.dirname(INGEST), "ingest_ref.npz"))[name]
    got = og.load_image(os.path.join(INGEST, f"{name}.pnm"))
    assert got.shape == ref.shape
    assert np.array_equal(got.astype(np.uint16), ref)
