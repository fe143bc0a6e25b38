"""The reference's per-piece files (src/main.cpp:444-452) written by the
library: the OpenCV FileStorage YAML matrix reads back exactly, and the PNG
decodes (stdlib zlib, checked CRCs) to the min..max 8-bit scaling of
OpenCVImageWriter (src/utilities.cpp:21-31).  Host code only."""
import re
import struct
import zlib

import numpy as np
import pytest


def _lib():
    import gpb
    return gpb._lib()


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(typ + body) & 0xffffffff == crc
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    W, H, depth, colour = ihdr[:4]
    assert depth == 8 and colour == 0
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(H, W + 1)
    assert not raw[:, 0].any()  # filter 0 on every row
    return raw[:, 1:]


@pytest.mark.parametrize("shape", [(5, 7), (300, 251)])
def test_png_minmax(tmp_path, shape):
    rng = np.random.default_rng(shape[0])
    a = rng.random(shape).astype(np.float32) * 3 - 1
    p = str(tmp_path / "x.png")
    assert _lib().gpb_write_png_minmax(p.encode(), a.ctypes.data, shape[0], shape[1]) == 0
    got = _read_png(p)
    d = a.astype(np.float64)
    mn, mx = d.min(), d.max()
    want = np.clip(np.rint(d * (255.0 / (mx - mn)) + (-mn * 255.0 / (mx - mn))), 0, 255).astype(np.uint8)
    assert np.array_equal(got, want)


def test_png_constant_plane(tmp_path):
    a = np.full((4, 6), 0.25, np.float32)
    p = str(tmp_path / "c.png")
    assert _lib().gpb_write_png_minmax(p.encode(), a.ctypes.data, 4, 6) == 0
    assert not _read_png(p).any()


def test_yml_reads_back_exactly(tmp_path):
    rng = np.random.default_rng(1)
    a = (rng.random((9, 13)) * 1e-3).astype(np.float32)
    p = str(tmp_path / "m.yml")
    assert _lib().gpb_write_yml(p.encode(), b"gpb_nonmax", a.ctypes.data, 9, 13) == 0
    txt = open(p).read()
    assert txt.startswith("%YAML:1.0\n---\ngpb_nonmax: !!opencv-matrix")
    assert re.search(r"rows: 9\s+cols: 13\s+dt: d", txt)
    vals = np.array([float(v) for v in re.search(r"data: \[(.*)\]", txt, re.S).group(1).split(",")])
    assert np.array_equal(vals.astype(np.float32).reshape(9, 13), a)


def test_yml_codebook_values(tmp_path):
    """A 13 x K matrix written as texton_codebook carries every value exactly
    (the GPU test loads it back through gpb_load_codebook_yml)."""
    cb = np.random.default_rng(2).random((13, 32)).astype(np.float32)
    p = str(tmp_path / "cb.yml")
    assert _lib().gpb_write_yml(p.encode(), b"texton_codebook", cb.ctypes.data, 13, 32) == 0
    txt = open(p).read()
    vals = np.array([float(v) for v in re.search(r"data: \[(.*)\]", txt, re.S).group(1).split(",")], np.float32)
    assert np.array_equal(vals.reshape(13, 32), cb)


def test_write_piece_files(tmp_path):
    import gpb
    nm = np.random.default_rng(3).random((20, 30)).astype(np.float32)
    ori = np.random.default_rng(4).random((8, 20, 30)).astype(np.float32)
    prefix = str(tmp_path / "piece_0_0")
    gpb.write_piece_files(prefix, nm, ori)
    for o in range(8):
        assert _read_png("%s_gpb_orient_%d.png" % (prefix, o)).shape == (20, 30)
    assert _read_png(prefix + "_gpb_nmax.png").shape == (20, 30)
    assert "gpb_nonmax" in open(prefix + "_gpb_nmax.yml").read()
