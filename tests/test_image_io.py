"""Image output of the command-line render (pt_image_save): the PNG bytes equal those the
reference's own Image::save writes with renderOneShot's options (tests/golden/image_io.npz,
made by tests/golden/make_golden.py --image), the tone map is main.cpp's 1 - exp(-c), and
the EXR holds the half-precision image and is read back by the reference's own loader.
Host code only: runs without a GPU."""
import os
import struct
import zlib

import numpy as np
import pytest

from conftest import load_golden


def _lib():
    from rendu_gb300 import build

    build.build()
    from rendu_gb300 import pathtracer as P

    return P


def read_png(path):
    """Minimal reader for the PNGs pt_image_save writes (8-bit RGB/RGBA, filter 0)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h, ch = 8, b"", None, None, 3
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert zlib.crc32(data[pos + 4:pos + 8 + n]) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            ch = 4 if ctype == 6 else 3
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * ch)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, ch)


def read_exr(path):
    """Minimal reader for the uncompressed scanline EXRs pt_image_save writes."""
    d = open(path, "rb").read()
    assert d[:4] == b"\x76\x2f\x31\x01"
    pos, chans, win = 8, [], None
    while d[pos] != 0:
        e = d.index(b"\0", pos)
        name = d[pos:e].decode()
        e2 = d.index(b"\0", e + 1)
        size = struct.unpack("<I", d[e2 + 1:e2 + 5])[0]
        val = d[e2 + 5:e2 + 5 + size]
        if name == "channels":
            q = 0
            while val[q] != 0:
                z = val.index(b"\0", q)
                chans.append(val[q:z].decode())
                q = z + 1 + 16
        elif name == "compression":
            assert val[0] == 0
        elif name == "dataWindow":
            win = struct.unpack("<iiii", val)
        pos = e2 + 5 + size
    pos += 1
    w, h = win[2] - win[0] + 1, win[3] - win[1] + 1
    offs = struct.unpack(f"<{h}Q", d[pos:pos + 8 * h])
    out = {c: np.zeros((h, w), np.float16) for c in chans}
    for y, o in enumerate(offs):
        yy, size = struct.unpack("<iI", d[o:o + 8])
        row = np.frombuffer(d[o + 8:o + 8 + size], np.float16).reshape(len(chans), w)
        for k, c in enumerate(chans):
            out[c][yy] = row[k]
    return out


def test_png_bytes_equal_the_reference(tmp_path):
    P = _lib()
    g = load_golden("image_io.npz")
    path = str(tmp_path / "out.png")
    P.save_image(g["image"], path, tonemap=False)
    np.testing.assert_array_equal(read_png(path), g["ldr"])


def test_png_tone_map_is_one_minus_exp(tmp_path):
    P = _lib()
    rng = np.random.default_rng(3)
    hdr = rng.exponential(1.0, (20, 30, 3)).astype(np.float32)
    path = str(tmp_path / "t.png")
    P.save_image(hdr, path, tonemap=True)
    mapped = (1.0 - np.exp(-hdr)).astype(np.float32)
    expect = np.clip(255.0 * np.power(mapped, np.float32(1.0 / 2.2)), 0, 255).astype(np.uint8)
    diff = np.abs(read_png(path).astype(int) - expect)
    assert diff.max() <= 1 and (diff > 0).mean() < 0.005


def test_exr_holds_half_precision_image(tmp_path):
    P = _lib()
    rng = np.random.default_rng(4)
    img = (rng.exponential(2.0, (18, 21, 3)) * rng.choice([1, 100], (18, 21, 1))).astype(np.float32)
    path = str(tmp_path / "out.exr")
    P.save_image(img, path)
    ch = read_exr(path)
    assert sorted(ch) == ["B", "G", "R"]
    got = np.stack([ch["R"], ch["G"], ch["B"]], -1).astype(np.float32)
    np.testing.assert_array_equal(got, img.astype(np.float16).astype(np.float32))
    from oracle import oracle as O

    if O.ref_available():  # the reference's own loader reads it the same way
        np.testing.assert_array_equal(O.ref_load_image(path, 3), got)


def test_image_save_rejects_bad_arguments(tmp_path):
    from rendu_gb300 import RenduError

    P = _lib()
    with pytest.raises(RenduError, match="16 x 16"):
        P.save_image(np.zeros((8, 8, 3), np.float32), str(tmp_path / "small.exr"))
    with pytest.raises(RenduError, match="RGB"):
        P.save_image(np.zeros((8, 8, 1), np.float32), str(tmp_path / "gray.png"))
    with pytest.raises(RenduError, match="cannot open"):
        P.save_image(np.zeros((8, 8, 3), np.float32), os.path.join(str(tmp_path), "missing", "x.png"))
