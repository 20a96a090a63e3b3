"""Image decoding for scene textures: what Image::load does for the texture files a scene names
(src/engine/resources/Image.cpp:108-113 of kosua20/Rendu).

  * PNG (Image::loadLDR, Image.cpp:291-333, through stb_image): every colour type and bit
    depth, interlaced or not, expanded to the requested channel count the way stb_image
    does it (grey -> (g, g, g), missing alpha -> 255, 16-bit samples -> their high byte,
    low bit depths scaled to 0..255, palette and tRNS transparency), then each byte
    divided by 255 in single precision.
  * OpenEXR (Image::loadHDR, Image.cpp:335-420, through tinyexr): single-part scanline
    files, uncompressed, RLE, ZIPS or ZIP, half / float / uint channels; R, G, B, A taken
    by name, a missing colour channel is 0 and a missing alpha 1.

  * JPEG (Image::loadLDR through stb_image): sequential and progressive Huffman files with
    1 or 3 components, decoded by the native library (pt_jpeg_decode). Its inverse DCT,
    chroma upsampling and colour conversion are computed in the standard way rather than
    with stb_image's fixed-point approximations, so samples may differ from the
    reference's by a few units of 1/255.

``flip`` mirrors the rows, as the reference does for the faces of cube maps
(ResourcesManager.cpp:509). BMP and TGA files (also accepted by stb_image) are not decoded:
loading one raises ``ImageFormatError`` naming the file.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


class ImageFormatError(ValueError):
    """An image file this decoder does not read (unsupported format or corrupt data)."""


# --------------------------------------------------------------------------------------
# PNG
# --------------------------------------------------------------------------------------

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
# scale of a low-bit-depth grey sample to 0..255
_DEPTH_SCALE = {1: 0xFF, 2: 0x55, 4: 0x11, 8: 0x01}
# Adam7 passes: (x0, y0, dx, dy)
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _unfilter(raw: bytes, width: int, height: int, bpp_bits: int) -> np.ndarray:
    """Undo the PNG scanline filters of one (sub)image: (height, row_bytes) uint8. The
    byte-sequential part runs in the native library (pt_png_unfilter)."""
    from . import _lib as L

    row_bytes = (width * bpp_bits + 7) // 8
    need = height * (row_bytes + 1)
    if len(raw) < need:
        raise ImageFormatError("PNG image data is truncated")
    src = np.frombuffer(raw, np.uint8, count=need)
    out = np.empty((height, row_bytes), np.uint8)
    try:
        L.call("pt_png_unfilter", src.ctypes.data, height, row_bytes, max(1, bpp_bits // 8), out.ctypes.data)
    except L.RenduError as e:
        raise ImageFormatError(str(e)) from None
    return out


def _samples(rows: np.ndarray, width: int, channels: int, depth: int) -> np.ndarray:
    """Unpack filtered rows into (h, w, channels) samples (uint16 for depth 16)."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, : width * channels].reshape(h, width, channels)
    if depth == 16:
        v = rows[:, : width * channels * 2].reshape(h, width * channels, 2).astype(np.uint16)
        return ((v[..., 0] << 8) | v[..., 1]).reshape(h, width, channels)
    # 1, 2 or 4 bits: one channel (grey or palette index), most significant bits first
    per = 8 // depth
    bits = np.zeros((h, rows.shape[1] * per), np.uint8)
    for k in range(per):
        bits[:, k::per] = (rows >> (8 - depth * (k + 1))) & ((1 << depth) - 1)
    return bits[:, :width].reshape(h, width, 1)


def decode_png(data: bytes, channels: int = 4, flip: bool = False) -> np.ndarray:
    """PNG bytes -> (h, w, channels) float32 in [0, 1], as stb_image + Image::loadLDR."""
    if data[:8] != _PNG_SIG:
        raise ImageFormatError("not a PNG file")
    pos, idat = 8, []
    ihdr = plte = trns = None
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body[:13])
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    if ihdr is None or not idat:
        raise ImageFormatError("PNG without IHDR or image data")
    width, height, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _PNG_CHANNELS or comp != 0 or filt != 0 or interlace > 1 or width == 0 or height == 0:
        raise ImageFormatError("unsupported PNG header")
    if depth not in ((1, 2, 4, 8, 16) if ctype in (0, 3) else (8, 16)) or (ctype == 3 and depth == 16):
        raise ImageFormatError("unsupported PNG bit depth")
    if ctype == 3 and plte is None:
        raise ImageFormatError("palette PNG without PLTE")
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise ImageFormatError(f"corrupt PNG image data: {e}") from None
    nch = _PNG_CHANNELS[ctype]
    bpp_bits = nch * depth
    if interlace == 0:
        img = _samples(_unfilter(raw, width, height, bpp_bits), width, nch, depth)
    else:
        img = np.zeros((height, width, nch), np.uint16 if depth == 16 else np.uint8)
        off = 0
        for x0, y0, dx, dy in _ADAM7:
            pw = (width - x0 + dx - 1) // dx if width > x0 else 0
            ph = (height - y0 + dy - 1) // dy if height > y0 else 0
            if pw == 0 or ph == 0:
                continue
            size = ph * ((pw * bpp_bits + 7) // 8 + 1)
            sub = _samples(_unfilter(raw[off:off + size], pw, ph, bpp_bits), pw, nch, depth)
            img[y0::dy, x0::dx][:ph, :pw] = sub
            off += size

    # to 8-bit RGBA-like samples with stb_image's rules
    alpha = None
    if ctype == 3:
        idx = img[..., 0].astype(np.int64)
        if idx.max(initial=0) >= len(plte):
            raise ImageFormatError("PNG palette index out of range")
        pal_a = np.full(len(plte), 255, np.uint8)
        if trns is not None:
            t = np.frombuffer(trns, np.uint8)[: len(plte)]
            pal_a[: len(t)] = t
        rgb = plte[idx]
        alpha = pal_a[idx]
        base = rgb
    else:
        key = None
        if trns is not None and ctype in (0, 2):
            vals = struct.unpack(">" + "H" * (len(trns) // 2), trns[: 2 * (len(trns) // 2)])
            key = np.array(vals[:nch], np.int64)
            if depth < 8:
                key = (key & 0xFF) * _DEPTH_SCALE[depth]
        if depth == 16:
            if key is not None:
                alpha = np.where((img.astype(np.int64) == key).all(-1), 0, 255).astype(np.uint8)
            s8 = (img >> 8).astype(np.uint8)
        else:
            s8 = img.astype(np.uint8)
            if depth < 8:
                s8 = (s8.astype(np.int32) * _DEPTH_SCALE[depth]).astype(np.uint8)
            if key is not None:
                alpha = np.where((s8.astype(np.int64) == key).all(-1), 0, 255).astype(np.uint8)
        if ctype in (4, 6):
            alpha = s8[..., -1]
            base = s8[..., :-1]
        else:
            base = s8
    if base.shape[-1] == 1:
        grey = base[..., 0]
        rgb = np.stack([grey, grey, grey], -1)
    else:
        rgb = base
        # stb_image's luminance for colour images converted to grey: (77 r + 150 g + 29 b) >> 8
        r16 = rgb.astype(np.int32)
        grey = ((r16[..., 0] * 77 + r16[..., 1] * 150 + r16[..., 2] * 29) >> 8).astype(np.uint8)
    a = alpha if alpha is not None else np.full(rgb.shape[:2], 255, np.uint8)
    if channels == 1:
        out = grey[..., None]
    elif channels == 2:
        out = np.stack([grey, a], -1)
    else:
        out = np.concatenate([rgb, a[..., None]], -1)
    out = np.ascontiguousarray(out[:, :, :channels])
    if flip:
        out = out[::-1]
    return out.astype(np.float32) / np.float32(255.0)


# --------------------------------------------------------------------------------------
# OpenEXR
# --------------------------------------------------------------------------------------

_EXR_MAGIC = b"\x76\x2f\x31\x01"
_EXR_LINES = {0: 1, 1: 1, 2: 1, 3: 16}
_EXR_TYPES = {0: (np.uint32, 4), 1: (np.float16, 2), 2: (np.float32, 4)}


def _exr_undo_zip(raw: bytes) -> bytes:
    t = np.frombuffer(raw, np.uint8).astype(np.int32)
    # predictor: running sum of (delta - 128), modulo 256
    if len(t):
        d = t.copy()
        d[1:] -= 128
        t = (np.cumsum(d) & 0xFF).astype(np.uint8)
    else:
        t = t.astype(np.uint8)
    half = (len(t) + 1) // 2
    out = np.empty(len(t), np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def _exr_undo_rle(raw: bytes, expect: int) -> bytes:
    """OpenEXR RLE: a signed count byte, then -count literal bytes or one byte repeated
    count + 1 times; the result then goes through the same predictor and interleave as ZIP."""
    out = bytearray()
    i = 0
    while i < len(raw) and len(out) < expect:
        c = struct.unpack("b", raw[i:i + 1])[0]
        i += 1
        if c < 0:
            out += raw[i:i - c]
            i -= c
        else:
            out += raw[i:i + 1] * (c + 1)
            i += 1
    return _exr_undo_zip(bytes(out))


def decode_exr(data: bytes, channels: int = 3, flip: bool = False) -> np.ndarray:
    """OpenEXR bytes -> (h, w, channels) float32, channels taken as R, G, B, A by name."""
    if data[:4] != _EXR_MAGIC:
        raise ImageFormatError("not an OpenEXR file")
    version = struct.unpack("<I", data[4:8])[0]
    if version & 0x200 or version & 0x800 or version & 0x1000:
        raise ImageFormatError("tiled, deep or multi-part OpenEXR files are not supported")
    pos = 8
    chans, comp, win = [], 0, None
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode("latin-1")
        e2 = data.index(b"\0", e + 1)
        size = struct.unpack("<I", data[e2 + 1:e2 + 5])[0]
        val = data[e2 + 5:e2 + 5 + size]
        if name == "channels":
            q = 0
            while val[q] != 0:
                z = val.index(b"\0", q)
                ptype = struct.unpack("<i", val[z + 1:z + 5])[0]
                xs, ys = struct.unpack("<ii", val[z + 9:z + 17])
                if ptype not in _EXR_TYPES or xs != 1 or ys != 1:
                    raise ImageFormatError("unsupported OpenEXR channel type or subsampling")
                chans.append((val[q:z].decode("latin-1"), ptype))
                q = z + 17
        elif name == "compression":
            comp = val[0]
        elif name == "dataWindow":
            win = struct.unpack("<iiii", val)
        pos = e2 + 5 + size
    pos += 1
    if comp not in _EXR_LINES:
        raise ImageFormatError(f"OpenEXR compression {comp} is not supported (none, RLE, ZIPS, ZIP are)")
    if win is None or not chans:
        raise ImageFormatError("OpenEXR header without dataWindow or channels")
    w, h = win[2] - win[0] + 1, win[3] - win[1] + 1
    lines = _EXR_LINES[comp]
    nblocks = (h + lines - 1) // lines
    offsets = struct.unpack(f"<{nblocks}Q", data[pos:pos + 8 * nblocks])
    planes = {name: np.zeros((h, w), np.float32) for name, _ in chans}
    line_bytes = sum(_EXR_TYPES[t][1] for _, t in chans) * w
    for off in offsets:
        y, size = struct.unpack("<iI", data[off:off + 8])
        y0 = y - win[1]
        nl = min(lines, h - y0)
        raw = data[off + 8:off + 8 + size]
        expect = nl * line_bytes
        if len(raw) < expect:
            if comp == 1:
                raw = _exr_undo_rle(raw, expect)
            elif comp in (2, 3):
                raw = _exr_undo_zip(zlib.decompress(raw))
            else:
                raise ImageFormatError("OpenEXR block is truncated")
        q = 0
        for k in range(nl):
            for name, t in chans:
                dt, sz = _EXR_TYPES[t]
                planes[name][y0 + k] = np.frombuffer(raw, dt, count=w, offset=q).astype(np.float32)
                q += sz * w
    out = np.zeros((h, w, channels), np.float32)
    for c, name in enumerate("RGBA"[:channels]):
        if name in planes:
            out[..., c] = planes[name]
        elif name == "A":
            out[..., c] = 1.0
    if flip:
        out = out[::-1]
    return np.ascontiguousarray(out)


def decode_jpeg(data: bytes, channels: int = 4, flip: bool = False) -> np.ndarray:
    """JPEG bytes -> (h, w, channels) float32 in [0, 1] (native decoder, pt_jpeg_decode)."""
    import ctypes as C

    from . import _lib as L

    w, h = C.c_uint32(), C.c_uint32()
    src = np.frombuffer(data, np.uint8)
    try:
        L.call("pt_jpeg_decode", src.ctypes.data, len(src), channels, None, 0, C.byref(w), C.byref(h))
        out = np.empty((h.value, w.value, channels), np.uint8)
        L.call("pt_jpeg_decode", src.ctypes.data, len(src), channels, out.ctypes.data, out.size, C.byref(w),
               C.byref(h))
    except L.RenduError as e:
        raise ImageFormatError(str(e)) from None
    if flip:
        out = out[::-1]
    return np.ascontiguousarray(out).astype(np.float32) / np.float32(255.0)


def load_image(path: str, channels: int = 4, flip: bool = False) -> np.ndarray:
    """Image::load(path, channels, flip): (h, w, channels) float32 from a PNG or EXR file.
    A channel count of 0 means the reference's defaults: 4 for 8-bit files, 3 for EXR."""
    with open(path, "rb") as f:
        data = f.read()
    if path.endswith(".exr"):  # Image::isFloat (Image.cpp:122-124)
        return decode_exr(data, channels or 3, flip)
    if data[:8] == _PNG_SIG:
        return decode_png(data, channels or 4, flip)
    if data[:2] == b"\xff\xd8":
        try:
            return decode_jpeg(data, channels or 4, flip)
        except ImageFormatError as e:
            raise ImageFormatError(f"{path}: {e}") from None
    raise ImageFormatError(f"{path}: only PNG, JPEG and OpenEXR images are decoded (BMP and TGA are not)")
