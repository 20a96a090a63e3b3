"""Write the demo scene used by the scene-loading tests (tests/golden/scene_demo/).

A small scene in the reference's .scene format with its own meshes and textures, made
here from seeded procedural content (nothing is taken from the reference's resources). It
exercises what the loader has to get right: nested and array tokens, comments, commas;
a scene-wide transformation; OBJ files with and without texture coordinates and normals,
single-slash face tokens and a UV sphere with a seam and poles; PNG textures of several
colour types (RGB with every filter type, palette with tRNS alpha, grey + alpha, 16-bit,
interlaced), JPEG textures (sequential 4:2:0 with restart markers; progressive 4:4:4 with
spectral selection and DC successive approximation), constant-colour textures, an OpenEXR
cube map (uncompressed half, ZIP compressed, float RGBA faces); point, spot and directional lights; an object with
``skipuvs``; a masked material and an emissive one; a probe block.

    python tests/golden/scene_demo/make_scene.py
"""
from __future__ import annotations

import math
import os
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SEED = 20261204


# --------------------------------------------------------------------------------------
# image writers
# --------------------------------------------------------------------------------------


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _filter_row(row: np.ndarray, prior: np.ndarray, fb: int, ftype: int) -> np.ndarray:
    x = row.astype(np.int32)
    b = prior.astype(np.int32)
    a = np.concatenate([np.zeros(fb, np.int32), x[:-fb]]) if len(x) > fb else np.zeros_like(x)
    c = np.concatenate([np.zeros(fb, np.int32), b[:-fb]]) if len(b) > fb else np.zeros_like(b)
    if ftype == 0:
        pred = 0
    elif ftype == 1:
        pred = a
    elif ftype == 2:
        pred = b
    elif ftype == 3:
        pred = (a + b) >> 1
    else:
        p = a + b - c
        pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
        pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
    return ((x - pred) & 0xFF).astype(np.uint8)


def _pack_rows(samples: np.ndarray, depth: int) -> np.ndarray:
    """(h, w, ch) samples -> (h, row_bytes) packed big-endian bytes."""
    h, w, ch = samples.shape
    if depth == 8:
        return samples.reshape(h, w * ch).astype(np.uint8)
    if depth == 16:
        s = samples.reshape(h, w * ch).astype(np.uint16)
        return np.stack([(s >> 8).astype(np.uint8), (s & 0xFF).astype(np.uint8)], -1).reshape(h, -1)
    per = 8 // depth
    flat = samples.reshape(h, w).astype(np.uint8)
    pad = (-w) % per
    flat = np.concatenate([flat, np.zeros((h, pad), np.uint8)], 1)
    out = np.zeros((h, flat.shape[1] // per), np.uint8)
    for k in range(per):
        out |= (flat[:, k::per] << (8 - depth * (k + 1))).astype(np.uint8)
    return out


def write_png(path, samples, ctype, depth=8, palette=None, trns=None, interlace=False, filters=(0, 1, 2, 3, 4)):
    samples = np.asarray(samples)
    h, w, ch = samples.shape
    bpp_bits = ch * depth
    fb = max(1, bpp_bits // 8)

    def encode(sub):
        rows = _pack_rows(sub, depth)
        prior = np.zeros(rows.shape[1], np.uint8)
        out = bytearray()
        for y in range(rows.shape[0]):
            ft = filters[y % len(filters)]
            out.append(ft)
            out += _filter_row(rows[y], prior, fb, ft).tobytes()
            prior = rows[y]
        return bytes(out)

    if not interlace:
        raw = encode(samples)
    else:
        raw = b""
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            sub = samples[y0::dy, x0::dx]
            if sub.size:
                raw += encode(sub)
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        data += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        data += _chunk(b"tRNS", trns)
    z = zlib.compress(raw, 9)
    data += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def write_exr(path, img, ptype=1, compression=0):
    """Scanline OpenEXR: channels named from the image's component count, pixel type
    1 (half) or 2 (float), compression 0 (none) or 3 (ZIP, 16 lines per block)."""
    h, w, c = img.shape
    names = {3: ["B", "G", "R"], 4: ["A", "B", "G", "R"]}[c]
    src = {"R": 0, "G": 1, "B": 2, "A": 3}
    dt, sz = (np.float16, 2) if ptype == 1 else (np.float32, 4)

    def attr(name, kind, val):
        return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<I", len(val)) + val

    chl = b"".join(n.encode() + b"\0" + struct.pack("<i", ptype) + b"\0\0\0\0" + struct.pack("<ii", 1, 1)
                   for n in names) + b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    hdr = (b"\x76\x2f\x31\x01" + struct.pack("<I", 2) + attr("channels", "chlist", chl)
           + attr("compression", "compression", bytes([compression])) + attr("dataWindow", "box2i", box)
           + attr("displayWindow", "box2i", box) + attr("lineOrder", "lineOrder", b"\0")
           + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
           + attr("screenWindowCenter", "v2f", struct.pack("<ff", 0, 0))
           + attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    lines = 16 if compression == 3 else 1
    blocks = []
    for y0 in range(0, h, lines):
        raw = b"".join(img[y, :, src[n]].astype(dt).tobytes() for y in range(y0, min(h, y0 + lines)) for n in names)
        if compression == 3:
            t = np.frombuffer(raw, np.uint8)
            inter = np.concatenate([t[0::2], t[1::2]]).astype(np.int32)
            d = inter.copy()
            d[1:] = (inter[1:] - inter[:-1] + 128 + 256) & 0xFF
            raw = zlib.compress(d.astype(np.uint8).tobytes())
        blocks.append(struct.pack("<iI", y0, len(raw)) + raw)
    table = len(hdr) + 8 * len(blocks)
    offs, pos = [], table
    for b in blocks:
        offs.append(pos)
        pos += len(b)
    with open(path, "wb") as f:
        f.write(hdr + struct.pack(f"<{len(blocks)}Q", *offs) + b"".join(blocks))
    del sz


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value: int, length: int):
        for k in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> k) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


_ZZ = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14,
       21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53,
       60, 61, 54, 47, 55, 62, 63]


def _category(v: int) -> int:
    return int(abs(v)).bit_length()


def _bits_of(v: int, s: int) -> int:
    return v if v >= 0 else v + (1 << s) - 1


def _code_table(symbols):
    """Canonical code for a symbol set: the 16 most frequent symbols get 5-bit codes, the
    others 12-bit codes (exercises both short and long code paths of a decoder)."""
    freq = {}
    for sym in symbols:
        freq[sym] = freq.get(sym, 0) + 1
    order = sorted(freq, key=lambda s_: (-freq[s_], s_))
    short, long_ = order[:16], order[16:]
    counts = [0] * 17
    counts[5], counts[12] = len(short), len(long_)
    codes, code = {}, 0
    for length, group in ((5, short), (12, long_)):
        for sym in group:
            codes[sym] = (code, length)
            code += 1
        if length == 5:
            code <<= 7
    return counts, short + long_, codes


def write_jpeg(path, rgb, subsample=True, restart=0, progressive=False):
    """Huffman JPEG of an 8-bit RGB image: JFIF YCbCr, 4:2:0 (or 4:4:4), quality-75 style
    quantisation, a float forward DCT. Sequential (optionally with restart markers), or
    progressive with an interleaved DC scan at Al = 1, a DC refinement scan and per
    component AC scans by spectral selection (bands 1-5 and 6-63, one EOB per block)."""
    rgb = np.asarray(rgb, np.float64)
    h, w, _ = rgb.shape
    y = 0.299 * rgb[..., 0] + 0.587 * rgb[..., 1] + 0.114 * rgb[..., 2]
    cb = -0.168736 * rgb[..., 0] - 0.331264 * rgb[..., 1] + 0.5 * rgb[..., 2] + 128
    cr = 0.5 * rgb[..., 0] - 0.418688 * rgb[..., 1] - 0.081312 * rgb[..., 2] + 128
    hs = 2 if subsample else 1
    mw, mh = 8 * hs, 8 * hs
    W, H = -(-w // mw) * mw, -(-h // mh) * mh
    pad = lambda a: np.pad(a, ((0, H - h), (0, W - w)), mode="edge")  # noqa: E731
    planes = [pad(y)]
    for c in (cb, cr):
        c = pad(c)
        if subsample:
            c = c.reshape(H // 2, 2, W // 2, 2).mean((1, 3))
        planes.append(c)
    qy = np.array([8 + (k % 8 + k // 8) * 3 for k in range(64)], np.int32)
    qc = np.array([10 + (k % 8 + k // 8) * 4 for k in range(64)], np.int32)
    qts = [qy, qc, qc]
    xs = np.arange(8)
    basis = np.array([[(np.sqrt(0.125) if u == 0 else 0.5) * np.cos((2 * x + 1) * u * np.pi / 16) for x in xs]
                      for u in range(8)])
    blocks = []  # per component: (by, bx) -> quantised natural-order coefficients
    for ci, pl in enumerate(planes):
        bh, bw = pl.shape[0] // 8, pl.shape[1] // 8
        t = pl.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3) - 128.0
        f = np.einsum("ux,abxy,vy->abuv", basis, t, basis)
        blocks.append(np.round(f.reshape(bh, bw, 64) / qts[ci]).astype(np.int64))
    ids = (1, 2, 3)
    samp = (hs * 16 + hs, 0x11, 0x11)
    mcu_order = []  # (component, by, bx) in interleaved MCU order
    for my in range(H // mh):
        for mx in range(W // mw):
            for v in range(hs):
                for u in range(hs):
                    mcu_order.append((0, my * hs + v, mx * hs + u))
            mcu_order += [(1, my, mx), (2, my, mx)]

    def seg(marker, body):
        return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body

    def dht(tc, th, counts, vals):
        return seg(0xC4, bytes([tc * 16 + th]) + bytes(counts[1:]) + bytes(vals))

    out = bytearray(b"\xff\xd8")
    out += seg(0xE0, b"JFIF\0" + bytes([1, 1, 0, 0, 1, 0, 1, 0, 0]))
    for t, q in enumerate((qy, qc)):
        out += seg(0xDB, bytes([t]) + bytes(int(q[_ZZ[k]]) for k in range(64)))
    sof = 0xC2 if progressive else 0xC0
    out += seg(sof, bytes([8]) + struct.pack(">HH", h, w) + bytes([3]) +
               b"".join(bytes([ids[c], samp[c], 0 if c == 0 else 1]) for c in range(3)))
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))

    def dc_symbols(units, al):
        pred = [0, 0, 0]
        syms = []
        for c, by, bx in units:
            dcv = int(blocks[c][by, bx, 0]) >> al
            d = dcv - pred[c]
            pred[c] = dcv
            syms.append((c, _category(d), d))
        return syms

    def ac_symbols(coefs, ss, se):
        syms, run = [], 0
        last = max([k for k in range(ss, se + 1) if coefs[_ZZ[k]] != 0], default=-1)
        for k in range(ss, se + 1):
            if k > last:
                syms.append((0x00, 0, 0))
                break
            v = int(coefs[_ZZ[k]])
            if v == 0:
                run += 1
                continue
            while run > 15:
                syms.append((0xF0, 0, 0))
                run -= 16
            s_ = _category(v)
            syms.append((run * 16 + s_, s_, v))
            run = 0
        return syms

    if not progressive:
        per_unit = []
        for c, by, bx in mcu_order:
            per_unit.append((c, by, bx))
        # symbol statistics per table class
        dc_s = dc_symbols(per_unit, 0)
        ac_s = [ac_symbols(blocks[c][by, bx], 1, 63) for c, by, bx in per_unit]
        tables = {}
        for cls in (0, 1):
            comps = (0,) if cls == 0 else (1, 2)
            dsyms = [s_[1] for s_ in dc_s if s_[0] in comps]
            asyms = [a[0] for (c, _, _), syms in zip(per_unit, ac_s) if c in comps for a in syms]
            tables[cls] = (_code_table(dsyms), _code_table(asyms))
            out += dht(0, cls, tables[cls][0][0], tables[cls][0][1]) + dht(1, cls, tables[cls][1][0], tables[cls][1][1])
        out += seg(0xDA, bytes([3]) + b"".join(bytes([ids[c], 0 if c == 0 else 0x11]) for c in range(3)) +
                   bytes([0, 63, 0]))
        bw_ = _BitWriter()
        units_per_mcu = hs * hs + 2
        rst = 0
        for i, ((c, by, bx), d, syms) in enumerate(zip(per_unit, dc_s, ac_s)):
            if restart and i and i % (units_per_mcu * restart) == 0:
                bw_.flush()
                out += bw_.out + bytes([0xFF, 0xD0 + rst % 8])
                bw_ = _BitWriter()
                rst += 1
                # predictors restart: recompute the remaining DC differences
                dc_s[i:] = dc_symbols(per_unit[i:], 0)
                d = dc_s[i]
            cls = 0 if c == 0 else 1
            (_, _, dcodes), (_, _, acodes) = tables[cls]
            code, length = dcodes[d[1]]
            bw_.put(code, length)
            if d[1]:
                bw_.put(_bits_of(d[2], d[1]), d[1])
            for sym, s_, v in syms:
                code, length = acodes[sym]
                bw_.put(code, length)
                if s_:
                    bw_.put(_bits_of(v, s_), s_)
        bw_.flush()
        out += bw_.out
    else:
        # DC first (Al = 1), interleaved
        dc_s = dc_symbols(mcu_order, 1)
        for cls in (0, 1):
            comps = (0,) if cls == 0 else (1, 2)
            counts, vals, _ = _code_table([s_[1] for s_ in dc_s if s_[0] in comps])
            out += dht(0, cls, counts, vals)
        codes = {cls: _code_table([s_[1] for s_ in dc_s if s_[0] in ((0,) if cls == 0 else (1, 2))])[2]
                 for cls in (0, 1)}
        out += seg(0xDA, bytes([3]) + b"".join(bytes([ids[c], 0 if c == 0 else 0x10]) for c in range(3)) +
                   bytes([0, 0, 0x01]))
        bw_ = _BitWriter()
        for c, _, d in dc_s:
            code, length = codes[0 if c == 0 else 1][_category(d)]
            bw_.put(code, length)
            if _category(d):
                bw_.put(_bits_of(d, _category(d)), _category(d))
        bw_.flush()
        out += bw_.out
        # DC refinement (Ah = 1, Al = 0): the low bit of every DC value
        out += seg(0xDA, bytes([3]) + b"".join(bytes([ids[c], 0]) for c in range(3)) + bytes([0, 0, 0x10]))
        bw_ = _BitWriter()
        for c, by, bx in mcu_order:
            bw_.put(int(blocks[c][by, bx, 0]) & 1, 1)
        bw_.flush()
        out += bw_.out
        # AC first scans, one component each, bands 1-5 and 6-63 (non-interleaved order)
        for c in range(3):
            hc = hs if c == 0 else 1  # the component's sampling factor (hmax = vmax = hs)
            cw_ = -(-(-(-w * hc // hs)) // 8)  # blocks covering the component's own size
            ch_ = -(-(-(-h * hc // hs)) // 8)
            for ss, se in ((1, 5), (6, 63)):
                syms = [ac_symbols(blocks[c][by, bx], ss, se) for by in range(ch_) for bx in range(cw_)]
                counts, vals, acodes = _code_table([a[0] for sy in syms for a in sy])
                out += dht(1, 0, counts, vals)
                out += seg(0xDA, bytes([1, ids[c], 0x00, ss, se, 0]))
                bw_ = _BitWriter()
                for sy in syms:
                    for sym, s_, v in sy:
                        code, length = acodes[sym]
                        bw_.put(code, length)
                        if s_:
                            bw_.put(_bits_of(v, s_), s_)
                bw_.flush()
                out += bw_.out
    out += b"\xff\xd9"
    with open(path, "wb") as f:
        f.write(bytes(out))


# --------------------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------------------


def _fmt(x):
    return f"{x:.6f}"


def write_floor(path):
    lines = ["# floor quad with texture coordinates and one normal"]
    lines += [f"v {_fmt(x)} 0.000000 {_fmt(z)}" for x, z in ((-1, -1), (1, -1), (1, 1), (-1, 1))]
    lines += [f"vt {_fmt(u)} {_fmt(v)}" for u, v in ((0, 0), (2, 0), (2, 2), (0, 2))]
    lines += ["vn 0.000000 1.000000 0.000000", "f 1/1/1 3/3/1 2/2/1", "f 1/1/1 4/4/1 3/3/1"]
    open(path, "w").write("\n".join(lines) + "\n")


def write_crate(path):
    """A box with positions and faces only: normals are computed, texture coordinates are
    the constant ones; CRLF line endings."""
    lines = ["# crate"]
    for z in (-1, 1):
        for y in (-1, 1):
            for x in (-1, 1):
                lines.append(f"v {_fmt(x)} {_fmt(y)} {_fmt(z)}")
    quads = [(1, 3, 4, 2), (5, 6, 8, 7), (1, 2, 6, 5), (3, 7, 8, 4), (1, 5, 7, 3), (2, 4, 8, 6)]
    for a, b, c, d in quads:
        lines += [f"f {a} {b} {c}", f"f {a} {c} {d}"]
    open(path, "w", newline="").write("\r\n".join(lines) + "\r\n")


def write_ball(path, rings=8, segs=12, seed=SEED):
    """UV sphere: a texture seam at u = 0 / 1, one pole vertex per pole, radial noise."""
    rng = np.random.default_rng(seed)
    v, vt, vn, faces = [], [], [], []
    for i in range(rings + 1):
        th = math.pi * i / rings
        for j in range(segs + 1):
            ph = 2 * math.pi * j / segs
            n = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            r = 1.0 + (0.03 * rng.standard_normal() if 0 < i < rings and j < segs else 0.0)
            v.append(tuple(r * c for c in n))
            vn.append(n)
            vt.append((j / segs, 1 - i / rings))
    idx = lambda i, j: i * (segs + 1) + j + 1  # noqa: E731
    for i in range(rings):
        for j in range(segs):
            a, b, c, d = idx(i, j), idx(i, j + 1), idx(i + 1, j + 1), idx(i + 1, j)
            if i > 0:
                faces.append((a, b, c))
            if i < rings - 1:
                faces.append((a, c, d))
    lines = ["# ball"] + [f"v {_fmt(a)} {_fmt(b)} {_fmt(c)}" for a, b, c in v]
    lines += [f"vt {_fmt(a)} {_fmt(b)}" for a, b in vt] + [f"vn {_fmt(a)} {_fmt(b)} {_fmt(c)}" for a, b, c in vn]
    lines += ["s 1"] + ["f " + " ".join(f"{k}/{k}/{k}" for k in f) for f in faces]
    open(path, "w").write("\n".join(lines) + "\n")


def write_leaf(path):
    """A leaf card with texture coordinates but no normals, single-slash face tokens and an
    extra vertex on one face line (only the first three vertices of a face are read)."""
    lines = ["v -0.5 0.0 0.0", "v 0.5 0.0 0.0", "v 0.5 1.0 0.0", "v -0.5 1.0 0.0", "v 0.0 1.2 0.0",
             "vt 0 0", "vt 1 0", "vt 1 1", "vt 0 1", "vt 0.5 1",
             "g leaf", "f 1/1 2/2 3/3 5/5", "f 1/1 3/3 4/4"]
    open(path, "w").write("\n".join(lines) + "\n")


def write_lamp(path):
    lines = ["v -0.4 0.0 -0.4", "v 0.4 0.0 -0.4", "v 0.4 0.0 0.4", "v -0.4 0.0 0.4",
             "vn 0 -1 0", "f 1//1 2//1 3//1", "f 1//1 3//1 4//1"]
    open(path, "w").write("\n".join(lines) + "\n")


# --------------------------------------------------------------------------------------
# textures
# --------------------------------------------------------------------------------------


def write_textures(rng):
    n = 32
    yy, xx = np.mgrid[0:n, 0:n]
    check = ((xx // 8 + yy // 8) % 2).astype(np.float64)
    rgb = np.stack([60 + 150 * check, 70 + 120 * check + 20 * (yy / n), 90 + 60 * (1 - check)], -1)
    rgb = np.clip(rgb + rng.integers(-8, 9, rgb.shape), 0, 255).astype(np.uint8)
    write_png(os.path.join(HERE, "demo_checker.png"), rgb, ctype=2)
    # 16-bit normal map: gentle bumps
    nx = 0.25 * np.sin(xx / n * 2 * math.pi * 2)
    ny = 0.25 * np.cos(yy / n * 2 * math.pi * 3)
    nz = np.sqrt(1 - nx ** 2 - ny ** 2)
    nm = np.stack([nx, ny, nz], -1) * 0.5 + 0.5
    write_png(os.path.join(HERE, "demo_normal.png"), np.round(nm * 65535).astype(np.uint16), ctype=2, depth=16)
    # roughness / metalness / occlusion: grey + alpha (grey replicated to rgb), interlaced
    rough = np.stack([np.clip(40 + 6 * xx + rng.integers(0, 20, xx.shape), 0, 255),
                      np.full(xx.shape, 255)], -1).astype(np.uint8)
    write_png(os.path.join(HERE, "demo_rough.png"), rough, ctype=4, interlace=True)
    # palette leaf colour with transparent holes (tRNS), 4-bit indices
    pal = np.array([[40, 120, 30], [70, 160, 40], [110, 190, 60], [20, 60, 15], [200, 220, 80]], np.uint8)
    ind = rng.integers(0, 5, (24, 20)).astype(np.uint8)
    ind[(np.mgrid[0:24, 0:20][0] - 12) ** 2 + (np.mgrid[0:24, 0:20][1] - 10) ** 2 > 90] = 3
    write_png(os.path.join(HERE, "demo_leaf_color.png"), ind[..., None], ctype=3, depth=4, palette=pal,
              trns=bytes([255, 255, 255, 0, 255]))
    # JPEG colour textures: sequential 4:2:0 with restart markers, progressive 4:4:4
    wood = np.stack([120 + 60 * np.sin(xx * 0.7 + 2 * np.sin(yy * 0.2)), 80 + 30 * np.sin(xx * 0.7), 40 + 10 * yy / n],
                    -1)
    wood = np.clip(np.kron(wood, np.ones((2, 2, 1)))[:58, :46] + rng.integers(-6, 7, (58, 46, 3)), 0, 255)
    write_jpeg(os.path.join(HERE, "demo_crate_color.jpg"), wood.astype(np.uint8), subsample=True, restart=3)
    write_jpeg(os.path.join(HERE, "demo_wall_color.jpg"), rgb[:, :27], subsample=False, progressive=True)
    # sky cube map faces: +y bright, -y dark, sides a gradient; three encodings
    for k, suf in enumerate(("px", "nx", "ny", "py", "pz", "nz")):
        m = 8
        gy = np.linspace(0.0, 1.0, m)[:, None, None]
        base = {"py": (2.0, 2.2, 2.6), "ny": (0.1, 0.08, 0.05)}.get(suf, (0.6 + 0.1 * k, 0.7, 0.9))
        img = (np.asarray(base, np.float64) * (0.6 + 0.8 * gy) * np.ones((m, m, 1))).astype(np.float32)
        if suf == "pz":
            write_exr(os.path.join(HERE, f"demo_sky_{suf}.exr"), img, ptype=1, compression=3)
        elif suf == "nz":
            rgba = np.concatenate([img, np.ones((m, m, 1), np.float32)], -1)
            write_exr(os.path.join(HERE, f"demo_sky_{suf}.exr"), rgba, ptype=2)
        else:
            write_exr(os.path.join(HERE, f"demo_sky_{suf}.exr"), img)


SCENE = """# Demo scene of the scene-loading tests (generated by make_scene.py).
* scene:
\torientation: 0.0 1.0 0.0 0.3
\ttranslation: 0.0,-0.1,0.0

* probe:
\tposition: 0.0 1.0 0.0
\tsize: 3.0 3.0 3.0
\tfade: 0.1

* background:
\tcube: rgb32cube: demo_sky

* camera:
\tposition: 0.2 1.3 3.2
\tcenter: 0.0 0.55 0.0   # looking at the ball and the crate
\tup: 0.0 1.0 0.0
\tfov: 1.1
\tplanes: 0.01 50.0

* point:
\tintensity: 6.0 5.5 5.0
\tshadows: true
\tposition: 0.4 2.0 0.6
\tradius: 4.0

* spot:
\tintensity: 8.0, 8.0, 9.0
\tposition: -1.2 2.2 1.0
\tdirection: 0.5 -1.0 -0.3
\tcone: 0.8 1.2
\tshadows: false
\tradius: 6.0

* directional:
\tintensity: 0.6 0.6 0.5
\tdirection: -0.3 -1.0 -0.2
\tshadows: true

* object:
\tmesh: demo_lamp
\tmaterial: lamp_mat
\ttranslation: 0.0 2.3 0.0

* object:
\tmesh: demo_floor
\tmaterial: floor_mat
\tscaling: 3.0
\tshadows: true

* object:
\tmesh: demo_ball
\tmaterial: ball_mat
\ttranslation: -0.5 0.5 0.0
\tscaling: 0.5

* object:
\tmesh: demo_crate
\tmaterial: crate_mat
\ttranslation: 0.7 0.35 -0.3
\torientation: 0.0 1.0 0.0 0.6
\tscaling: 0.35
\tskipuvs: true

* object:
\tmesh: demo_leaf
\tmaterial: leaf_mat
\ttranslation: 0.1 0.3 -0.9

* material:
\ttype: Emissive
\tname: lamp_mat
\ttextures:
\t\t- rgb32: 4.0,3.6,3.0

* material:
\ttype: Regular
\tname: floor_mat
\ttextures:
\t\t- srgb: demo_checker
\t\t- rgb: demo_normal
\t\t- rgb: demo_rough

* material:
\ttype: Regular
\tname: ball_mat
\ttextures:
\t\t- srgb: 0.8 0.3 0.2
\t\t- rgb: demo_normal
\t\t- rgb: 0.3,1.0,1.0

* material:
\ttype: Regular
\tname: crate_mat
\ttwosided: false
\ttextures:
\t\t- srgb: demo_checker
\t\t- rgb: 0.5,0.5,1.0
\t\t- rgb: 0.6,0.0,1.0

* material:
\ttype: Regular
\tname: leaf_mat
\tmasked: true
\ttextures:
\t\t- srgb: demo_leaf_color
\t\t- rgb: demo_normal
\t\t- rgb: 0.7,0.0,1.0
"""


def main():
    rng = np.random.default_rng(SEED)
    write_floor(os.path.join(HERE, "demo_floor.obj"))
    write_crate(os.path.join(HERE, "demo_crate.obj"))
    write_ball(os.path.join(HERE, "demo_ball.obj"))
    write_leaf(os.path.join(HERE, "demo_leaf.obj"))
    write_lamp(os.path.join(HERE, "demo_lamp.obj"))
    write_textures(rng)
    with open(os.path.join(HERE, "demo.scene"), "w") as f:
        f.write(SCENE)


if __name__ == "__main__":
    main()
