"""Write the demo scene used by the scene-loading tests (tests/golden/scene_demo/).

A small scene in the reference's .scene format with its own meshes and textures, made
here from seeded procedural content (nothing is taken from the reference's resources). It
exercises what the loader has to get right: nested and array tokens, comments, commas;
a scene-wide transformation; OBJ files with and without texture coordinates and normals,
single-slash face tokens and a UV sphere with a seam and poles; PNG textures of several
colour types (RGB with every filter type, palette with tRNS alpha, grey + alpha, 16-bit,
interlaced), constant-colour textures, an OpenEXR cube map (uncompressed half, ZIP
compressed, float RGBA faces); point, spot and directional lights; an object with
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
