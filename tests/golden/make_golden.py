"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own Raycaster, MaterialGGX, Random and Camera code, compiled from the
reference sources by ``make -C oracle ref`` (the glue is oracle/ref_capi.cpp), on seeded
inputs, and stores inputs and outputs as compressed .npz files. The fixtures are committed;
the reference tree is only needed to regenerate them:

    python tests/golden/make_golden.py            (needs the reference tree)
    python tests/golden/make_golden.py --renders [scene ...]  (reference path-tracer renders)
    python tests/golden/make_golden.py --sky      (the sky's scattering table and MaterialSky)
    python tests/golden/make_golden.py --image    (8-bit output of renderOneShot)
    python tests/golden/make_golden.py --scene-io (scene loading: meshes, MikkTSpace,
                                                   texture decoding, transformations)
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from rendu_gb300 import scenes as S  # noqa: E402

SEED = 20261203


def raycaster_scene():
    """Four meshes: displaced icosphere (5120 tris), a transformed box, a flat quad lying in
    a coordinate plane, and a second transformed icosphere (320 tris) that overlaps the box."""
    sphere = S.icosphere_mesh(4, seed=SEED)
    box = S.box_mesh((1.0, 0.6, 0.8))
    quad = S.quad_mesh((-2.0, -1.2, -2.0), (4.0, 0.0, 0.0), (0.0, 0.0, 4.0))
    small = S.icosphere_mesh(2, seed=SEED + 1, displacement=0.2)
    meshes = [
        (sphere.positions, sphere.indices, None),
        (box.positions, box.indices, S.translation((1.4, 0.1, 0.2)) @ S.rotation_y(0.6) @ S.scaling(0.9)),
        (quad.positions, quad.indices, None),
        (small.positions, small.indices, S.translation((1.2, 0.5, 0.0)) @ S.scaling(0.45)),
    ]
    return meshes


def raycaster_rays(meshes, n_random=6000, n_aimed=3000, seed=SEED):
    rng = np.random.default_rng(seed)
    allp = np.concatenate([
        (np.c_[p.reshape(-1, 3), np.ones(len(p.reshape(-1, 3)))] @ (np.eye(4) if m is None else m).T)[:, :3]
        for p, _, m in meshes])
    lo, hi = allp.min(0), allp.max(0)
    rays = [S.random_rays(n_random, lo, hi, seed + 1)]
    # Rays aimed at random vertices (with jitter) so that many hit.
    o = 0.5 * (lo + hi) + (rng.random((n_aimed, 3)) * 2 - 1) * 1.5 * (hi - lo)
    tgt = allp[rng.integers(0, len(allp), n_aimed)] + rng.normal(0, 0.02, (n_aimed, 3))
    d = tgt - o
    a = np.zeros((n_aimed, 8), np.float32)
    a[:, 0:3] = o
    a[:, 3] = 1e-4
    a[:, 4:7] = d
    a[:, 7] = 1e8
    rays.append(a)
    # Windows: short tmax, large tmin, and origins placed on the geometry.
    w = a[: n_aimed // 3].copy()
    w[:, 7] = rng.uniform(0.1, 3.0, len(w)).astype(np.float32)
    w[:, 3] = rng.uniform(0.0, 0.5, len(w)).astype(np.float32)
    rays.append(w)
    on = np.zeros((1000, 8), np.float32)
    on[:, 0:3] = allp[rng.integers(0, len(allp), 1000)]
    z = rng.random(1000) * 2 - 1
    ph = rng.random(1000) * 2 * math.pi
    r = np.sqrt(1 - z * z)
    on[:, 4] = r * np.cos(ph)
    on[:, 5] = r * np.sin(ph)
    on[:, 6] = z
    on[:, 3] = 1e-4
    on[:, 7] = 1e8
    rays.append(on)
    # Axis-aligned directions (zero components, infinite reciprocals).
    ax = np.zeros((600, 8), np.float32)
    ax[:, 0:3] = o[:600]
    for k in range(600):
        ax[k, 4 + (k % 3)] = 1.0 if (k // 3) % 2 == 0 else -1.0
    ax[:, 3] = 1e-4
    ax[:, 7] = 1e8
    rays.append(ax)
    return np.concatenate(rays).astype(np.float32)


def make_raycaster():
    meshes = raycaster_scene()
    rays = raycaster_rays(meshes)
    ref = O.RefRaycaster()
    for p, i, m in meshes:
        ref.add_mesh(p, i, m)
    ref.build()
    hits = ref.intersect(rays, parallel=False)
    anyh = ref.intersect_any(rays, parallel=False)
    rng = np.random.default_rng(SEED + 7)
    segs = np.concatenate([rays[:2000, 0:3], rays[:2000, 0:3] + rng.uniform(0.2, 3.0, (2000, 1)) *
                           rays[:2000, 4:7] / np.linalg.norm(rays[:2000, 4:7], axis=1, keepdims=True)], 1)
    segs = segs.astype(np.float32)
    vis = ref.visible(segs)
    out = {"rays": rays, "hit_t": hits["t"], "hit_u": hits["u"], "hit_v": hits["v"], "hit_prim": hits["prim"],
           "any": anyh, "segs": segs, "visible": vis}
    for k, (p, i, m) in enumerate(meshes):
        out[f"mesh{k}_pos"] = np.asarray(p, np.float32)
        out[f"mesh{k}_idx"] = np.asarray(i, np.uint32)
        out[f"mesh{k}_model"] = np.eye(4, dtype=np.float32) if m is None else np.asarray(m, np.float32)
        out[f"mesh{k}_has_model"] = np.array(m is not None)
    np.savez_compressed(os.path.join(HERE, "raycaster_small.npz"), **out)
    print("raycaster_small.npz:", len(rays), "rays,", int((hits["prim"] != O.NO_HIT).sum()), "hits")


def make_material():
    rng = np.random.default_rng(SEED + 11)
    n = 3000

    def hemi(m, below_frac=0.1):
        z = rng.random(m) * 2 - 1
        z = np.where(rng.random(m) < below_frac, -np.abs(z), np.abs(z))
        ph = rng.random(m) * 2 * math.pi
        r = np.sqrt(1 - z * z)
        return np.stack([r * np.cos(ph), r * np.sin(ph), z], 1)

    wo = hemi(n)
    wi = hemi(n)
    base = rng.uniform(0.0, 1.0, (n, 3))
    rough = np.where(rng.random(n) < 0.1, rng.uniform(0.0, 0.05, n), rng.uniform(0.0, 1.0, n))
    metal = np.where(rng.random(n) < 0.3, rng.integers(0, 2, n).astype(float), rng.random(n))
    ev = np.concatenate([wo, base, rough[:, None], metal[:, None], wi], 1).astype(np.float32)
    ev_out = O.ref_ggx_eval(ev)
    sm = np.concatenate([hemi(n, 0.05), base, rough[:, None], metal[:, None]], 1).astype(np.float32)
    seeds = rng.integers(0, 2**31 - 1, n).astype(np.uint32)
    uni, sm_out = O.ref_ggx_sample(sm, seeds)
    cos = O.ref_cosine_hemisphere(seeds[:1000])
    np.savez_compressed(os.path.join(HERE, "material_ggx.npz"), eval_in=ev, eval_out=ev_out, sample_in=sm,
                        sample_uniforms=uni, sample_out=sm_out, cosine=cos)
    print("material_ggx.npz:", n, "eval and sample cases")


def make_camera():
    import ctypes as C

    from rendu_gb300._lib import pt_camera_desc

    rng = np.random.default_rng(SEED + 13)
    cams, outs = [], []
    for k in range(16):
        eye = rng.uniform(-3, 3, 3)
        center = rng.uniform(-1, 1, 3)
        up = np.array([0.0, 1.0, 0.0]) if k % 2 == 0 else rng.normal(0, 1, 3)
        fov = rng.uniform(0.4, 1.6)
        ratio = rng.uniform(0.5, 2.0)
        d = pt_camera_desc((C.c_float * 3)(*eye), (C.c_float * 3)(*center), (C.c_float * 3)(*up), fov, ratio)
        out = np.zeros(12, np.float32)
        O.ref_lib().ref_pixel_shifts(C.byref(d), out)
        cams.append(np.concatenate([eye, center, up, [fov, ratio]]).astype(np.float32))
        outs.append(out)
    np.savez_compressed(os.path.join(HERE, "camera.npz"), cameras=np.array(cams), shifts=np.array(outs))
    print("camera.npz: 16 cameras")


if __name__ == "__main__" and not {"--renders", "--sky", "--image", "--scene-io"} & set(sys.argv):
    if O.build_ref() is None:
        sys.exit("the reference tree is needed to regenerate the fixtures")
    make_raycaster()
    make_material()
    make_camera()


def make_renders(names=None):
    """Renders of the reference's own PathTracer (two independent runs per scene: the
    second calibrates the Monte-Carlo noise floor of a same-spp comparison). `names`
    regenerates only those scenes and keeps the others' stored renders."""
    path = os.path.join(HERE, "renders.npz")
    out = dict(np.load(path)) if names and os.path.exists(path) else {}
    for name, make, w, h, spp, depth in [
        ("cornell", lambda: S.cornell_scene(SEED), 48, 48, 256, 5),
        ("cornell_lit", lambda: S.cornell_scene(SEED, with_light=True), 48, 48, 256, 5),
        ("mixed", lambda: S.feature_scene(SEED), 40, 40, 256, 4),
        # the large path-tracer workload's scene (2,049,210 triangles in 205 meshes, cube-map
        # sky with the sun disc, emissive quads) at a reduced size
        ("instanced", lambda: S.instanced_scene(20261206), 160, 90, 64, 8),
    ]:
        if names and name not in names:
            continue
        sc = make()
        tr = O.RefPathTracer(sc)
        cam = dict(sc.camera, ratio=w / h)
        a = tr.render(cam, spp, depth, w, h, seed=SEED)
        b = tr.render(cam, spp, depth, w, h, seed=SEED + 1)
        out[f"{name}_a"] = a
        out[f"{name}_b"] = b
        out[f"{name}_cfg"] = np.array([w, h, spp, depth], np.int32)
        tr.close()
    np.savez_compressed(path, **out)
    print("renders.npz:", ", ".join(k for k in out if k.endswith("_a")))


if __name__ == "__main__" and "--renders" in sys.argv:
    make_renders([a for a in sys.argv[sys.argv.index("--renders") + 1:] if not a.startswith("--")] or None)


def sky_cases(n=3000, seed=SEED):
    """Rays for MaterialSky::eval: origins near the ground (heights 0-120), directions on the
    sphere, a quarter of them aimed within the sun's disc, suns above and below the horizon."""
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(-60, 60, n), rng.uniform(0, 120, n), rng.uniform(-60, 60, n)], 1)
    sun = rng.normal(size=(n, 3))
    sun[: 3 * n // 4, 1] = np.abs(sun[: 3 * n // 4, 1])
    sun /= np.linalg.norm(sun, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    k = n // 4
    d[:k] = sun[:k] + rng.normal(scale=0.02, size=(k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d, sun], 1).astype(np.float32)


def make_sky(exr):
    """The reference's scattering table (resources/common/scattering-precomputed.exr, read by
    its own Image::load) and its MaterialSky::eval on seeded rays with that table."""
    table = O.ref_load_image(exr, 4)
    cases = sky_cases()
    out = O.ref_sky_eval(table, cases)
    np.savez_compressed(os.path.join(HERE, "sky.npz"), table_sub=table[::8, ::8, :3], table_shape=np.array(table.shape),
                        table_row_sums=table[..., :3].astype(np.float64).sum(axis=1), cases=cases, eval_out=out)
    print("sky.npz:", table.shape, len(cases), "cases")


if __name__ == "__main__" and "--sky" in sys.argv:
    if O.build_ref() is None:
        sys.exit("the reference tree is needed to regenerate the fixtures")
    make_sky(os.path.join(O.reference_root(), "resources", "common",
                          "scattering-precomputed.exr"))


def image_io_input(seed=SEED):
    """A 40 x 24 RGB image covering saveAsLDR's cases: values in [0, 1.3] (clamping above 1),
    negatives, exact 8-bit boundaries k/255, zeros and a NaN."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, 1.3, (24, 40, 3)).astype(np.float32)
    x[0, :10] = -rng.uniform(0, 1, (10, 3))
    x[1, :, :] = (np.arange(40 * 3).reshape(40, 3) % 256 / 255.0) ** 2.2
    x[2, 0, 0] = np.nan
    x[3, :5] = 0.0
    return x


def make_image_io():
    """The reference's Image::save with renderOneShot's options (main.cpp:119) of a seeded
    image, read back with its own Image::load (bytes = value x 255)."""
    import tempfile

    x = image_io_input()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ref.png")
        O.ref_save_image(x, path)
        back = O.ref_load_image(path, 3)
    np.savez_compressed(os.path.join(HERE, "image_io.npz"), image=x, ldr=np.rint(back * 255.0).astype(np.uint8))
    print("image_io.npz:", x.shape)


if __name__ == "__main__" and "--image" in sys.argv:
    if O.build_ref() is None:
        sys.exit("the reference tree is needed to regenerate the fixtures")
    make_image_io()


# --------------------------------------------------------------------------------------
# scene loading: meshes, tangent spaces, textures, transformations
# --------------------------------------------------------------------------------------

SCENE_DEMO = os.path.join(HERE, "scene_demo")


def synthetic_meshes(seed=SEED):
    """Triangle lists that stress the tangent-space generator: a grid with random UV islands
    (mirrored and rotated), duplicated corners, position-degenerate and UV-degenerate
    triangles, a fan with exactly opposite tangents, and constant UVs."""
    rng = np.random.default_rng(seed)
    out = []
    # 1. 9 x 9 grid, heights and UVs jittered; four UV islands, two of them mirrored
    n = 9
    g = np.stack(np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n)), -1).reshape(-1, 2)
    pos = np.concatenate([g[:, :1], 0.2 * np.sin(3 * g[:, :1] + 2 * g[:, 1:]), g[:, 1:]], 1)
    idx = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = i * n + j, i * n + j + 1, (i + 1) * n + j + 1, (i + 1) * n + j
            idx += [a, b, c, a, c, d]
    idx = np.asarray(idx)
    P, U = pos[idx], g[idx] * 0.5 + 0.5
    island = (np.arange(len(idx)) // 3 // 16) % 4
    U = np.where((island == 1)[:, None], U[:, ::-1], U)
    U = np.where((island == 2)[:, None], U * np.array([-1.0, 1.0]), U)
    N = np.tile([0.0, 1.0, 0.0], (len(idx), 1)) + 0.1 * rng.standard_normal((len(idx), 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    # weld what is identical: corners of the same grid vertex in the same island share data
    key = np.concatenate([P, N * 0 + np.round(N, 1), U], 1)
    _, first, inv = np.unique(np.round(key, 6), axis=0, return_index=True, return_inverse=True)
    N = N[first][inv.reshape(-1)]
    verts, ind = np.unique(np.concatenate([P, N, U], 1), axis=0, return_inverse=True)
    tri = ind.reshape(-1).astype(np.uint32)
    tri[6:9] = tri[[6, 6, 7]]  # a position-degenerate triangle
    out.append(("grid_islands", verts[:, :3], verts[:, 3:6], verts[:, 6:8], tri))
    # 2. random soup with shared vertices, some UV-degenerate triangles
    m = 60
    v = rng.normal(size=(m, 3))
    nn = v / np.linalg.norm(v, axis=1, keepdims=True)
    uv = rng.uniform(0, 1, (m, 2))
    uv[:5] = uv[0]
    tri = rng.integers(0, m, (120, 3))
    tri = tri[(tri[:, 0] != tri[:, 1]) & (tri[:, 1] != tri[:, 2]) & (tri[:, 0] != tri[:, 2])]
    tri[:4] = [[0, 1, 2], [1, 2, 3], [2, 3, 4], [0, 3, 4]]
    out.append(("soup", v, nn, uv, tri.reshape(-1).astype(np.uint32)))
    # 3. a symmetric pole fan: opposite triangles have exactly opposite tangents
    k = 8
    ring = np.stack([np.cos(2 * np.pi * np.arange(k) / k), np.zeros(k), np.sin(2 * np.pi * np.arange(k) / k)], 1)
    v = np.concatenate([[[0.0, 1.0, 0.0]], ring * 0.5 + [0, 0.8, 0]], 0)
    nn = v / np.linalg.norm(v, axis=1, keepdims=True)
    uv = np.concatenate([[[0.5, 0.5]], ring[:, [0, 2]] * 0.5 + 0.5], 0)
    tri = np.asarray([[0, 1 + (i + 1) % k, 1 + i] for i in range(k)]).reshape(-1).astype(np.uint32)
    out.append(("pole_fan", v, nn, uv, tri))
    # 4. constant UVs (what a mesh without texture coordinates gets)
    v = rng.normal(size=(30, 3))
    tri = np.asarray([[i, (i + 1) % 30, (i + 7) % 30] for i in range(30)]).reshape(-1).astype(np.uint32)
    out.append(("constant_uv", v, v / np.linalg.norm(v, axis=1, keepdims=True), np.full((30, 2), 0.5), tri))
    return [(name, np.asarray(p, np.float32), np.asarray(nr, np.float32), np.asarray(u, np.float32), t)
            for name, p, nr, u, t in out]


def png_variants():
    """(name, samples, writer kwargs) of PNG files covering the colour types and bit depths."""
    rng = np.random.default_rng(SEED + 7)
    h, w = 13, 11
    pal = rng.integers(0, 256, (16, 3)).astype(np.uint8)
    return [
        ("grey1", rng.integers(0, 2, (h, w, 1)), dict(ctype=0, depth=1)),
        ("grey2", rng.integers(0, 4, (h, w, 1)), dict(ctype=0, depth=2)),
        ("grey4_interlaced", rng.integers(0, 16, (h, w, 1)), dict(ctype=0, depth=4, interlace=True)),
        ("grey8_key", rng.integers(0, 4, (h, w, 1)) * 60, dict(ctype=0, depth=8, trns=b"\x00\x3c")),
        ("grey16", rng.integers(0, 65536, (h, w, 1)), dict(ctype=0, depth=16)),
        ("rgb8_key", rng.integers(0, 2, (h, w, 3)) * 200, dict(ctype=2, depth=8, trns=b"\x00\xc8\x00\x00\x00\xc8")),
        ("rgb16_interlaced", rng.integers(0, 65536, (h, w, 3)), dict(ctype=2, depth=16, interlace=True)),
        ("palette2", rng.integers(0, 4, (h, w, 1)), dict(ctype=3, depth=2, palette=pal[:4], trns=b"\x10\xff")),
        ("palette8", rng.integers(0, 16, (h, w, 1)), dict(ctype=3, depth=8, palette=pal)),
        ("greyalpha16", rng.integers(0, 65536, (h, w, 2)), dict(ctype=4, depth=16)),
        ("rgba8_interlaced", rng.integers(0, 256, (h, w, 4)), dict(ctype=6, depth=8, interlace=True)),
        ("rgba16", rng.integers(0, 65536, (h, w, 4)), dict(ctype=6, depth=16, filters=(4, 3))),
    ]


def transformation_cases(n=200, seed=SEED):
    rng = np.random.default_rng(seed)
    axis = rng.normal(size=(n, 3)).astype(np.float32)
    angle = rng.uniform(-7, 7, n).astype(np.float32)
    angle[:10] = 0.0
    trans = (rng.normal(size=(n, 3)) * 5).astype(np.float32)
    scale = rng.uniform(0.1, 4, n).astype(np.float32)
    return axis, angle, trans, scale


def make_scene_io():
    import glob
    import tempfile

    sys.path.insert(0, SCENE_DEMO)
    import make_scene as MS  # noqa: E402

    out = {}
    for path in sorted(glob.glob(os.path.join(SCENE_DEMO, "*.obj"))):
        name = os.path.basename(path)[:-4]
        r = O.ref_mesh_load_obj(open(path, "rb").read())
        for k in ("positions", "normals", "texcoords", "tangents", "bitangents", "indices"):
            out[f"obj_{name}_{k}"] = r[k]
        out[f"obj_{name}_had_uv"] = np.asarray(r["had_uv"])
    for name, p, n, u, t in synthetic_meshes():
        out[f"mk_{name}_in_pos"], out[f"mk_{name}_in_nor"], out[f"mk_{name}_in_uv"], out[f"mk_{name}_in_idx"] = p, n, u, t
        out[f"mk_{name}_out"] = O.ref_mikktspace(p, n, u, t)
    for path in sorted(glob.glob(os.path.join(SCENE_DEMO, "*.png")) + glob.glob(os.path.join(SCENE_DEMO, "*.exr"))
                       + glob.glob(os.path.join(SCENE_DEMO, "*.jpg"))):
        out[f"img_{os.path.basename(path)}"] = O.ref_load_image(path, 4)
    with tempfile.TemporaryDirectory() as d:
        for name, samples, kw in png_variants():
            path = os.path.join(d, name + ".png")
            MS.write_png(path, samples, **kw)
            for ch in (3, 4):
                out[f"png_{name}_{ch}"] = O.ref_load_image(path, ch)
    axis, angle, trans, scale = transformation_cases()
    out["tf_axis"], out["tf_angle"], out["tf_trans"], out["tf_scale"] = axis, angle, trans, scale
    out["tf_out"] = np.stack([O.ref_transformation(a, g, t, s) for a, g, t, s in zip(axis, angle, trans, scale)])
    np.savez_compressed(os.path.join(HERE, "scene_io.npz"), **out)
    print("scene_io.npz:", len(out), "arrays")


if __name__ == "__main__" and "--scene-io" in sys.argv:
    if O.build_ref() is None:
        sys.exit("the reference tree is needed to regenerate the fixtures")
    make_scene_io()
