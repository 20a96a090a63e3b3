"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own Raycaster, MaterialGGX, Random and Camera code, compiled from the
reference sources by ``make -C oracle ref`` (the glue is oracle/ref_capi.cpp), on seeded
inputs, and stores inputs and outputs as compressed .npz files. The fixtures are committed;
the reference tree is only needed to regenerate them:

    python tests/golden/make_golden.py            (needs the reference tree)
    python tests/golden/make_golden.py --renders  (reference path-tracer renders)
    python tests/golden/make_golden.py --sky      (the sky's scattering table and MaterialSky)
    python tests/golden/make_golden.py --image    (8-bit output of renderOneShot)
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


if __name__ == "__main__" and not {"--renders", "--sky", "--image"} & set(sys.argv):
    if O.build_ref() is None:
        sys.exit("the reference tree is needed to regenerate the fixtures")
    make_raycaster()
    make_material()
    make_camera()


def make_renders():
    """Renders of the reference's own PathTracer (two independent runs per scene: the
    second calibrates the Monte-Carlo noise floor of a same-spp comparison)."""
    out = {}
    for name, sc, w, h, spp, depth in [
        ("cornell", S.cornell_scene(SEED), 48, 48, 256, 5),
        ("cornell_lit", S.cornell_scene(SEED, with_light=True), 48, 48, 256, 5),
        ("mixed", S.feature_scene(SEED), 40, 40, 256, 4),
    ]:
        tr = O.RefPathTracer(sc)
        a = tr.render(sc.camera, spp, depth, w, h, seed=SEED)
        b = tr.render(sc.camera, spp, depth, w, h, seed=SEED + 1)
        out[f"{name}_a"] = a
        out[f"{name}_b"] = b
        out[f"{name}_cfg"] = np.array([w, h, spp, depth], np.int32)
        tr.close()
    np.savez_compressed(os.path.join(HERE, "renders.npz"), **out)
    print("renders.npz:", ", ".join(k for k in out if k.endswith("_a")))


if __name__ == "__main__" and "--renders" in sys.argv:
    make_renders()


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
    make_sky(os.path.join(os.environ.get("RENDU_REFERENCE_ROOT", O.REF_ROOT_DEFAULT), "resources", "common",
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
