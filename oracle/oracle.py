"""Python access to the two CPU oracles -- test infrastructure only.

* ``liboracle_port.so``  -- the plain-C restatement of the reference's raycaster and path
  tracer (oracle/port/). Builds anywhere (``make -C oracle port``); it is the CPU
  baseline timed on the measurement host and the parity checker used by the GPU tests.
* ``_ref/libref_oracle.so`` -- the reference's own sources compiled in place
  (``make -C oracle ref``) with the glue in oracle/ref_capi.cpp. Present only where the
  reference tree is; it pins the restatement and generates tests/golden/.

Only tests/, bench.py's CPU-baseline leg and the smoke check import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_oracle.so")

NO_HIT = 0xFFFFFFFF
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_hitp = np.ctypeslib.ndpointer(HIT_DTYPE, flags="C_CONTIGUOUS")


def build_port(quiet: bool = True) -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True, capture_output=quiet)
    return PORT_LIB


def reference_root() -> str:
    """Where the reference tree is read from: $RENDU_REFERENCE_ROOT, else the build recipe's
    REF_ROOT (oracle/Makefile is the one place that names a location)."""
    root = os.environ.get("RENDU_REFERENCE_ROOT")
    if root:
        return root
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref-root"], capture_output=True,
                       text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def build_ref(quiet: bool = True, jobs: int = 8) -> str | None:
    """Compile the reference oracle when the reference tree exists; None otherwise."""
    root = reference_root()
    if not root or not os.path.isdir(os.path.join(root, "src", "engine", "raycaster")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs}", "ref", f"REF_ROOT={root}"], check=True,
                   capture_output=quiet)
    return REF_LIB


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def _model_colmajor(model):
    if model is None:
        return None
    m = np.asarray(model, np.float32)
    return np.ascontiguousarray(m.T.reshape(16))


_port = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = C.CDLL(PORT_LIB)
        lib.port_rc_create.restype = C.c_void_p
        lib.port_rc_destroy.argtypes = [C.c_void_p]
        lib.port_rc_add_mesh.argtypes = [C.c_void_p, _f32p, C.c_size_t, _u32p, C.c_size_t, C.c_void_p]
        lib.port_rc_build.argtypes = [C.c_void_p]
        lib.port_rc_node_count.argtypes = [C.c_void_p]
        lib.port_rc_node_count.restype = C.c_size_t
        lib.port_rc_intersect.argtypes = [C.c_void_p, _f32p, C.c_size_t, _hitp, C.c_int, C.c_void_p]
        lib.port_rc_intersect_any.argtypes = [C.c_void_p, _f32p, C.c_size_t, _u8p, C.c_int]
        lib.port_rc_brute.argtypes = [C.c_void_p, _f32p, C.c_size_t, _hitp, C.c_int]
        lib.port_rc_test_triangle.argtypes = [C.c_void_p, _f32p, C.c_uint32, _hitp]
        lib.port_default_threads.restype = C.c_int
        _port = lib
    return _port


_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            raise FileNotFoundError("reference oracle not built (needs the reference tree)")
        lib = C.CDLL(REF_LIB)
        lib.ref_rc_create.restype = C.c_void_p
        lib.ref_rc_destroy.argtypes = [C.c_void_p]
        lib.ref_rc_add_mesh.argtypes = [C.c_void_p, _f32p, C.c_size_t, _u32p, C.c_size_t, C.c_void_p]
        lib.ref_rc_build.argtypes = [C.c_void_p]
        lib.ref_rc_intersect.argtypes = [C.c_void_p, _f32p, C.c_size_t, _hitp, C.c_int]
        lib.ref_rc_intersect_any.argtypes = [C.c_void_p, _f32p, C.c_size_t, _u8p, C.c_int]
        lib.ref_rc_visible.argtypes = [C.c_void_p, _f32p, C.c_size_t, _u8p]
        lib.ref_ggx_eval.argtypes = [_f32p, C.c_size_t, _f32p]
        lib.ref_ggx_sample.argtypes = [_f32p, _u32p, C.c_size_t, _f32p, _f32p]
        lib.ref_cosine_hemisphere.argtypes = [_u32p, C.c_size_t, _f32p]
        lib.ref_pixel_shifts.argtypes = [C.c_void_p, _f32p]
        _pt_sigs(_Names(lib), "ref_pt_")
        lib.ref_pt_render.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _f32p,
                                      C.c_uint32, C.c_uint32]
        _ref = lib
    return _ref


class _RaycasterBase:
    _prefix = ""

    def __init__(self, lib):
        self.lib = lib
        self.h = getattr(lib, self._prefix + "rc_create")()
        self._keep = []
        self.tri_offsets = []
        self.tris = 0

    def add_mesh(self, positions, indices, model=None) -> int:
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        m = _model_colmajor(model)
        self._keep += [pos, idx, m]
        mp = m.ctypes.data if m is not None else None
        r = getattr(self.lib, self._prefix + "rc_add_mesh")(self.h, pos, len(pos) // 3, idx, len(idx), mp)
        if r < 0:
            raise ValueError("add_mesh rejected the mesh")
        self.tri_offsets.append(self.tris)
        self.tris += len(idx) // 3
        return r

    def build(self):
        getattr(self.lib, self._prefix + "rc_build")(self.h)

    def close(self):
        if self.h:
            getattr(self.lib, self._prefix + "rc_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PortRaycaster(_RaycasterBase):
    """The C restatement of Raycaster (oracle/port/rt_port.c)."""

    _prefix = "port_"

    def __init__(self):
        super().__init__(port_lib())

    def intersect(self, rays, threads: int = 0, counters: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), HIT_DTYPE)
        cnt = np.zeros(2, np.uint64)
        self.lib.port_rc_intersect(self.h, rays.reshape(-1), len(rays), out, threads, cnt.ctypes.data)
        return (out, cnt) if counters else out

    def intersect_any(self, rays, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), np.uint8)
        self.lib.port_rc_intersect_any(self.h, rays.reshape(-1), len(rays), out, threads)
        return out

    def brute(self, rays, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), HIT_DTYPE)
        self.lib.port_rc_brute(self.h, rays.reshape(-1), len(rays), out, threads)
        return out

    def test_triangle(self, ray, prim):
        ray = np.ascontiguousarray(ray, np.float32).reshape(-1)
        out = np.zeros(1, HIT_DTYPE)
        r = self.lib.port_rc_test_triangle(self.h, ray, int(prim), out)
        return r, out[0]

    @property
    def node_count(self):
        return self.lib.port_rc_node_count(self.h)


class RefRaycaster(_RaycasterBase):
    """The reference's own Raycaster, compiled from its sources."""

    _prefix = "ref_"

    def __init__(self):
        super().__init__(ref_lib())

    def intersect(self, rays, parallel: bool = True):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), HIT_DTYPE)
        self.lib.ref_rc_intersect(self.h, rays.reshape(-1), len(rays), out, int(parallel))
        return out

    def intersect_any(self, rays, parallel: bool = True):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), np.uint8)
        self.lib.ref_rc_intersect_any(self.h, rays.reshape(-1), len(rays), out, int(parallel))
        return out

    def visible(self, segs):
        segs = np.ascontiguousarray(segs, np.float32)
        out = np.zeros(len(segs), np.uint8)
        self.lib.ref_rc_visible(self.h, segs.reshape(-1), len(segs), out)
        return out


def ref_ggx_eval(cases):
    cases = np.ascontiguousarray(cases, np.float32)
    out = np.zeros((len(cases), 3), np.float32)
    ref_lib().ref_ggx_eval(cases.reshape(-1), len(cases), out.reshape(-1))
    return out


def ref_ggx_sample(cases, seeds):
    cases = np.ascontiguousarray(cases, np.float32)
    seeds = np.ascontiguousarray(seeds, np.uint32)
    uni = np.zeros((len(cases), 3), np.float32)
    out = np.zeros((len(cases), 6), np.float32)
    ref_lib().ref_ggx_sample(cases.reshape(-1), seeds, len(cases), uni.reshape(-1), out.reshape(-1))
    return uni, out


def ref_cosine_hemisphere(seeds):
    seeds = np.ascontiguousarray(seeds, np.uint32)
    out = np.zeros((len(seeds), 5), np.float32)
    ref_lib().ref_cosine_hemisphere(seeds, len(seeds), out.reshape(-1))
    return out


# ---- path tracer oracles ------------------------------------------------------------------
def _pt_sigs(lib, prefix):
    lib[prefix + "create"].restype = C.c_void_p
    lib[prefix + "destroy"].argtypes = [C.c_void_p]
    lib[prefix + "add_texture"].argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _f32p]
    lib[prefix + "add_mesh"].argtypes = [C.c_void_p, C.c_void_p]
    lib[prefix + "add_material"].argtypes = [C.c_void_p, C.c_void_p]
    lib[prefix + "add_object"].argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    lib[prefix + "add_light"].argtypes = [C.c_void_p, C.c_void_p]
    lib[prefix + "set_background"].argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib[prefix + "commit"].argtypes = [C.c_void_p]


class _OracleTracer:
    """Loads an in-memory scene (rendu_gb300.scenes.Scene) into a CPU path tracer oracle."""

    def __init__(self, lib, prefix, scene):
        from rendu_gb300 import _lib as L
        from rendu_gb300.pathtracer import light_desc

        self.lib, self.p = lib, prefix
        f = lambda n: getattr(lib, prefix + n)  # noqa: E731
        self.h = f("create")()
        self._keep = []
        for img in scene.textures:
            a = np.ascontiguousarray(img, np.float32)
            hgt, wid = a.shape[:2]
            ch = 1 if a.ndim == 2 else a.shape[2]
            self._keep.append(a)
            f("add_texture")(self.h, wid, hgt, ch, a.reshape(-1))
        for m in scene.meshes:
            arrs = [np.ascontiguousarray(x, np.float32).reshape(-1) for x in (m.positions, m.normals, m.tangents,
                                                                                m.bitangents)]
            uv = None if m.texcoords is None else np.ascontiguousarray(m.texcoords, np.float32).reshape(-1)
            idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1)
            self._keep += arrs + [uv, idx]
            d = L.pt_mesh_desc(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data, arrs[3].ctypes.data,
                               uv.ctypes.data if uv is not None else None, len(arrs[0]) // 3, idx.ctypes.data, len(idx))
            f("add_mesh")(self.h, C.byref(d))
        for mat in scene.materials:
            d = L.pt_material_desc(int(mat["type"]), int(bool(mat["masked"])), (C.c_uint32 * 3)(*mat["tex"]))
            f("add_material")(self.h, C.byref(d))
        for o in scene.objects:
            m = np.ascontiguousarray(np.asarray(o["model"], np.float32).T.reshape(16))
            self._keep.append(m)
            f("add_object")(self.h, int(o["mesh"]), int(o["material"]), m.ctypes.data)
        for l in scene.lights:
            f("add_light")(self.h, C.byref(light_desc(l)))
        bg = scene.background
        col = (C.c_float * 3)(*[float(x) for x in bg.get("color", (0, 0, 0))])
        f("set_background")(self.h, int(bg["mode"]), col, (C.c_uint32 * 6)(*bg.get("tex", (0,) * 6)))
        if bg.get("sky_table") is not None and hasattr(lib, prefix + "set_sky_table"):
            t = np.ascontiguousarray(bg["sky_table"], np.float32)
            self._keep.append(t)
            f("set_sky_table")(self.h, t.reshape(-1), t.shape[1], t.shape[0])
        env = getattr(scene, "environment", None)
        if env is not None and hasattr(lib, prefix + "set_environment"):
            f("set_environment")(self.h, int(env["tex"]), C.c_float(float(env.get("intensity", 1.0))))
        f("commit")(self.h)

    def close(self):
        if self.h:
            getattr(self.lib, self.p + "destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PortPathTracer(_OracleTracer):
    """The C restatement of PathTracer (oracle/port/pt_port.c); Philox random stream."""

    def __init__(self, scene):
        lib = port_lib()
        if not hasattr(lib, "_pt_ready"):
            _pt_sigs(_Names(lib), "port_pt_")
            lib.port_pt_render.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, _f32p,
                                           C.c_uint32, C.c_uint32, C.c_int, _u64p]
            lib.port_pt_render_ex.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, _f32p,
                                              C.c_uint32, C.c_uint32, C.c_int, _u64p, C.c_int, C.c_float]
            lib.port_pt_set_environment.argtypes = [C.c_void_p, C.c_uint32, C.c_float]
            lib.port_pt_set_sky_table.argtypes = [C.c_void_p, _f32p, C.c_uint32, C.c_uint32]
            lib.port_ggx_eval.argtypes = [_f32p, C.c_size_t, _f32p]
            lib.port_ggx_sample.argtypes = [_f32p, _f32p, C.c_size_t, _f32p]
            lib.port_pixel_shifts.argtypes = [C.c_void_p, _f32p]
            lib._pt_ready = True
        super().__init__(lib, "port_pt_", scene)

    def render(self, camera, samples, depth, width, height, seed=0, threads=0, image=None, mode=0, clamp=5.0):
        from rendu_gb300.pathtracer import camera_desc

        img = np.zeros((height, width, 3), np.float32) if image is None else image
        rays = np.zeros(3, np.uint64)
        cam = camera_desc(camera)
        r = self.lib.port_pt_render_ex(self.h, C.byref(cam), int(samples), int(depth), int(seed), img.reshape(-1),
                                       width, height, int(threads), rays, int(mode), float(clamp))
        if r != 0:
            raise RuntimeError("port render failed")
        self.rays = rays
        return img


class RefPathTracer(_OracleTracer):
    """The reference's own PathTracer compiled from its sources (mt19937 random streams)."""

    def __init__(self, scene):
        super().__init__(ref_lib(), "ref_pt_", scene)

    def render(self, camera, samples, depth, width, height, seed=0):
        from rendu_gb300.pathtracer import camera_desc

        img = np.zeros((height, width, 3), np.float32)
        cam = camera_desc(camera)
        self.lib.ref_pt_render(self.h, C.byref(cam), int(samples), int(depth), int(seed), img.reshape(-1), width,
                               height)
        return img


class _Names(dict):
    def __init__(self, lib):
        super().__init__()
        self.lib = lib

    def __getitem__(self, k):
        return getattr(self.lib, k)


def port_ggx_eval(cases):
    lib = port_lib()
    lib.port_ggx_eval.argtypes = [_f32p, C.c_size_t, _f32p]
    c = np.ascontiguousarray(cases, np.float32)
    out = np.zeros((len(c), 3), np.float32)
    lib.port_ggx_eval(c.reshape(-1), len(c), out.reshape(-1))
    return out


def port_ggx_sample(cases, uniforms):
    lib = port_lib()
    lib.port_ggx_sample.argtypes = [_f32p, _f32p, C.c_size_t, _f32p]
    c = np.ascontiguousarray(cases, np.float32)
    u = np.ascontiguousarray(uniforms, np.float32)
    out = np.zeros((len(c), 6), np.float32)
    lib.port_ggx_sample(c.reshape(-1), u.reshape(-1), len(c), out.reshape(-1))
    return out


def port_pixel_shifts(camera: dict):
    from rendu_gb300.pathtracer import camera_desc

    lib = port_lib()
    lib.port_pixel_shifts.argtypes = [C.c_void_p, _f32p]
    out = np.zeros(12, np.float32)
    cam = camera_desc(camera)
    lib.port_pixel_shifts(C.byref(cam), out)
    return out


# ---- atmosphere (MaterialSky, AtmosphereApp::precomputeTable) -------------------------------
def port_sky_table(res: int = 512, samples: int = 256, half: bool = True) -> np.ndarray:
    """The C restatement of AtmosphereApp::precomputeTable: (res, res, 4) float32, rounded to
    half precision like the reference's stored table unless half=False."""
    lib = port_lib()
    lib.port_sky_table.argtypes = [C.c_uint32, C.c_uint32, C.c_int, _f32p]
    out = np.zeros((res, res, 4), np.float32)
    lib.port_sky_table(res, samples, int(half), out.reshape(-1))
    return out


def port_round_half(x) -> np.ndarray:
    lib = port_lib()
    lib.port_round_half.argtypes = [C.c_float]
    lib.port_round_half.restype = C.c_float
    a = np.asarray(x, np.float32).reshape(-1)
    return np.array([lib.port_round_half(float(v)) for v in a], np.float32)


def port_sky_eval(table, cases) -> np.ndarray:
    """The C restatement of MaterialSky::eval for cases (n, 9) {origin, direction, sun}."""
    lib = port_lib()
    lib.port_sky_eval.argtypes = [_f32p, C.c_uint32, C.c_uint32, _f32p, C.c_size_t, _f32p]
    t = np.ascontiguousarray(table, np.float32)
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 9)
    out = np.zeros((len(c), 3), np.float32)
    lib.port_sky_eval(t.reshape(-1), t.shape[1], t.shape[0], c.reshape(-1), len(c), out.reshape(-1))
    return out


def ref_load_image(path: str, channels: int = 4, max_pixels: int = 1 << 22) -> np.ndarray:
    """The reference's Image::load of a file (2-D texture orientation): (h, w, channels)."""
    lib = ref_lib()
    lib.ref_load_image.argtypes = [C.c_char_p, C.c_uint, _f32p, C.c_size_t, C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32)]
    buf = np.zeros(max_pixels * channels, np.float32)
    w, h = C.c_uint32(), C.c_uint32()
    r = lib.ref_load_image(path.encode(), channels, buf, buf.size, C.byref(w), C.byref(h))
    if r != 0:
        raise RuntimeError(f"reference Image::load failed ({r}) on {path}")
    return buf[: w.value * h.value * channels].reshape(h.value, w.value, channels).copy()


def ref_sky_eval(table, cases) -> np.ndarray:
    """The reference's MaterialSky::eval with the given scattering table."""
    lib = ref_lib()
    lib.ref_set_sky_table.argtypes = [_f32p, C.c_uint32, C.c_uint32]
    lib.ref_sky_eval.argtypes = [_f32p, C.c_size_t, _f32p]
    t = np.ascontiguousarray(table, np.float32)
    lib.ref_set_sky_table(t.reshape(-1), t.shape[1], t.shape[0])
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 9)
    out = np.zeros((len(c), 3), np.float32)
    lib.ref_sky_eval(c.reshape(-1), len(c), out.reshape(-1))
    return out


def ref_save_image(image, path: str) -> int:
    """The reference's Image::save with renderOneShot's options (main.cpp:119)."""
    lib = ref_lib()
    lib.ref_save_image.argtypes = [_f32p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p]
    a = np.ascontiguousarray(image, np.float32)
    h, w, c = a.shape
    return lib.ref_save_image(a.reshape(-1), w, h, c, path.encode())


def ref_mesh_load_obj(text) -> dict:
    """The reference's mesh loading of an OBJ text (getMesh with FORCE_FRAME, restated in
    oracle/ref_mesh.cpp around the reference's glm and mikktspace.c)."""
    lib = ref_lib()
    data = text.encode() if isinstance(text, str) else bytes(text)
    counts = np.zeros(3, np.uint64)
    lib.ref_mesh_load_obj.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64)]
    lib.ref_mesh_error.restype = C.c_char_p
    r = lib.ref_mesh_load_obj(data, len(data), counts.ctypes.data_as(C.POINTER(C.c_uint64)))
    if r != 0:
        raise ValueError(lib.ref_mesh_error().decode())
    nv, ni = int(counts[0]), int(counts[1])
    out = {k: np.zeros((nv, d), np.float32) for k, d in (("positions", 3), ("normals", 3), ("texcoords", 2),
                                                          ("tangents", 3), ("bitangents", 3))}
    out["indices"] = np.zeros(ni, np.uint32)
    lib.ref_mesh_get.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p, _u32p]
    lib.ref_mesh_get(*(out[k].reshape(-1) for k in ("positions", "normals", "texcoords", "tangents", "bitangents",
                                                     "indices")))
    out["had_uv"] = bool(counts[2])
    return out


def ref_mikktspace(positions, normals, texcoords, indices) -> np.ndarray:
    """The reference's own mikktspace.c: per-corner (tangent xyz, sign), (len(indices), 4)."""
    lib = ref_lib()
    lib.ref_mikktspace.argtypes = [_f32p, _f32p, _f32p, C.c_size_t, _u32p, C.c_size_t, _f32p]
    p = np.ascontiguousarray(positions, np.float32)
    n = np.ascontiguousarray(normals, np.float32)
    u = np.ascontiguousarray(texcoords, np.float32)
    i = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    out = np.zeros((len(i), 4), np.float32)
    if lib.ref_mikktspace(p.reshape(-1), n.reshape(-1), u.reshape(-1), len(p), i, len(i), out.reshape(-1)) != 0:
        raise ValueError("mikktspace failed")
    return out


def ref_transformation(axis, angle, trans, scale) -> np.ndarray:
    """glm's translate * rotate * scale of Codable::decodeTransformation: row-major 4x4."""
    lib = ref_lib()
    lib.ref_transformation.argtypes = [_f32p, C.c_float, _f32p, C.c_float, _f32p]
    out = np.zeros(16, np.float32)
    lib.ref_transformation(np.asarray(axis, np.float32), float(angle), np.asarray(trans, np.float32), float(scale), out)
    return out.reshape(4, 4).T.copy()


def ref_mat_mul(a, b) -> np.ndarray:
    """glm's mat4 product of two row-major 4x4 matrices."""
    lib = ref_lib()
    lib.ref_mat_mul.argtypes = [_f32p, _f32p, _f32p]
    out = np.zeros(16, np.float32)
    lib.ref_mat_mul(np.ascontiguousarray(np.asarray(a, np.float32).T).reshape(-1),
                    np.ascontiguousarray(np.asarray(b, np.float32).T).reshape(-1), out)
    return out.reshape(4, 4).T.copy()
