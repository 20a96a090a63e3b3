"""Host-side mirror of Rendu's ``PathTracer`` (src/apps/pathtracer/PathTracer.hpp:11-76)
over the C-ABI ``pt_*`` entry points.

``PathTracer(scene)`` uploads the scene and builds its raycaster (PathTracer.cpp:11-21);
``render(camera, samples, depth, image)`` accumulates ``samples`` (rounded to a power of
two) paths per pixel into ``image`` and normalises, as PathTracer::render does
(PathTracer.cpp:159-299). ``image`` is a float32 array (H, W, C>=3) on the host or a CUDA
tensor of the same shape.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .raycaster import Raycaster


KERNEL_KINDS = ("raygen", "trace", "shade", "shadow", "accumulate")  # pt_render_stats.kernel_ms order


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def camera_desc(cam: dict) -> L.pt_camera_desc:
    return L.pt_camera_desc(_f3(cam["eye"]), _f3(cam["center"]), _f3(cam["up"]), float(cam.get("fov", 1.3)),
                            float(cam.get("ratio", 1.0)))


def light_desc(l: dict) -> L.pt_light_desc:
    return L.pt_light_desc(int(l["type"]), int(bool(l.get("shadows", False))), _f3(l.get("color", (1, 1, 1))),
                           _f3(l.get("position", (0, 0, 0))), _f3(l.get("direction", (0, -1, 0))),
                           float(l.get("radius", 1.0)), float(l.get("inner", 0.5)), float(l.get("outer", 0.8)))


class PathTracer:
    """Device path tracer over an in-memory scene (rendu_gb300.scenes.Scene)."""

    def __init__(self, scene, device: int = 0):
        h = C.c_void_p()
        L.call("pt_scene_create", C.byref(h), int(device))
        self._h = h
        self.device = device
        self._keep = []
        self.scene = scene
        try:
            self._upload(scene)
        except Exception:
            self.close()
            raise

    def _upload(self, sc):
        tid = C.c_uint32()
        for img in sc.textures:
            a = np.ascontiguousarray(img, np.float32)
            hgt, wid = a.shape[:2]
            ch = 1 if a.ndim == 2 else a.shape[2]
            L.call("pt_scene_add_texture", self._h, wid, hgt, ch, a.ctypes.data, C.byref(tid))
        for m in sc.meshes:
            arrs = [np.ascontiguousarray(x, np.float32).reshape(-1) for x in (m.positions, m.normals, m.tangents,
                                                                                m.bitangents)]
            uv = None if m.texcoords is None else np.ascontiguousarray(m.texcoords, np.float32).reshape(-1)
            idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1)
            self._keep += arrs + [uv, idx]
            d = L.pt_mesh_desc(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data, arrs[3].ctypes.data,
                               uv.ctypes.data if uv is not None else None, len(arrs[0]) // 3, idx.ctypes.data, len(idx))
            L.call("pt_scene_add_mesh", self._h, C.byref(d), C.byref(tid))
        for mat in sc.materials:
            d = L.pt_material_desc(int(mat["type"]), int(bool(mat["masked"])), (C.c_uint32 * 3)(*mat["tex"]))
            L.call("pt_scene_add_material", self._h, C.byref(d), C.byref(tid))
        for o in sc.objects:
            m = np.ascontiguousarray(np.asarray(o["model"], np.float32).T.reshape(16))
            L.call("pt_scene_add_object", self._h, int(o["mesh"]), int(o["material"]), m.ctypes.data, C.byref(tid))
        for l in sc.lights:
            L.call("pt_scene_add_light", self._h, C.byref(light_desc(l)))
        bg = sc.background
        L.call("pt_scene_set_background", self._h, int(bg["mode"]), _f3(bg.get("color", (0, 0, 0))),
               (C.c_uint32 * 6)(*bg.get("tex", (0,) * 6)))
        if bg.get("sky_table") is not None:  # ATMOSPHERE: a caller-supplied scattering table
            t = np.ascontiguousarray(bg["sky_table"], np.float32)
            self._keep.append(t)
            L.call("pt_scene_set_sky_table", self._h, t.ctypes.data, t.shape[1], t.shape[0])
        if getattr(sc, "environment", None) is not None:
            L.call("pt_scene_set_environment", self._h, int(sc.environment["tex"]),
                   float(sc.environment.get("intensity", 1.0)))
        L.call("pt_scene_commit", self._h)

    def render(self, camera, samples: int, depth: int, image, seed: int = 0, mode: int = 0, clamp: float = 5.0,
               fp64: bool = False, aov=None, ranks: int = 1, rank: int = 0, profile: bool = False):
        """PathTracer::render(camera, samples, depth, image): accumulate and normalise into
        ``image`` (H, W, C) float32, host array or CUDA tensor; returns ``image``.
        ``mode`` 1 selects the extended estimator (NEE on emitters and the environment
        map with MIS); ``clamp`` is the per-sample clamp (the reference's 5; <= 0: none);
        ``fp64`` accumulates each pixel's samples in double precision; ``aov`` (H, W, 8)
        float32 (same place as ``image``) receives first-hit albedo, normal and distance
        and the standard error of the pixel's mean luminance.
        ``ranks`` > 1 renders only the pixel tiles of ``rank`` and zeroes the others
        (pt_render_options.ranks; see render_split). ``profile`` times every kernel class
        (last_stats()["kernel_ms"]), launching the kernels without the captured graph."""
        cam = camera_desc(camera if isinstance(camera, dict) else camera.__dict__)
        aov_ptr = None
        if aov is not None:
            aov_ptr = aov.data_ptr() if type(aov).__module__.startswith("torch") else aov.ctypes.data
        opts = L.pt_render_options(int(mode), float(clamp), int(bool(fp64)), aov_ptr, int(ranks), int(rank),
                                   int(bool(profile)))
        if type(image).__module__.startswith("torch") and getattr(image, "is_cuda", False):
            import torch

            hgt, wid, comp = image.shape
            assert image.is_contiguous() and image.dtype == torch.float32
            L.call("pt_render_ex", self._h, C.byref(cam), int(samples), int(depth), int(seed),
                   C.c_void_p(image.data_ptr()), wid, hgt, comp, C.byref(opts),
                   C.c_void_p(torch.cuda.current_stream().cuda_stream), L.RT_FLAG_DEVICE_PTRS)
            return image
        if not (isinstance(image, np.ndarray) and image.dtype == np.float32 and image.flags.c_contiguous):
            raise TypeError("image must be a C-contiguous float32 array (H, W, C)")
        hgt, wid, comp = image.shape
        L.call("pt_render_ex", self._h, C.byref(cam), int(samples), int(depth), int(seed), image.ctypes.data, wid, hgt,
               comp, C.byref(opts), None, 0)
        return image

    def last_stats(self) -> dict:
        s = L.pt_render_stats()
        L.call("pt_get_render_stats", self._h, C.byref(s))
        d = {k: getattr(s, k) for k, _ in s._fields_}
        d["kernel_ms"] = dict(zip(KERNEL_KINDS, list(s.kernel_ms)))
        d["rays"] = d["primary_rays"] + d["bounce_rays"] + d["shadow_rays"]
        return d

    def raycaster(self) -> Raycaster:
        """PathTracer::raycaster() (PathTracer.hpp:29): the scene's raycaster (not owned)."""
        return Raycaster(self.device, _handle=L.lib().pt_scene_raycaster(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pt_scene_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rank_tile_mask(height: int, width: int, ranks: int, rank: int) -> np.ndarray:
    """(H, W) bool: the pixels a rank renders under pt_render_options' split (row-major
    tiles of PT_RANK_TILE_PIXELS pixels, tile k owned by rank k % ranks)."""
    tile = np.arange(height * width, dtype=np.int64) // L.PT_RANK_TILE_PIXELS
    return (tile % max(ranks, 1) == rank).reshape(height, width)


def render_split(tracer, camera, samples: int, depth: int, image, seed: int = 0, mode: int = 0, clamp: float = 5.0,
                 fp64: bool = False, group=None, dst: int | None = None):
    """PathTracer::render split over the processes of a torch.distributed group, one GPU each
    (the reference splits image rows over threads: System::forParallel, System.hpp:72-104,
    called at PathTracer.cpp:186). Every rank holds the scene and the caller's image; it
    renders its interleaved pixel tiles (the other pixels come back as 0) and one sum over
    the ranks -- all_reduce, or reduce to rank ``dst`` -- assembles the image. Each pixel is
    rendered whole by one rank with the one-process random stream and summation order, and
    the other ranks add exact zeros, so the result equals a one-process render bit for bit.
    ``image``: (H, W, C) float32 CUDA tensor or numpy array, updated in place (on every rank
    after all_reduce, on ``dst`` after reduce). With gloo the sum runs on host copies."""
    import torch
    import torch.distributed as dist

    ranks, rank = dist.get_world_size(group), dist.get_rank(group)
    tracer.render(camera, samples, depth, image, seed=seed, mode=mode, clamp=clamp, fp64=fp64, ranks=ranks, rank=rank)
    t = image if isinstance(image, torch.Tensor) else torch.from_numpy(image)
    nccl = dist.get_backend(group) == "nccl"
    buf = t if t.is_cuda == nccl else (t.cuda() if nccl else t.cpu())
    if dst is None:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    else:
        dist.reduce(buf, dst, op=dist.ReduceOp.SUM, group=group)
    if buf is not t:
        t.copy_(buf)
    return image


def material_eval(cases):
    """MaterialGGX::eval on the device for n cases {wo.xyz, base.rgb, rough, metal, wi.xyz}."""
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 11)
    out = np.zeros((len(c), 3), np.float32)
    L.call("pt_material_eval", c.ctypes.data, len(c), out.ctypes.data, 0)
    return out


def save_image(image, path: str, tonemap: bool = True) -> None:
    """Write a render as renderOneShot does (main.cpp:106-119): ".exr" -> linear half-float
    EXR; otherwise PNG of 1 - exp(-c) (tonemap) with the reference's 8-bit sRGB conversion."""
    img = np.ascontiguousarray(image, np.float32)
    if img.ndim == 2:
        img = img[..., None]
    h, w, c = img.shape
    L.call("pt_image_save", img.ctypes.data, w, h, c, str(path).encode(), int(bool(tonemap)))


def sky_table(res: int = 512, samples: int = 256, half: bool = True, device: int = 0):
    """AtmosphereApp::precomputeTable on the device: (res, res, 4) float32."""
    out = np.zeros((res, res, 4), np.float32)
    L.call("pt_sky_table", int(res), int(samples), int(bool(half)), out.ctypes.data, int(device))
    return out


def sky_eval(cases, table=None, device: int = 0):
    """MaterialSky::eval on the device for cases (n, 9) {origin, direction, sun}; table
    (h, w, 4) float32 or None for the default table."""
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 9)
    out = np.zeros((len(c), 3), np.float32)
    if table is None:
        L.call("pt_sky_eval", None, 0, 0, c.ctypes.data, len(c), out.ctypes.data, int(device))
    else:
        t = np.ascontiguousarray(table, np.float32)
        L.call("pt_sky_eval", t.ctypes.data, t.shape[1], t.shape[0], c.ctypes.data, len(c), out.ctypes.data,
               int(device))
    return out


def material_sample(cases, uniforms):
    """MaterialGGX::sampleAndEval on the device for n cases {wo.xyz, base.rgb, rough, metal}
    with the three uniforms it draws given per case; returns (n, 6) {weight.rgb, wi.xyz}."""
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 8)
    u = np.ascontiguousarray(uniforms, np.float32).reshape(-1, 3)
    out = np.zeros((len(c), 6), np.float32)
    L.call("pt_material_sample", c.ctypes.data, u.ctypes.data, len(c), out.ctypes.data, 0)
    return out


class BatchRenderer:
    """Many renders in one call (pt_batch_render): jobs of different scenes, resolutions,
    sample counts and depths share waves run by one CUDA graph launch. Each job is a dict
    with ``tracer`` (a PathTracer), ``camera``, ``samples``, ``depth``, ``seed`` and
    ``image`` (host float32 (H, W, C) arrays, or CUDA tensors for all jobs)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        L.call("pt_batch_create", C.byref(h), int(device))
        self._h = h
        self.device = device

    @staticmethod
    def _jobs(jobs):
        arr = (L.pt_batch_job * len(jobs))()
        dev = None
        for k, j in enumerate(jobs):
            img = j["image"]
            is_dev = type(img).__module__.startswith("torch") and getattr(img, "is_cuda", False)
            if dev is None:
                dev = is_dev
            if dev != is_dev:
                raise TypeError("all images of a batch must be on the host or all on the device")
            hgt, wid, comp = img.shape
            ptr = img.data_ptr() if is_dev else img.ctypes.data
            cam = j["camera"]
            arr[k] = L.pt_batch_job(j["tracer"]._h.value, camera_desc(cam), int(j["samples"]), int(j["depth"]),
                                    int(j.get("seed", 0)), ptr, wid, hgt, comp)
        return arr, bool(dev)

    def render(self, jobs, mode: int = 0, clamp: float = 5.0, tuning=None, profile: bool = False) -> dict:
        arr, dev = self._jobs(jobs)
        opts = L.pt_render_options(int(mode), float(clamp), 0, None, 0, 0, int(bool(profile)))
        t = None if tuning is None else L.pt_batch_tuning(*(int(tuning[k]) for k in ("wave_paths", "tile_pixels",
                                                                                       "max_samples")))
        stream = None
        if dev:
            import torch

            stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        L.call("pt_batch_render", self._h, arr, len(jobs), C.byref(opts), C.byref(t) if t is not None else None,
               stream, L.RT_FLAG_DEVICE_PTRS if dev else 0)
        s = L.pt_render_stats()
        L.call("pt_batch_get_stats", self._h, C.byref(s))
        d = {k: getattr(s, k) for k, _ in s._fields_}
        d["kernel_ms"] = dict(zip(KERNEL_KINDS, list(s.kernel_ms)))
        d["rays"] = d["primary_rays"] + d["bounce_rays"] + d["shadow_rays"]
        return d

    def autotune(self, jobs, mode: int = 0, clamp: float = 5.0, cache_path: str | None = None) -> dict:
        arr, _ = self._jobs(jobs)
        opts = L.pt_render_options(int(mode), float(clamp), 0, None)
        out = L.pt_batch_tuning()
        L.call("pt_batch_autotune", self._h, arr, len(jobs), C.byref(opts),
               cache_path.encode() if cache_path else None, C.byref(out))
        return {"wave_paths": out.wave_paths, "tile_pixels": out.tile_pixels, "max_samples": out.max_samples}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pt_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
