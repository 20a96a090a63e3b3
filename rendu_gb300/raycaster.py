"""Host-side mirror of Rendu's ``Raycaster`` (src/engine/raycaster/Raycaster.hpp:10-157)
over the C-ABI ``rt_*`` entry points.

Same member names and argument meaning as the reference (``addMesh``, ``updateHierarchy``,
``intersects``, ``intersectsAny``, ``visible``, ``interpolateAttribute``, ``Hit``), plus the
batched forms that are the fast path (``intersect_batch``, ``intersect_any_batch``,
``visible_batch``). Batches are numpy arrays (host; copied through the library) or CUDA
torch tensors (device; no copy, launched on torch's current stream).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

RAY_DTYPE = np.dtype([("ox", "<f4"), ("oy", "<f4"), ("oz", "<f4"), ("tmin", "<f4"), ("dx", "<f4"), ("dy", "<f4"),
                      ("dz", "<f4"), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])
FLT_MAX = float(np.finfo(np.float32).max)


@dataclass
class Hit:
    """Raycaster::Hit (Raycaster.hpp:16-42)."""

    hit: bool = False
    dist: float = FLT_MAX
    u: float = 0.0
    v: float = 0.0
    w: float = 0.0
    localId: int = 0
    meshId: int = 0


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _torch_stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _colmajor(model):
    if model is None:
        return None
    m = np.asarray(model, np.float32).reshape(4, 4)
    return np.ascontiguousarray(m.T.reshape(16))


class Raycaster:
    """Device BVH raycaster with the reference's API (one CUDA device per instance)."""

    def __init__(self, device: int = 0, _handle=None):
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            L.call("rt_create", C.byref(h), int(device))
            self._h = h
        else:
            self._h = C.c_void_p(_handle)
        self.device = device
        self._meshes = []  # (first_tri, tri_count) per mesh

    # ---- construction (Raycaster.cpp:14-142) ------------------------------------------
    def addMesh(self, mesh, model=None) -> int:
        """Raycaster::addMesh(mesh, model): ``mesh`` has ``positions`` (V,3) and ``indices``."""
        return self.add_mesh(mesh.positions, mesh.indices, model)

    def add_mesh(self, positions, indices, model=None) -> int:
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        m = _colmajor(model)
        mid = C.c_uint32()
        L.call("rt_add_mesh", self._h, pos.ctypes.data, len(pos) // 3, idx.ctypes.data, len(idx),
               m.ctypes.data if m is not None else None, C.byref(mid))
        first = sum(c for _, c in self._meshes)
        self._meshes.append((first, len(idx) // 3))
        return mid.value

    def updateHierarchy(self):
        """Raycaster::updateHierarchy (Raycaster.cpp:54-142): builds the device hierarchy."""
        L.call("rt_update_hierarchy", self._h)

    update_hierarchy = updateHierarchy

    # ---- single-ray API (Raycaster.hpp:57-83) ------------------------------------------
    def intersects(self, origin, direction, mini: float = 1e-4, maxi: float = 1e8) -> Hit:
        ray = np.zeros(1, RAY_DTYPE)
        ray[0] = (*origin, mini, *direction, maxi)
        h = self.intersect_batch(ray)[0]
        return self.to_hit(h)

    def intersectsAny(self, origin, direction, mini: float = 1e-4, maxi: float = 1e8) -> bool:
        ray = np.zeros(1, RAY_DTYPE)
        ray[0] = (*origin, mini, *direction, maxi)
        return bool(self.intersect_any_batch(ray)[0])

    def visible(self, p0, p1) -> bool:
        seg = np.asarray([*p0, *p1], np.float32).reshape(1, 6)
        return bool(self.visible_batch(seg)[0])

    def to_hit(self, h) -> Hit:
        prim = int(h["prim"])
        if prim == L.RT_NO_HIT:
            return Hit()
        mesh_id, local_id = self.prim_info(prim)
        u, v = float(h["u"]), float(h["v"])
        w = float(np.float32(np.float32(1.0) - np.float32(u)) - np.float32(v))
        return Hit(True, float(h["t"]), u, v, w, local_id, mesh_id)

    @staticmethod
    def interpolateAttribute(hit: Hit, mesh, attribute):
        """Raycaster::interpolateAttribute (Raycaster.hpp:90-97): w*A[i0] + u*A[i1] + v*A[i2]."""
        i0, i1, i2 = (int(mesh.indices[hit.localId + k]) for k in range(3))
        a = np.asarray(attribute, np.float32)
        return np.float32(hit.w) * a[i0] + np.float32(hit.u) * a[i1] + np.float32(hit.v) * a[i2]

    # ---- batched API --------------------------------------------------------------------
    def intersect_batch(self, rays, out=None):
        """Closest hits for rays: (n,8) float32 / RAY_DTYPE numpy (host) or a CUDA tensor
        (n,8) float32 (device). Returns HIT_DTYPE numpy or an (n,4) float32 CUDA tensor
        whose last column holds the triangle id bits."""
        if _is_torch_cuda(rays):
            import torch

            n = rays.shape[0]
            if out is None:
                out = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
            L.call("rt_intersect", self._h, C.c_void_p(rays.data_ptr()), n, C.c_void_p(out.data_ptr()),
                   _torch_stream(), L.RT_FLAG_DEVICE_PTRS)
            return out
        r = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
        n = len(r)
        if out is None:
            out = np.empty(n, HIT_DTYPE)
        L.call("rt_intersect", self._h, r.ctypes.data, n, out.ctypes.data, None, 0)
        return out

    def intersect_any_batch(self, rays, out=None):
        if _is_torch_cuda(rays):
            import torch

            n = rays.shape[0]
            if out is None:
                out = torch.empty(n, dtype=torch.uint8, device=rays.device)
            L.call("rt_intersect_any", self._h, C.c_void_p(rays.data_ptr()), n, C.c_void_p(out.data_ptr()),
                   _torch_stream(), L.RT_FLAG_DEVICE_PTRS)
            return out
        r = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
        if out is None:
            out = np.empty(len(r), np.uint8)
        L.call("rt_intersect_any", self._h, r.ctypes.data, len(r), out.ctypes.data, None, 0)
        return out

    def visible_batch(self, segs):
        s = np.ascontiguousarray(segs, np.float32).reshape(-1, 6)
        out = np.empty(len(s), np.uint8)
        L.call("rt_visible", self._h, s.ctypes.data, len(s), out.ctypes.data, None, 0)
        return out

    def count_visits(self, rays):
        r = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
        nv = np.empty(len(r), np.uint32)
        nt = np.empty(len(r), np.uint32)
        L.call("rt_count_visits", self._h, r.ctypes.data, len(r), nv.ctypes.data, nt.ctypes.data, None, 0)
        return nv, nt

    def prim_info(self, prim: int):
        m = C.c_uint32()
        lid = C.c_uint32()
        L.call("rt_prim_info", self._h, int(prim), C.byref(m), C.byref(lid))
        return m.value, lid.value

    def stats(self) -> dict:
        s = L.rt_stats()
        L.call("rt_get_stats", self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in s._fields_}

    @property
    def handle(self):
        return self._h.value

    def close(self):
        if self._owned and self._h is not None and self._h.value:
            L.lib().rt_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
