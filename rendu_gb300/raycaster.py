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
        self._mesh_data = []  # (positions, indices, model) per mesh, for triangle()

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
        self._mesh_data.append((pos, idx, None if model is None else np.asarray(model, np.float32).reshape(4, 4)))
        return mid.value

    def triangle(self, mesh_id: int, local_id: int) -> np.ndarray:
        """The three vertices (3, 3) of triangle localId / 3 of a mesh, transformed by its model
        matrix as addMesh stores them (Raycaster.cpp:22-36)."""
        pos, idx, model = self._mesh_data[mesh_id]
        v = pos.reshape(-1, 3)[idx[local_id:local_id + 3]].astype(np.float32)
        if model is None:
            return v
        m = model
        out = np.empty_like(v)
        for k in range(3):  # glm's mat4 * vec4(p, 1) in column order
            out[:, k] = ((m[k, 0] * v[:, 0] + m[k, 1] * v[:, 1]) + m[k, 2] * v[:, 2]) + m[k, 3]
        return out

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

    def hit_info(self, hits):
        """(meshId, localId) of every hit of a batch (Raycaster::Hit's fields), RT_NO_HIT on
        misses: HIT_DTYPE numpy in -> two uint32 numpy arrays; an (n,4) CUDA tensor from
        intersect_batch -> two int32 CUDA tensors holding the uint32 bits."""
        if _is_torch_cuda(hits):
            import torch

            n = hits.shape[0]
            m = torch.empty(n, dtype=torch.int32, device=hits.device)
            lid = torch.empty(n, dtype=torch.int32, device=hits.device)
            L.call("rt_hit_info", self._h, C.c_void_p(hits.data_ptr()), n, C.c_void_p(m.data_ptr()),
                   C.c_void_p(lid.data_ptr()), _torch_stream(), L.RT_FLAG_DEVICE_PTRS)
            return m, lid
        h = np.ascontiguousarray(hits)
        m = np.empty(len(h), np.uint32)
        lid = np.empty(len(h), np.uint32)
        L.call("rt_hit_info", self._h, h.ctypes.data, len(h), m.ctypes.data, lid.ctypes.data, None, 0)
        return m, lid

    def status(self, stream=None) -> int:
        """Read and clear the failures of asynchronous (device-pointer) calls ordered on
        `stream` (the current torch stream by default): RT_OK, RT_ERR_OVERFLOW or
        RT_ERR_TIMEOUT, as rt_get_status returns it."""
        word = C.c_uint32()
        st = _torch_stream() if stream is None else C.c_void_p(stream)
        return L.lib().rt_get_status(self._h, st, C.byref(word))

    def set_traversal_stack(self, entries: int):
        """Cap the traversal stack (0 = the hierarchy's exact bound); see rt_set_traversal_stack."""
        L.call("rt_set_traversal_stack", self._h, int(entries))

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


# ---- hierarchy display geometry -------------------------------------------------------------

# the 12 edges of a box as degenerate triangles over BoundingBox::getCorners' corner order
# (x slowest, z fastest) -- RaycasterVisualisation.cpp:128-129
_BOX_LINES = np.array([0, 1, 0, 0, 2, 0, 1, 3, 1, 2, 3, 2, 4, 5, 4, 4, 6, 4, 5, 7, 5, 6, 7, 6, 1, 5, 1, 0, 4, 0, 2, 6,
                       2, 3, 7, 3], np.uint32)


def _hsv_to_rgb(h: float, s: float, v: float) -> np.ndarray:
    """Hue in degrees, saturation and value to RGB (single precision)."""
    h, s, v = np.float32(h), np.float32(s), np.float32(v)
    if s == 0:
        return np.array([v, v, v], np.float32)
    sector = np.floor(h * (np.float32(1) / np.float32(60)))
    frac = h * (np.float32(1) / np.float32(60)) - sector
    o = v * (np.float32(1) - s)
    p = v * (np.float32(1) - s * frac)
    q = v * (np.float32(1) - s * (np.float32(1) - frac))
    table = {1: (p, v, o), 2: (o, v, q), 3: (o, p, v), 4: (q, o, v), 5: (v, o, p)}
    return np.array(table.get(int(sector), (v, q, o)), np.float32)


def _box_meshes(boxes: np.ndarray, depths: np.ndarray) -> list:
    """createBVHMeshes (RaycasterVisualisation.cpp:107-157): one line mesh per depth, every
    box as its 8 corners and 12 edges, coloured by relative depth (hue 300 depth^2,
    value 0.75 - 0.5 depth^2)."""
    if len(boxes) == 0:
        return []
    max_depth = int(depths.max())
    meshes = []
    for d in range(max_depth + 1):
        sel = boxes[depths == d]
        lo, hi = sel[:, :3], sel[:, 3:]
        corners = np.stack([np.where([(k >> 2) & 1, (k >> 1) & 1, k & 1], hi, lo) for k in range(8)], 1)
        rel = np.float32(d) / np.float32(max_depth) if max_depth else np.float32(0)
        rel = rel * rel
        color = _hsv_to_rgb(np.float32(300) * rel, 1.0, np.float32(0.5) * (np.float32(1) - rel) + np.float32(0.25))
        idx = (np.arange(len(sel), dtype=np.uint32)[:, None] * 8 + _BOX_LINES[None, :]).reshape(-1)
        meshes.append({"name": f"Level {d}", "positions": corners.reshape(-1, 3).astype(np.float32), "indices": idx,
                       "colors": np.tile(color, (len(sel) * 8, 1))})
    return meshes


class RaycasterVisualisation:
    """RaycasterVisualisation (src/engine/raycaster/RaycasterVisualisation.hpp) over the
    device hierarchy: line meshes of node boxes by depth, for display or for writing out
    with ``save_line_obj``. The boxes are those of this library's 4-wide hierarchy."""

    def __init__(self, raycaster: Raycaster):
        self._rc = raycaster

    def _call(self, func, *args):
        """Two calls of a box query: the count, then the boxes, their info and the hit."""
        count = C.c_size_t()
        hit = np.zeros(1, HIT_DTYPE)
        extra = [] if func == "rt_hierarchy_boxes" else [hit.ctypes.data]
        L.call(func, self._rc._h, *args, None, None, 0, C.byref(count), *extra)
        n = count.value
        boxes = np.zeros((n, 6), np.float32)
        info = np.zeros((n, 2), np.int32)
        L.call(func, self._rc._h, *args, boxes.ctypes.data, info.ctypes.data, n, C.byref(count), *extra)
        return boxes, info, hit[0]

    def getAllLevels(self) -> list:
        """Every node of the hierarchy (getAllLevels, RaycasterVisualisation.cpp:9-33)."""
        boxes, info, _ = self._call("rt_hierarchy_boxes")
        return _box_meshes(boxes, info[:, 0])

    def getRayLevels(self, origin, direction, mini: float = 1e-4, maxi: float = 1e8):
        """The boxes a ray enters and its closest hit (getRayLevels, RaycasterVisualisation.cpp:
        35-81): (line meshes, Hit)."""
        ray = np.zeros(1, RAY_DTYPE)
        ray[0] = (*origin, mini, *direction, maxi)
        boxes, info, hit = self._call("rt_ray_levels", ray.ctypes.data)
        return _box_meshes(boxes, info[:, 0]), self._rc.to_hit(hit)

    def getRayMesh(self, ray_pos, ray_dir, hit: Hit, default_length: float = 1.0) -> dict:
        """getRayMesh (RaycasterVisualisation.cpp:83-105): the ray segment up to the hit (or
        default_length), green when it hit and red otherwise, plus the hit triangle."""
        d = np.asarray(ray_dir, np.float32)
        d = d * (np.float32(1) / np.sqrt(np.float32((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])))
        length = np.float32(hit.dist if hit.hit else default_length)
        p0 = np.asarray(ray_pos, np.float32)
        color = np.array([0.0, 1.0, 0.0] if hit.hit else [1.0, 0.0, 0.0], np.float32)
        pos = [p0, p0 + length * d]
        idx = [0, 1, 0]
        if hit.hit:
            pos += list(self._rc.triangle(hit.meshId, hit.localId))
            idx += [2, 3, 4]
        return {"name": "Ray", "positions": np.asarray(pos, np.float32), "indices": np.asarray(idx, np.uint32),
                "colors": np.tile(color, (len(pos), 1))}


def save_line_obj(meshes: list, path: str) -> None:
    """Write line meshes (degenerate-triangle edges) as an OBJ of 'l' records, one group per
    mesh, with the colour appended to each vertex (a common OBJ extension)."""
    with open(path, "w") as f:
        base = 1
        for m in meshes:
            f.write(f"g {m['name'].replace(' ', '_')}\n")
            for p, c in zip(m["positions"], m["colors"]):
                f.write(f"v {p[0]:.6g} {p[1]:.6g} {p[2]:.6g} {c[0]:.4g} {c[1]:.4g} {c[2]:.4g}\n")
            tri = m["indices"].reshape(-1, 3)
            for a, b, _ in tri:
                f.write(f"l {a + base} {b + base}\n")
            base += len(m["positions"])
