"""Seeded synthetic inputs for the raycaster and path-tracer workloads.

The reference ships no benchmark data; its hot path is exercised here on procedural
inputs whose shapes follow the reference's own scene model:
  * triangle meshes as position/normal/tangent/bitangent/texcoord/index arrays
    (Mesh.hpp:126-132 of kosua20/Rendu), transformed by per-object model matrices
    (Object.hpp:59);
  * materials of type Regular (Lambert+GGX) or Emissive with three constant-colour
    textures, the convention the reference uses for colour-only materials
    (ResourcesManager.cpp:489-505: 8x8 float images);
  * a pinhole camera given as eye/center/up/fov/ratio (Camera.cpp:10-49).

Workloads
  * ``icosphere_mesh(8)`` + ``random_rays`` -- the raycaster workload: a subdivided
    icosphere (1,310,720 triangles at 8 subdivisions) radially displaced by 3-octave
    value noise of amplitude 0.1, and rays with origins uniform in a box three times
    the mesh bounds and directions uniform on the sphere.
  * ``cornell_scene`` -- the small path-tracer workload: a 5-wall room (10 triangles),
    two boxes rotated by a seeded angle (24 triangles) and a 2-triangle emissive ceiling
    quad of radiance 15.
  * ``instanced_scene`` -- the large path-tracer workload: displaced icospheres and
    boxes on a ground plane, about 2M triangles in 200 instances, emissive quads and a
    procedural sky environment.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# --------------------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------------------


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array(
        [
            [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
            [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
            [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1],
        ],
        dtype=np.float64,
    )
    f = np.array(
        [
            [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
            [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
            [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
            [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
        ],
        dtype=np.int64,
    )
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, f


def _subdivide(v, f):
    """One 4-to-1 subdivision with shared edge midpoints, projected on the unit sphere."""
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    e_sorted = np.sort(e, axis=1)
    key = e_sorted[:, 0] * (len(v) + 1) + e_sorted[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a = uniq // (len(v) + 1)
    b = uniq % (len(v) + 1)
    mid = v[a] + v[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    nf = len(f)
    m01 = len(v) + inv[:nf]
    m12 = len(v) + inv[nf : 2 * nf]
    m20 = len(v) + inv[2 * nf :]
    v2 = np.concatenate([v, mid], axis=0)
    f2 = np.concatenate(
        [
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1),
        ],
        axis=0,
    )
    return v2, f2


class ValueNoise:
    """Seeded 3-D value noise: random values on an integer lattice (hashed, period 256),
    trilinear interpolation with a smoothstep fade; ``octaves`` summed with halving
    amplitude and doubling frequency, normalised to [-1, 1]."""

    def __init__(self, seed: int, octaves: int = 3, base_freq: float = 2.0):
        rng = np.random.default_rng(seed)
        self.table = rng.uniform(-1.0, 1.0, size=256 * 256 * 256 // 64).astype(np.float64)
        self.perm = rng.permutation(256).astype(np.int64)
        self.octaves = octaves
        self.base_freq = base_freq

    def _lattice(self, i, j, k):
        h = self.perm[(self.perm[(self.perm[i & 255] + j) & 255] + k) & 255]
        h2 = self.perm[(h + i * 7 + j * 13 + k * 17) & 255]
        return self.table[(h * 256 + h2) % len(self.table)]

    def _octave(self, p):
        fl = np.floor(p)
        i = fl.astype(np.int64)
        f = p - fl
        s = f * f * (3.0 - 2.0 * f)
        out = 0.0
        for dx in (0, 1):
            wx = s[:, 0] if dx else 1.0 - s[:, 0]
            for dy in (0, 1):
                wy = s[:, 1] if dy else 1.0 - s[:, 1]
                for dz in (0, 1):
                    wz = s[:, 2] if dz else 1.0 - s[:, 2]
                    out = out + wx * wy * wz * self._lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
        return out

    def __call__(self, p):
        total = np.zeros(len(p))
        amp, freq, norm = 1.0, self.base_freq, 0.0
        for _ in range(self.octaves):
            total += amp * self._octave(p * freq)
            norm += amp
            amp *= 0.5
            freq *= 2.0
        return total / norm


@dataclass
class Mesh:
    """Vertex attributes + triangle indices, the layout of the reference's Mesh."""

    positions: np.ndarray  # (V,3) float32
    indices: np.ndarray  # (3T,) uint32
    normals: np.ndarray | None = None
    tangents: np.ndarray | None = None
    bitangents: np.ndarray | None = None
    texcoords: np.ndarray | None = None

    @property
    def triangle_count(self) -> int:
        return len(self.indices) // 3

    def with_frames(self) -> "Mesh":
        """Fill area-weighted vertex normals and an orthonormal tangent frame (the path
        tracer needs normals, tangents and bitangents on every mesh, PathTracer.cpp:14-16)."""
        p = self.positions.astype(np.float64)
        f = self.indices.reshape(-1, 3).astype(np.int64)
        n = np.zeros_like(p)
        fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
        for k in range(3):
            np.add.at(n, f[:, k], fn)
        ln = np.linalg.norm(n, axis=1, keepdims=True)
        ln[ln == 0] = 1.0
        n /= ln
        ref = np.where(np.abs(n[:, 1:2]) < 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
        t = np.cross(ref, n)
        t /= np.linalg.norm(t, axis=1, keepdims=True)
        b = np.cross(n, t)
        self.normals = n.astype(np.float32)
        self.tangents = t.astype(np.float32)
        self.bitangents = b.astype(np.float32)
        return self


def icosphere_mesh(subdivisions: int, radius: float = 1.0, displacement: float = 0.1, seed: int = 0,
                   octaves: int = 3) -> Mesh:
    """Icosphere with 20 * 4^subdivisions triangles, vertices moved along the radius by
    ``displacement`` x seeded value noise (3 octaves)."""
    v, f = _icosahedron()
    for _ in range(subdivisions):
        v, f = _subdivide(v, f)
    if displacement:
        noise = ValueNoise(seed, octaves=octaves)
        v = v * (radius * (1.0 + displacement * noise(v)))[:, None]
    else:
        v = v * radius
    return Mesh(v.astype(np.float32), f.reshape(-1).astype(np.uint32))


def box_mesh(size=(1.0, 1.0, 1.0)) -> Mesh:
    """Axis-aligned box centred on the origin, 12 triangles, 24 vertices (flat faces)."""
    sx, sy, sz = (0.5 * s for s in size)
    faces = [
        ([1, 0, 0], [0, 0, -1]), ([-1, 0, 0], [0, 0, 1]),
        ([0, 1, 0], [1, 0, 0]), ([0, -1, 0], [1, 0, 0]),
        ([0, 0, 1], [1, 0, 0]), ([0, 0, -1], [-1, 0, 0]),
    ]
    pos, nrm, tan, bit, uv, idx = [], [], [], [], [], []
    for n, t in faces:
        n = np.array(n, float)
        t = np.array(t, float)
        b = np.cross(n, t)
        c = n * np.array([sx, sy, sz])
        base = len(pos)
        for du, dv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            pos.append(c + du * t * np.array([sx, sy, sz]) + dv * b * np.array([sx, sy, sz]))
            nrm.append(n)
            tan.append(t)
            bit.append(b)
            uv.append([(du + 1) * 0.5, (dv + 1) * 0.5])
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    return Mesh(
        np.array(pos, np.float32), np.array(idx, np.uint32), np.array(nrm, np.float32),
        np.array(tan, np.float32), np.array(bit, np.float32), np.array(uv, np.float32),
    )


def quad_mesh(corner, edge_u, edge_v, normal=None) -> Mesh:
    """Two-triangle quad corner, corner+u, corner+u+v, corner+v."""
    c = np.asarray(corner, float)
    u = np.asarray(edge_u, float)
    v = np.asarray(edge_v, float)
    n = np.cross(u, v) if normal is None else np.asarray(normal, float)
    n = n / np.linalg.norm(n)
    t = u / np.linalg.norm(u)
    b = np.cross(n, t)
    pos = np.array([c, c + u, c + u + v, c + v], np.float32)
    return Mesh(
        pos, np.array([0, 1, 2, 0, 2, 3], np.uint32), np.tile(n, (4, 1)).astype(np.float32),
        np.tile(t, (4, 1)).astype(np.float32), np.tile(b, (4, 1)).astype(np.float32),
        np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32),
    )


# --------------------------------------------------------------------------------------
# rays
# --------------------------------------------------------------------------------------


def random_rays(n: int, lo, hi, seed: int, scale: float = 3.0, tmin: float = 1e-4, tmax: float = 1e8) -> np.ndarray:
    """n rays as an (n, 8) float32 array {o.xyz, tmin, d.xyz, tmax}: origins uniform in
    the box ``scale`` times the [lo, hi] bounds about their centre, directions uniform on
    the unit sphere (z = 2u - 1, phi = 2 pi v)."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    h = 0.5 * (hi - lo) * scale
    rays = np.empty((n, 8), np.float32)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        o = c + (rng.random((m, 3)) * 2.0 - 1.0) * h
        z = rng.random(m) * 2.0 - 1.0
        phi = rng.random(m) * 2.0 * math.pi
        r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        rays[s : s + m, 0:3] = o
        rays[s : s + m, 3] = tmin
        rays[s : s + m, 4] = r * np.cos(phi)
        rays[s : s + m, 5] = r * np.sin(phi)
        rays[s : s + m, 6] = z
        rays[s : s + m, 7] = tmax
    return rays


def raycaster_workload(subdivisions: int = 8, n_rays: int = 1 << 24, seed: int = 20261204):
    """The raycaster workload: displaced icosphere (1,310,720 triangles at 8 subdivisions)
    and ``n_rays`` rays (16,777,216 by default)."""
    mesh = icosphere_mesh(subdivisions, seed=seed)
    lo = mesh.positions.min(0)
    hi = mesh.positions.max(0)
    rays = random_rays(n_rays, lo, hi, seed + 1)
    return mesh, rays


# --------------------------------------------------------------------------------------
# path-tracer scenes
# --------------------------------------------------------------------------------------


def rotation_y(angle: float) -> np.ndarray:
    c, s = math.cos(angle), math.sin(angle)
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def translation(t) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = t
    return m


def scaling(s) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[1, 1], m[2, 2] = (s, s, s) if np.isscalar(s) else s
    return m


def constant_texture(rgba, size: int = 8) -> np.ndarray:
    """A size x size RGBA float image of one colour (the reference's colour textures)."""
    return np.tile(np.asarray(rgba, np.float32), (size, size, 1))


@dataclass
class Scene:
    """In-memory scene: textures, meshes, materials, objects, lights, background, camera.
    Matrices are row-major numpy 4x4 here and passed column-major across the C-ABI."""

    textures: list = field(default_factory=list)  # (H, W, C) float32 arrays
    meshes: list = field(default_factory=list)  # Mesh
    materials: list = field(default_factory=list)  # dict(type, masked, tex=(a, n, r))
    objects: list = field(default_factory=list)  # dict(mesh, material, model)
    lights: list = field(default_factory=list)  # dict(type, color, position, direction, radius, inner, outer, shadows)
    background: dict = field(default_factory=lambda: {"mode": 0, "color": (0.0, 0.0, 0.0), "tex": (0,) * 6})
    camera: dict = field(default_factory=dict)
    environment: dict | None = None  # {"tex": id, "intensity": s}: equirect map of the extended estimator

    def add_texture(self, img) -> int:
        self.textures.append(np.ascontiguousarray(img, np.float32))
        return len(self.textures) - 1

    def add_material(self, albedo, rough=1.0, metal=0.0, emissive=False, masked=False, normal_tex=None,
                     albedo_tex=None) -> int:
        """A Regular (Lambert+GGX) or Emissive material from constant colours, or from a
        given albedo / normal-map texture id."""
        a = albedo_tex if albedo_tex is not None else self.add_texture(constant_texture(list(albedo) + [1.0]))
        n = normal_tex if normal_tex is not None else self.add_texture(constant_texture([0.5, 0.5, 1.0, 1.0]))
        r = self.add_texture(constant_texture([rough, metal, 1.0, 1.0]))
        self.materials.append({"type": 8 if emissive else 1, "masked": bool(masked), "tex": (a, n, r)})
        return len(self.materials) - 1

    def add_mesh(self, mesh: Mesh) -> int:
        if mesh.normals is None:
            mesh.with_frames()
        self.meshes.append(mesh)
        return len(self.meshes) - 1

    def add_object(self, mesh: int, material: int, model=None) -> int:
        self.objects.append({"mesh": mesh, "material": material,
                             "model": np.eye(4, dtype=np.float32) if model is None else np.asarray(model, np.float32)})
        return len(self.objects) - 1

    @property
    def triangle_count(self) -> int:
        return sum(self.meshes[o["mesh"]].triangle_count for o in self.objects)


def cornell_scene(seed: int = 20261204, with_light: bool = False) -> Scene:
    """Cornell-style room: 5 axis-aligned walls (10 triangles), 2 boxes rotated about y by
    seeded angles in [0, 45 deg] (24 triangles), a 2-triangle emissive ceiling quad of
    radiance 15. Lambert walls/boxes (Regular, roughness 1, metalness 0) with seeded albedo
    in [0.2, 0.8]^3; the second box is GGX with roughness 0.3. No analytic light unless
    ``with_light`` (then one shadowed point light, to exercise next-event estimation)."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    L = 2.0
    walls = [
        ((-1, 0, -1), (2, 0, 0), (0, 0, 2)),  # floor, faces +y
        ((-1, 2, 1), (2, 0, 0), (0, 0, -2)),  # ceiling, faces -y
        ((-1, 0, -1), (0, 2, 0), (2, 0, 0)),  # back wall z=-1, faces +z
        ((-1, 0, 1), (0, 2, 0), (0, 0, -2)),  # left wall x=-1, faces +x
        ((1, 0, -1), (0, 2, 0), (0, 0, 2)),  # right wall x=1, faces -x
    ]
    for c, u, v in walls:
        m = sc.add_mesh(quad_mesh(c, u, v))
        mat = sc.add_material(rng.uniform(0.2, 0.8, 3), rough=1.0, metal=0.0)
        sc.add_object(m, mat)
    for k, (pos, size, rough) in enumerate((((-0.35, 0.6, -0.3), (0.55, 1.2, 0.55), 1.0),
                                            ((0.4, 0.3, 0.35), (0.6, 0.6, 0.6), 0.3))):
        m = sc.add_mesh(box_mesh(size))
        mat = sc.add_material(rng.uniform(0.2, 0.8, 3), rough=rough, metal=0.0)
        angle = math.radians(rng.uniform(0.0, 45.0))
        sc.add_object(m, mat, translation(pos) @ rotation_y(angle))
    lm = sc.add_mesh(quad_mesh((-0.3, 1.999, 0.3), (0.6, 0, 0), (0, 0, -0.6)))
    lmat = sc.add_material((15.0, 15.0, 15.0), emissive=True)
    sc.add_object(lm, lmat)
    if with_light:
        sc.lights.append({"type": 0, "color": (2.0, 2.0, 2.0), "position": (0.0, 1.6, 0.5), "direction": (0, -1, 0),
                          "radius": 4.0, "inner": 0.5, "outer": 0.8, "shadows": True})
    sc.background = {"mode": 0, "color": (0.0, 0.0, 0.0), "tex": (0,) * 6}
    sc.camera = {"eye": (0.0, 1.0, 3.4), "center": (0.0, 1.0, 0.0), "up": (0.0, 1.0, 0.0), "fov": 1.3, "ratio": 1.0}
    _ = L
    return sc


def _checker(n, c0, c1, cells=4):
    ij = np.indices((n, n)).sum(0) // max(1, n // cells)
    img = np.where((ij % 2)[..., None] == 0, np.asarray(c0, np.float32), np.asarray(c1, np.float32))
    return img.astype(np.float32)


def feature_scene(seed: int = 20261204) -> Scene:
    """A small scene exercising every shading feature of the reference path tracer:
    textured albedo with wrapped texture coordinates, a normal map, an alpha cut-out
    (masked) quad, a metallic GGX sphere without texture coordinates, an emissive quad,
    point/spot lights with shadows and a directional light without, and a SKYBOX
    (cubemap) background seen by every bounce."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    # Ground: checker albedo, UVs scaled x3 so that sampling wraps.
    g = quad_mesh((-2, 0, -2), (4, 0, 0), (0, 0, 4))
    g.texcoords = g.texcoords * 3.0
    alb = sc.add_texture(_checker(16, (0.8, 0.8, 0.8, 1.0), (0.2, 0.3, 0.6, 1.0)))
    gm = sc.add_material(None, rough=0.7, metal=0.0, albedo_tex=alb)
    sc.add_object(sc.add_mesh(g), gm)
    # Box with a bumpy normal map.
    nrm = rng.normal(0.0, 0.25, (8, 8, 3))
    nrm[..., 2] = 1.0
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    ntex = sc.add_texture(np.concatenate([0.5 * nrm + 0.5, np.ones((8, 8, 1))], 2).astype(np.float32))
    bm = sc.add_material((0.7, 0.4, 0.2), rough=0.5, metal=0.0, normal_tex=ntex)
    sc.add_object(sc.add_mesh(box_mesh((0.6, 0.6, 0.6))), bm, translation((-0.7, 0.3, -0.2)) @ rotation_y(0.5))
    # Metallic sphere without texture coordinates.
    sph = icosphere_mesh(3, seed=seed, displacement=0.0)
    sph.with_frames()
    sm = sc.add_material((0.9, 0.8, 0.5), rough=0.2, metal=1.0)
    sc.add_object(sc.add_mesh(sph), sm, translation((0.6, 0.45, 0.1)) @ scaling(0.45))
    # Alpha cut-out quad (checker alpha).
    cut = quad_mesh((-1.5, 0.0, 0.8), (1.2, 0, 0), (0, 1.2, 0))
    ctex = sc.add_texture(_checker(8, (0.3, 0.8, 0.3, 1.0), (0.3, 0.8, 0.3, 0.0), cells=4))
    cm = sc.add_material(None, rough=0.9, metal=0.0, masked=True, albedo_tex=ctex)
    sc.add_object(sc.add_mesh(cut), cm, rotation_y(0.3))
    # Small emitter.
    em = sc.add_material((4.0, 3.5, 3.0), emissive=True)
    sc.add_object(sc.add_mesh(quad_mesh((0.2, 1.6, -0.8), (0.5, 0, 0), (0, 0, 0.5))), em)
    sc.lights += [
        {"type": 0, "color": (3.0, 3.0, 3.0), "position": (0.5, 1.8, 1.0), "radius": 6.0, "shadows": True},
        {"type": 2, "color": (4.0, 4.0, 3.0), "position": (-1.0, 2.0, 1.5), "direction": (0.4, -1.0, -0.6),
         "radius": 8.0, "inner": 0.6, "outer": 1.2, "shadows": True},
        {"type": 1, "color": (0.6, 0.6, 0.7), "direction": (-0.3, -1.0, -0.2), "shadows": False},
    ]
    faces = []
    for f in range(6):
        base = np.array([0.2 + 0.1 * f, 0.3, 0.5 - 0.05 * f], np.float32)
        ramp = np.linspace(0.5, 1.5, 8, dtype=np.float32)[:, None, None]
        faces.append(sc.add_texture(np.broadcast_to(base * ramp, (8, 8, 3)).copy()))
    sc.background = {"mode": 2, "color": (0, 0, 0), "tex": tuple(faces)}
    sc.camera = {"eye": (0.0, 1.2, 3.0), "center": (0.0, 0.4, 0.0), "up": (0.0, 1.0, 0.0), "fov": 1.1, "ratio": 1.0}
    return sc


def sky_equirect(width: int = 1024, height: int = 512, sun_dir=(0.4, 0.55, -0.5), sun_radiance: float = 5e4,
                 sun_radius: float = 0.02) -> np.ndarray:
    """Synthetic HDR environment (equirectangular, float32 RGB): a sky gradient from a
    horizon colour to a zenith colour, a darker ground half, and a sun disc of the given
    radiance and angular radius (radians)."""
    j, i = np.meshgrid(np.arange(width), np.arange(height))
    phi = (j + 0.5) / width * 2 * np.pi
    theta = (i + 0.5) / height * np.pi
    d = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], -1)
    return _sky_radiance(d, sun_dir, sun_radiance, sun_radius).astype(np.float32)


def _sky_radiance(d, sun_dir, sun_radiance, sun_radius):
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    up = np.clip(d[..., 1], -1.0, 1.0)
    t = np.clip(up, 0.0, 1.0)[..., None]
    horizon = np.array([0.9, 0.85, 0.8])
    zenith = np.array([0.25, 0.45, 0.9])
    ground = np.array([0.25, 0.22, 0.2])
    col = np.where(up[..., None] >= 0.0, horizon * (1 - t) + zenith * t, ground * (0.5 + 0.5 * (1 + up[..., None])))
    cosang = d @ s
    col = col + np.where(cosang[..., None] > np.cos(sun_radius), sun_radiance, 0.0)
    return col


def equirect_to_cubemap(env: np.ndarray, face: int = 256):
    """Resample an equirectangular map into the six faces (+x,-x,+y,-y,+z,-z) in the
    orientation Texture::sampleCubemap reads them (Texture.cpp:141-191): face texel (x, y)
    looks along the direction whose projection onto that face gives u = x, v = y."""
    h, w = env.shape[:2]
    c = (np.arange(face) + 0.5) / face * 2.0 - 1.0  # [-1, 1]
    xs, ys = np.meshgrid(c, c)  # xs: column (u), ys: row (v); v = 0.5*(-y/denom)+0.5 -> y = -v
    faces = []
    for f in range(6):
        u, v = xs, ys
        if f == 0:
            d = np.stack([np.ones_like(u), -v, -u], -1)
        elif f == 1:
            d = np.stack([-np.ones_like(u), -v, u], -1)
        elif f == 2:
            d = np.stack([u, np.ones_like(u), v], -1)
        elif f == 3:
            d = np.stack([u, -np.ones_like(u), -v], -1)
        elif f == 4:
            d = np.stack([u, -v, np.ones_like(u)], -1)
        else:
            d = np.stack([-u, -v, -np.ones_like(u)], -1)
        d = d / np.linalg.norm(d, axis=-1, keepdims=True)
        theta = np.arccos(np.clip(d[..., 1], -1, 1))
        phi = np.mod(np.arctan2(d[..., 2], d[..., 0]), 2 * np.pi)
        px = np.clip((phi / (2 * np.pi) * w).astype(np.int64), 0, w - 1)
        py = np.clip((theta / np.pi * h).astype(np.int64), 0, h - 1)
        faces.append(np.ascontiguousarray(env[py, px], np.float32))
    return faces


def instanced_scene(seed: int = 20261206, instances: int = 200, subdivisions: int = 5, prototypes: int = 6,
                    env_face: int = 256) -> Scene:
    """The large path-tracer workload: `instances` seeded instances, alternating displaced
    icospheres (20,480 triangles at 5 subdivisions) and boxes, on a 2-triangle ground plane
    (~2M triangles at 200 instances). Materials: GGX roughness U[0.05, 1], metalness
    Bernoulli(0.3), base colour U[0.2, 0.9]^3. Four emissive quads. Background: a synthetic
    1024x512 HDR sky (gradient + sun disc of radiance 5e4) resampled to a cubemap, the
    reference's SKYBOX mode. Camera for 1920x1080."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    ground = sc.add_mesh(quad_mesh((-40, 0, 40), (80, 0, 0), (0, 0, -80)))
    sc.add_object(ground, sc.add_material((0.5, 0.5, 0.5), rough=0.9, metal=0.0))
    protos = []
    for k in range(prototypes):
        m = icosphere_mesh(subdivisions, seed=seed + 17 * k, displacement=0.1)
        m.with_frames()
        protos.append(sc.add_mesh(m))
    box = sc.add_mesh(box_mesh())
    side = int(math.ceil(math.sqrt(instances)))
    cells = rng.permutation(side * side)[:instances]
    for k in range(instances):
        cx, cz = cells[k] % side, cells[k] // side
        x = (cx + 0.5) / side * 48.0 - 24.0 + rng.uniform(-0.6, 0.6)
        z = (cz + 0.5) / side * 48.0 - 24.0 + rng.uniform(-0.6, 0.6)
        s = rng.uniform(0.5, 1.2)
        metal = float(rng.random() < 0.3)
        mat = sc.add_material(rng.uniform(0.2, 0.9, 3), rough=float(rng.uniform(0.05, 1.0)), metal=metal)
        if k % 2 == 0:
            mesh = protos[int(rng.integers(0, prototypes))]
            model = translation((x, s * 1.1, z)) @ rotation_y(rng.uniform(0, 2 * math.pi)) @ scaling(s)
        else:
            mesh = box
            model = translation((x, s, z)) @ rotation_y(rng.uniform(0, 2 * math.pi)) @ scaling((1.6 * s, 2 * s, 1.6 * s))
        sc.add_object(mesh, mat, model)
    for k in range(4):
        ang = k * math.pi / 2 + 0.4
        c = (14 * math.cos(ang), 9.0, 14 * math.sin(ang))
        q = sc.add_mesh(quad_mesh((c[0] - 1.5, c[1], c[2] + 1.5), (3, 0, 0), (0, 0, -3), normal=(0, -1, 0)))
        sc.add_object(q, sc.add_material((25.0, 22.0, 18.0), emissive=True))
    env = sky_equirect()
    faces = equirect_to_cubemap(env, env_face)
    sc.background = {"mode": 2, "color": (0, 0, 0), "tex": tuple(sc.add_texture(f) for f in faces)}
    sc.environment = {"tex": sc.add_texture(env), "intensity": 1.0}
    sc.camera = {"eye": (0.0, 9.0, 34.0), "center": (0.0, 1.0, 0.0), "up": (0.0, 1.0, 0.0), "fov": 0.9,
                 "ratio": 1920.0 / 1080.0}
    return sc


def constant_environment(scene: Scene, radiance=(1.0, 1.0, 1.0), size: int = 16) -> Scene:
    """Give `scene` the same constant radiance both as a SKYBOX cubemap (the reference's
    background) and as an equirectangular environment (the extended estimator's), so the
    two estimators integrate exactly the same lighting."""
    img = np.broadcast_to(np.asarray(radiance, np.float32), (size, size, 3)).copy()
    faces = tuple(scene.add_texture(img) for _ in range(6))
    scene.background = {"mode": 2, "color": (0, 0, 0), "tex": faces}
    env = np.broadcast_to(np.asarray(radiance, np.float32), (size, 2 * size, 3)).copy()
    scene.environment = {"tex": scene.add_texture(env), "intensity": 1.0}
    return scene


def open_cornell_scene(seed: int = 20261204) -> Scene:
    """The Cornell room without its ceiling and front, lit by its emitter and by whatever
    environment is attached (see constant_environment)."""
    sc = cornell_scene(seed)
    keep = [o for k, o in enumerate(sc.objects) if k != 1]  # drop the ceiling (object 1)
    sc.objects = keep
    return sc


def batch_workload(seed: int = 20261207, jobs: int = 64, tri_range=(10_000, 500_000), res_range=(128, 1024),
                   spp_range=(4, 256), depth_range=(3, 10)):
    """The batched-rendering workload: `jobs` seeded scenes, each with a log-uniform triangle
    count in `tri_range` (instances of displaced icospheres and boxes on a ground plane,
    emissive quads, cubemap sky), a log-uniform square resolution in `res_range`, a
    log-uniform sample count in `spp_range` rounded to a power of two and a uniform depth in
    `depth_range`. Returns a list of dicts (scene, width, height, samples, depth, seed)."""
    rng = np.random.default_rng(seed)
    protos = {}
    out = []
    for k in range(jobs):
        tris = int(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        res = int(np.exp(rng.uniform(np.log(res_range[0]), np.log(res_range[1]))))
        spp = int(2 ** round(np.log2(np.exp(rng.uniform(np.log(spp_range[0]), np.log(spp_range[1]))))))
        depth = int(rng.integers(depth_range[0], depth_range[1] + 1))
        sub = 4 if tris < 60_000 else 5
        per = 20 * 4 ** sub
        inst = max(2, int(round(tris / per)))
        sc = _batch_scene(rng, inst, sub, protos)
        out.append({"scene": sc, "width": res, "height": res, "samples": spp, "depth": depth,
                    "seed": int(seed * 100 + k)})
    return out


def _batch_scene(rng, instances, sub, protos):
    sc = Scene()
    key = ("ico", sub)
    if key not in protos:
        protos[key] = [icosphere_mesh(sub, seed=100 + j, displacement=0.1).with_frames() for j in range(3)]
    meshes = [sc.add_mesh(m) for m in protos[key]]
    box = sc.add_mesh(box_mesh())
    sc.add_object(sc.add_mesh(quad_mesh((-20, 0, 20), (40, 0, 0), (0, 0, -40))), sc.add_material((0.5, 0.5, 0.5)))
    side = int(math.ceil(math.sqrt(instances)))
    for k in range(instances):
        x = ((k % side) + 0.5) / side * 24 - 12
        z = ((k // side) + 0.5) / side * 24 - 12
        s = float(rng.uniform(0.4, 1.0))
        mat = sc.add_material(rng.uniform(0.2, 0.9, 3), rough=float(rng.uniform(0.05, 1.0)), metal=float(rng.random() < 0.3))
        if k % 4 == 3:
            sc.add_object(box, mat, translation((x, s, z)) @ rotation_y(rng.uniform(0, 6.28)) @ scaling(1.5 * s))
        else:
            sc.add_object(meshes[k % 3], mat, translation((x, s * 1.1, z)) @ scaling(s))
    sc.add_object(sc.add_mesh(quad_mesh((-2, 7, 2), (4, 0, 0), (0, 0, -4), normal=(0, -1, 0))),
                  sc.add_material((20.0, 18.0, 16.0), emissive=True))
    faces = [constant_texture([0.4 + 0.05 * f, 0.5, 0.7], 4) for f in range(6)]
    sc.background = {"mode": 2, "color": (0, 0, 0), "tex": tuple(sc.add_texture(f) for f in faces)}
    sc.camera = {"eye": (0.0, 8.0, 20.0), "center": (0.0, 1.0, 0.0), "up": (0.0, 1.0, 0.0), "fov": 1.0, "ratio": 1.0}
    return sc


def denoiser_scene(seed: int = 20261208, instances: int = 60) -> Scene:
    """The denoiser's scenes: the large workload's kind of scene at a smaller size --
    `instances` seeded displaced icospheres (1,280 triangles at 3 subdivisions) and boxes
    with GGX materials on a ground plane, four emissive quads, the procedural HDR sky as a
    cubemap background and as the extended estimator's environment map."""
    return instanced_scene(seed, instances=instances, subdivisions=3, prototypes=3, env_face=64)


def random_cameras(seed: int, count: int, ratio: float = 1.0):
    """Seeded viewpoints over an instanced scene: eyes on rings 8-30 units from the centre
    at heights 1.5-10, looking at points near the ground within 10 units of the centre,
    vertical field of view 0.6-1.2 rad."""
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(count):
        a = rng.uniform(0, 2 * math.pi)
        r = rng.uniform(8.0, 30.0)
        eye = (r * math.cos(a), rng.uniform(1.5, 10.0), r * math.sin(a))
        b = rng.uniform(0, 2 * math.pi)
        q = rng.uniform(0.0, 10.0)
        center = (q * math.cos(b), rng.uniform(0.5, 1.5), q * math.sin(b))
        cams.append({"eye": eye, "center": center, "up": (0.0, 1.0, 0.0), "fov": float(rng.uniform(0.6, 1.2)),
                     "ratio": ratio})
    return cams


def atmosphere(scene: Scene, sun=(0.3, 0.6, -0.5), table=None) -> Scene:
    """Give `scene` the reference's ATMOSPHERE background (Scene::Background::ATMOSPHERE with
    a Sky object): MaterialSky's sky for the given sun direction, optionally with a
    caller-supplied scattering table (h, w, 4)."""
    scene.background = {"mode": 3, "color": tuple(float(x) for x in sun), "tex": (0,) * 6, "sky_table": table}
    return scene
