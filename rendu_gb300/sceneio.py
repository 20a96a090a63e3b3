"""Scene files: the reference's ``.scene`` text format and its resources, loaded into an
in-memory ``scenes.Scene`` the device path tracer takes, as ``Scene::init(Storage::CPU |
Storage::FORCE_FRAME)`` does for the reference's offline renderer (src/engine/scene/
Scene.cpp:29-118 of kosua20/Rendu, called from src/apps/pathtracer/main.cpp:88-91).

  * ``decode`` -- Codable::decode (Codable.cpp:185-268): ``#`` comments, ``key: values`` lines
    split at their first colon, further colons nesting a child token, values separated by
    spaces or commas, ``*`` opening a root block and ``-`` lines forming an array under the
    element before them.
  * ``Resources`` -- the resources index (ResourcesManager.cpp:76-118): every file below the
    given directories by file name, the first one found kept; images looked up as
    name.png / .jpg / .jpeg / .bmp / .tga / .exr (ResourcesManager.cpp:120-141).
  * textures (ResourcesManager.cpp:380-538): constant-colour names ("0.8,0.8,0.8") as 8 x 8
    images, 2-D images, mip chains (name_0, name_1, ...), cube maps name_px, _nx, _ny, _py,
    _pz, _nz loaded with rows flipped, all with 4 channels (the scene layouts srgb, rgb and
    rgb32 are 4-channel formats; 8-bit values divided by 255, no colour-space conversion);
  * meshes (ResourcesManager.cpp:306-340): ``meshio.load_obj``;
  * blocks: ``object`` (Object.cpp:10-44), ``material`` (Material.cpp:41-86), ``point`` /
    ``directional`` / ``spot`` (PointLight.cpp:89-99, DirectionalLight.cpp:46-59,
    SpotLight.cpp:83-107, Light.cpp:19-32), ``camera`` (Camera.cpp:66-107), ``background``
    (Scene.cpp:137-211: color, image, cube, sun), ``scene`` (a transformation applied to
    every object, Scene.cpp:213-216); ``probe`` blocks only feed the rasterised renderer and
    are read and ignored;
  * Scene::init's finish: materials matched to objects by name, objects ordered by material
    type (Scene.cpp:84-86; a stable order where the reference's std::sort leaves ties
    unspecified).

An object flagged ``skipuvs`` samples its material at uv (0.5, 0.5) and skips the normal map
(PathTracer.cpp:108, 217); it is given its own copy of the mesh without texture
coordinates, which is how the device path tracer marks an object without UVs.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import imageio, meshio
from .scenes import Mesh, Scene

_F32 = np.float32

MATERIAL_TYPES = {"None": 0, "Regular": 1, "Parallax": 2, "Clearcoat": 3, "Anisotropic": 4, "Sheen": 5,
                  "Iridescent": 6, "Subsurface": 7, "Emissive": 8, "Transparent": 9, "TransparentIrid": 10}
TEXTURE_LAYOUTS = ("srgb", "rgb", "rgb32", "srgbcube", "rgbcube", "rgb32cube")
IMAGE_EXTENSIONS = (".png", ".jpg", ".jpeg", ".bmp", ".tga", ".exr")
CUBE_SUFFIXES = ("_px", "_nx", "_ny", "_py", "_pz", "_nz")


class SceneError(ValueError):
    """A scene the reference would fail to load (missing resource, bad value)."""


@dataclass
class KeyValues:
    """One token of the scene format: key, values, child tokens (Codable.hpp's KeyValues)."""

    key: str
    values: list = field(default_factory=list)
    elements: list = field(default_factory=list)


def decode(text: str) -> list:
    """Codable::decode (Codable.cpp:185-268): the root tokens of a scene text."""
    raw = []
    for line in text.split("\n"):
        h = line.find("#")
        if h >= 0:
            line = line[:h]
        line = line.strip(" \t\r")
        if not line:
            continue
        c = line.find(":")
        if c < 0:
            continue
        tok = KeyValues(line[:c].strip(" \t"))
        raw.append(tok)
        prev = c + 1
        nxt = line.find(":", prev)
        while nxt >= 0:
            sub = line[prev:nxt].strip(" \t")
            if sub:
                child = KeyValues(sub)
                tok.elements.append(child)
                tok = child
            prev = nxt + 1
            nxt = line.find(":", prev)
        tok.values = [v for v in line[prev:].replace(",", " ").strip(" \t").split(" ") if v]
    roots = []
    i = 0
    while i < len(raw):
        tok = raw[i]
        if tok.key.startswith("*"):
            roots.append(KeyValues(tok.key[1:].strip("\t "), tok.values))
            i += 1
            continue
        if not roots:
            i += 1
            continue
        roots[-1].elements.append(tok)
        i += 1
        while i < len(raw) and raw[i].key.startswith("-"):
            item = raw[i]
            item.key = item.key[1:].strip("\t ")
            tok.elements.append(item)
            i += 1
    return roots


# --------------------------------------------------------------------------------------
# values (Codable.cpp:9-141)
# --------------------------------------------------------------------------------------


def _stof(s: str) -> np.float32:
    return meshio._stof(s.encode())


def decode_bool(p: KeyValues, pos: int = 0) -> bool:
    return len(p.values) > pos and p.values[pos] in ("true", "True", "yes", "Yes", "1", "y", "Y")


def decode_vec(p: KeyValues, n: int, pos: int = 0) -> np.ndarray:
    if len(p.values) < pos + n:
        raise SceneError(f"'{p.key}' needs {n} values")
    return np.array([_stof(v) for v in p.values[pos:pos + n]], _F32)


_LIBM = None


def _cosf_sinf(x: np.float32):
    """std::cos / std::sin of a float: the C library's single-precision functions."""
    global _LIBM
    if _LIBM is None:
        import ctypes
        import ctypes.util

        _LIBM = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        for f in (_LIBM.cosf, _LIBM.sinf):
            f.argtypes = [ctypes.c_float]
            f.restype = ctypes.c_float
    return _F32(_LIBM.cosf(float(x))), _F32(_LIBM.sinf(float(x)))


def _rotation(axis: np.ndarray, angle: np.float32) -> np.ndarray:
    """glm::rotate(identity, angle, axis) as a row-major 4x4 (single precision)."""
    a = axis * (_F32(1.0) / np.sqrt(meshio._dot(axis, axis)))
    c, s = _cosf_sinf(angle)
    t = (_F32(1.0) - c) * a
    r = np.eye(4, dtype=_F32)
    # column j of glm's matrix is row j here transposed: r[row, col]
    r[0, 0] = c + t[0] * a[0]
    r[1, 0] = t[0] * a[1] + s * a[2]
    r[2, 0] = t[0] * a[2] - s * a[1]
    r[0, 1] = t[1] * a[0] - s * a[2]
    r[1, 1] = c + t[1] * a[1]
    r[2, 1] = t[1] * a[2] + s * a[0]
    r[0, 2] = t[2] * a[0] + s * a[1]
    r[1, 2] = t[2] * a[1] - s * a[0]
    r[2, 2] = c + t[2] * a[2]
    return r


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """4x4 product with glm's single-precision accumulation order (row-major arrays):
    each element ((a0 b0 + a1 b1) + a2 b2) + a3 b3."""
    a = np.asarray(a, _F32)
    b = np.asarray(b, _F32)
    out = np.zeros((4, 4), _F32)
    for i in range(4):
        for j in range(4):
            out[i, j] = ((a[i, 0] * b[0, j] + a[i, 1] * b[1, j]) + a[i, 2] * b[2, j]) + a[i, 3] * b[3, j]
    return out


def decode_transformation(params: list) -> np.ndarray:
    """Codable::decodeTransformation (Codable.cpp:79-104): translation * rotation * scaling,
    row-major float32 4x4."""
    axis = np.zeros(3, _F32)
    trans = np.zeros(3, _F32)
    angle = _F32(0.0)
    scale = _F32(1.0)
    for p in params:
        if p.key == "orientation":
            v = decode_vec(p, 3)
            with np.errstate(divide="ignore", invalid="ignore"):
                axis = v * (_F32(1.0) / np.sqrt(meshio._dot(v, v)))
            if len(p.values) >= 4:
                angle = _stof(p.values[3])
        elif p.key == "translation":
            trans = decode_vec(p, 3)
        elif p.key == "scaling" and p.values:
            scale = _stof(p.values[0])
    t = np.eye(4, dtype=_F32)
    t[:3, 3] = trans
    r = _rotation(axis, angle) if angle != 0 else np.eye(4, dtype=_F32)
    s = np.diag(np.array([scale, scale, scale, 1.0], _F32))
    return mat_mul(mat_mul(t, r), s)


# --------------------------------------------------------------------------------------
# resources
# --------------------------------------------------------------------------------------


class Resources:
    """File lookup by name below a list of directories (ResourcesManager.cpp:76-141)."""

    def __init__(self, roots=()):
        self.files: dict[str, str] = {}
        for r in roots:
            self.add(r)

    def add(self, root: str):
        for dirpath, dirnames, filenames in os.walk(root):
            dirnames[:] = sorted(d for d in dirnames if not d.startswith("."))
            for f in sorted(filenames):
                if f and not f.startswith(".") and f not in self.files:
                    self.files[f] = os.path.join(dirpath, f)

    def path(self, filename: str) -> str | None:
        return self.files.get(filename)

    def image_path(self, name: str) -> str | None:
        for ext in IMAGE_EXTENSIONS:
            p = self.files.get(name + ext)
            if p:
                return p
        return None

    def text(self, filename: str) -> str | None:
        p = self.files.get(filename) or self.files.get(filename + ".txt")
        if p is None:
            return None
        with open(p, "rb") as f:
            return f.read().decode("utf-8", "replace")


# --------------------------------------------------------------------------------------
# scene loading
# --------------------------------------------------------------------------------------


@dataclass
class LoadedScene:
    """The device scene plus what the reference's Scene keeps beside it."""

    scene: Scene
    name: str
    camera: dict  # eye, center, up, fov (ratio set by the caller)
    planes: tuple
    object_names: list  # mesh name of each object, in the final (sorted) order
    material_names: list


class _Loader:
    def __init__(self, res: Resources):
        self.res = res
        self.sc = Scene()
        self.textures: dict = {}  # (name, layout) -> texture ids (6 for cube maps)
        self.meshes: dict = {}  # name -> (Mesh, had_uv)
        self.mesh_ids: dict = {}  # (name, use_uv) -> scene mesh id

    # textures ------------------------------------------------------------------------
    def _images(self, name: str, cube: bool):
        if name and all(ch in "0123456789,.-" for ch in name):
            col = np.array([0.0, 0.0, 0.0, 1.0], _F32)
            toks = [t for t in name.split(",") if t]
            for i, t in enumerate(toks[:4]):
                col[i] = _stof(t)
            return [np.broadcast_to(col, (8, 8, 4)).copy()], False
        p2d = self.res.image_path(name)
        if p2d:
            return [p2d], False
        faces = [self.res.image_path(name + s) for s in CUBE_SUFFIXES]
        if all(faces):
            return faces, True
        p2d = self.res.image_path(name + "_0")
        if p2d:
            return [p2d], False
        faces = [self.res.image_path(name + "_0" + s) for s in CUBE_SUFFIXES]
        if all(faces):
            return faces, True
        if self.res.image_path(name + "_s0") or self.res.image_path(name + "_0_s0") \
                or self.res.image_path(name + "_z0") or self.res.image_path(name + "_0_z0"):
            raise SceneError(f"texture '{name}' is a texture array or 3-D texture, which the path tracer does not use")
        raise SceneError(f"unable to find texture named '{name}'")

    def texture(self, name: str, layout: str):
        """Texture ids of a scene texture: 1 for 2-D, 6 for a cube map (faces in file order
        px, nx, ny, py, pz, nz as Texture::sampleCubemap indexes them)."""
        key = (name, layout)
        if key in self.textures:
            return self.textures[key]
        imgs, cube = self._images(name, layout.endswith("cube"))
        ids = []
        for im in imgs:
            if isinstance(im, str):
                im = imageio.load_image(im, 4, flip=cube)
            ids.append(self.sc.add_texture(im))
        self.textures[key] = ids
        return ids

    def default_texture(self, rgba):
        key = (",".join(repr(float(x)) for x in rgba), "default")
        if key not in self.textures:
            self.textures[key] = [self.sc.add_texture(np.broadcast_to(np.asarray(rgba, _F32), (8, 8, 4)).copy())]
        return self.textures[key]

    # meshes --------------------------------------------------------------------------
    def mesh(self, name: str, use_uv: bool) -> int:
        if name not in self.meshes:
            p = self.res.path(name + ".obj")
            if p is None:
                raise SceneError(f"unable to load mesh named '{name}'")
            with open(p, "rb") as f:
                self.meshes[name] = meshio.load_obj(f.read())
        key = (name, use_uv)
        if key not in self.mesh_ids:
            m, _ = self.meshes[name]
            if not use_uv:
                m = Mesh(positions=m.positions, indices=m.indices, normals=m.normals, tangents=m.tangents,
                         bitangents=m.bitangents, texcoords=None)
            self.mesh_ids[key] = self.sc.add_mesh(m)
        return self.mesh_ids[key]


def _layout_texture(p: KeyValues):
    """Codable::decodeTexture: (name, layout) of a texture token, or None."""
    if p.key not in TEXTURE_LAYOUTS or not p.values:
        return None
    return ",".join(p.values), p.key


def load_scene(scene: str, resources=(), default_resources: bool = True) -> LoadedScene:
    """Scene(name).init(Storage::CPU | Storage::FORCE_FRAME) for the offline renderer.

    ``scene`` is a path to a .scene file or a scene name looked up in the resources (".scene"
    appended when missing). ``resources`` are directories searched for the files the scene
    names; with ``default_resources`` the directory of a scene given by path and its parent
    are searched too."""
    roots = list(resources)
    path = scene if os.path.isfile(scene) else None
    if path and default_resources:
        d = os.path.dirname(os.path.abspath(path))
        roots = roots + [d, os.path.dirname(d)]
    res = Resources(roots)
    name = os.path.basename(scene)
    if not name.endswith(".scene"):
        name += ".scene"
    if path is None:
        path = res.path(name)
        if path is None:
            raise SceneError(f"unable to find scene '{name}'")
    with open(path, "rb") as f:
        text = f.read().decode("utf-8", "replace")
    ld = _Loader(res)
    sc = ld.sc
    objects, materials = [], []
    camera = {"eye": (0.0, 0.0, 1.0), "center": (0.0, 0.0, 0.0), "up": (0.0, 1.0, 0.0), "fov": 1.3}
    planes = (0.01, 100.0)
    scene_model = np.eye(4, dtype=_F32)
    background = None
    for blk in decode(text):
        k = blk.key
        if k == "object":
            objects.append(_object(blk))
        elif k == "material":
            materials.append(_material(blk, ld))
        elif k in ("point", "directional", "spot"):
            sc.lights.append(_light(blk))
        elif k == "camera":
            camera, planes = _camera(blk)
        elif k == "background":
            background = _background(blk, ld)
        elif k == "scene":
            scene_model = decode_transformation(blk.elements)
        elif k == "probe":
            pass
        else:
            raise SceneError(f"unknown block '{k}'")
    sc.background = background if background is not None else {"mode": 0, "color": (0.0, 0.0, 0.0),
                                                                "tex": (0,) * 6}
    # materials by name, objects in material-type order (stable)
    mat_ids, mat_types = {}, []
    for m in materials:
        if m["name"] in mat_ids:
            continue  # the first material of a name is the one objects find
        mat_ids[m["name"]] = len(sc.materials)
        sc.materials.append({"type": m["type"], "masked": m["masked"], "tex": m["tex"]})
        mat_types.append(m["type"])
    resolved = []
    for o in objects:
        if o["material"] not in mat_ids:
            raise SceneError(f"missing material '{o['material']}'")
        resolved.append((mat_types[mat_ids[o["material"]]], o))
    resolved.sort(key=lambda x: x[0])
    names = []
    for _, o in resolved:
        mesh_id = ld.mesh(o["mesh"], not o["skipuvs"])
        sc.add_object(mesh_id, mat_ids[o["material"]], mat_mul(scene_model, o["model"]))
        names.append(o["mesh"])
    sc.camera = dict(camera)
    return LoadedScene(sc, name[:-6], dict(camera), planes, names, list(mat_ids))


def _object(blk: KeyValues) -> dict:
    """Object::decode (Object.cpp:10-44)."""
    o = {"model": decode_transformation(blk.elements), "mesh": None, "material": "", "skipuvs": False}
    for p in blk.elements:
        if p.key == "mesh" and p.values:
            o["mesh"] = p.values[0]
        elif p.key == "material" and p.values:
            o["material"] = p.values[0]
        elif p.key == "skipuvs":
            o["skipuvs"] = decode_bool(p)
    if o["mesh"] is None:
        raise SceneError("object without a mesh")
    return o


def _material(blk: KeyValues, ld: _Loader) -> dict:
    """Material::decode (Material.cpp:41-86). The path tracer reads texture 0 (colour and
    alpha), 1 (normal map) and 2 (roughness, metalness, occlusion); missing ones are given a
    neutral constant texture."""
    m = {"type": 0, "masked": False, "name": "", "tex": []}
    for p in blk.elements:
        if p.key == "type" and p.values:
            if p.values[0] not in MATERIAL_TYPES:
                raise SceneError(f"unknown material type '{p.values[0]}'")
            m["type"] = MATERIAL_TYPES[p.values[0]]
        elif p.key == "textures":
            for t in p.elements:
                info = _layout_texture(t)
                if info is None:
                    raise SceneError(f"texture '{t.key}' has no known layout")
                m["tex"].append(ld.texture(*info)[0])
        elif p.key == "masked":
            m["masked"] = decode_bool(p)
        elif p.key == "name" and p.values:
            m["name"] = p.values[0]
    if not m["name"]:
        raise SceneError("material has no name")
    defaults = [(1.0, 1.0, 1.0, 1.0), (0.5, 0.5, 1.0, 1.0), (1.0, 0.0, 1.0, 1.0)]
    while len(m["tex"]) < 3:
        m["tex"].append(ld.default_texture(defaults[len(m["tex"])])[0])
    m["tex"] = tuple(m["tex"][:3])
    return m


def _light(blk: KeyValues) -> dict:
    """Light::decode and the per-type decoders; spot cone angles are halved (SpotLight.cpp:100)."""
    kind = {"point": 0, "directional": 1, "spot": 2}[blk.key]
    l = {"type": kind, "color": (1.0, 1.0, 1.0), "shadows": False, "position": (0.0, 0.0, 0.0), "radius": 1.0,
         "direction": (0.0, 0.0, 1.0) if kind == 1 else (1.0, 0.0, 0.0),
         "inner": math.pi / 4, "outer": math.pi / 2}
    for p in blk.elements:
        if p.key == "intensity":
            l["color"] = tuple(float(x) for x in decode_vec(p, 3))
        elif p.key == "shadows":
            l["shadows"] = decode_bool(p)
        elif p.key == "position" and kind != 1:
            l["position"] = tuple(float(x) for x in decode_vec(p, 3))
        elif p.key == "radius" and p.values and kind != 1:
            l["radius"] = float(_stof(p.values[0]))
        elif p.key == "direction" and kind != 0:
            d = decode_vec(p, 3)
            if not d.any():
                raise SceneError("invalid light direction")
            d = d * (_F32(1.0) / np.sqrt(meshio._dot(d, d)))
            l["direction"] = tuple(float(x) for x in d)
        elif p.key == "cone" and len(p.values) >= 2 and kind == 2:
            l["inner"] = float(_F32(0.5) * _stof(p.values[0]))
            l["outer"] = float(_F32(0.5) * _stof(p.values[1]))
    return l


def _camera(blk: KeyValues):
    """Camera::decode (Camera.cpp:66-107) with its validation."""
    pos = np.array([0, 0, 1], _F32)
    center = np.zeros(3, _F32)
    up = np.array([0, 1, 0], _F32)
    planes = np.array([0.01, 100.0], _F32)
    fov = _F32(1.3)
    for p in blk.elements:
        if p.key == "position":
            pos = decode_vec(p, 3)
        elif p.key == "center":
            center = decode_vec(p, 3)
        elif p.key == "up":
            up = decode_vec(p, 3)
        elif p.key == "fov" and p.values:
            fov = _stof(p.values[0])
        elif p.key == "planes":
            planes = decode_vec(p, 2)
    if fov > math.pi:
        raise SceneError("camera field of view is greater than 180 degrees")
    if planes[0] >= planes[1] or planes[0] <= 0 or planes[1] <= 0:
        raise SceneError("camera planes are invalid")
    d = pos - center
    with np.errstate(divide="ignore", invalid="ignore"):
        cosang = abs(float(np.dot(up / np.linalg.norm(up), d / np.linalg.norm(d))))
    if cosang > 0.99 or (pos == center).all() or not up.any():
        raise SceneError("camera look-at configuration is invalid")
    cam = {"eye": tuple(float(x) for x in pos), "center": tuple(float(x) for x in center),
           "up": tuple(float(x) for x in up), "fov": float(fov)}
    return cam, (float(planes[0]), float(planes[1]))


def _background(blk: KeyValues, ld: _Loader) -> dict:
    """Scene::loadBackground (Scene.cpp:137-211): the last recognised entry decides."""
    bg = {"mode": 0, "color": (0.0, 0.0, 0.0), "tex": (0,) * 6}
    for p in blk.elements:
        if p.key == "color":
            bg = {"mode": 0, "color": tuple(float(x) for x in decode_vec(p, 3)), "tex": (0,) * 6}
        elif p.key == "image" and p.elements:
            info = _layout_texture(p.elements[0])
            if info is None:
                raise SceneError("background image without a texture layout")
            ids = ld.texture(*info)
            bg = {"mode": 1, "color": (0.0, 0.0, 0.0), "tex": (ids[0],) + (0,) * 5}
        elif p.key == "cube" and p.elements:
            info = _layout_texture(p.elements[0])
            if info is None:
                raise SceneError("background cube map without a texture layout")
            ids = ld.texture(*info)
            if len(ids) != 6:
                raise SceneError(f"background '{info[0]}' is not a cube map")
            bg = {"mode": 2, "color": (0.0, 0.0, 0.0), "tex": tuple(ids)}
        elif p.key == "sun":
            sun = np.array([0.0, 1.0, 0.0], _F32)
            for q in blk.elements:  # Sky::decode (Sky.cpp:7-21)
                if q.key == "sun":
                    v = decode_vec(q, 3)
                    if not v.any():
                        raise SceneError("invalid null sun direction")
                    sun = v * (_F32(1.0) / np.sqrt(meshio._dot(v, v)))
            bg = {"mode": 3, "color": tuple(float(x) for x in sun), "tex": (0,) * 6}
    return bg
