"""Triangle meshes of a scene file, loaded as the reference's offline renderer loads them
(Resources::getMesh with Storage::FORCE_FRAME, ResourcesManager.cpp:306-340 of
kosua20/Rendu):

  1. ``parse_obj`` -- Mesh(std::istream &, Mesh::Load::Indexed) (Mesh.cpp:99-271): v / vt / vn
     / f records, v texture coordinate stored as 1 - v, the first three vertices of a face,
     one vertex per distinct face token in first-seen order, the token's sub-indices read
     with the reference's own substring rules;
  2. ``compute_normals`` when the file has none -- Mesh::computeNormals (Mesh.cpp:327-354):
     per face cross(normalize(v1 - v0), normalize(v2 - v0)) added to its three vertices in
     face order, then normalised;
  3. ``tangent_frames`` -- Mesh::computeTangentsAndBitangents(force) (Mesh.cpp:356-505):
     constant (0.5, 0.5) texture coordinates when the file has none, per-corner tangents and
     handedness from the MikkTSpace algorithm (M. Mikkelsen, "Simulation of wrinkled
     surfaces revisited", 2008; the reference links the public-domain mikktspace.c of
     src/libs/mikktspace with the default 180 degree angular threshold), then the
     reference's vertex split: a vertex whose consecutive face corners received different
     tangents is duplicated, and each tangent / bitangent pair is finished as the reference
     does (a fallback axis for tangents parallel to the normal, bitangent = -sign x
     cross(n, t), both normalised).

All arithmetic is single precision in the reference's operation order so that meshes equal
the reference's bit for bit. The tangent-space step follows the published algorithm
stage by stage (welding of identical corners, degenerate triangles, per-triangle
derivatives, edge adjacency, orientation-preserving vertex groups, angle-weighted
averaging); where it differs from mikktspace.c it is in the welding representative of
non-manifold edges shared by more than two triangles, which only changes which neighbour
such an edge is paired with.
"""
from __future__ import annotations

import re
from dataclasses import dataclass

import numpy as np

from .scenes import Mesh

_F32 = np.float32
_FLT_MIN = np.float32(np.finfo(np.float32).tiny)
_NUM = re.compile(rb"\s*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))", re.IGNORECASE)
_INT = re.compile(rb"\s*([+-]?\d+)")


class MeshFormatError(ValueError):
    """An OBJ file the reference's loader would not read (or would read out of bounds)."""


def _stof(tok: bytes) -> np.float32:
    """std::stof: the leading decimal number of the token, rounded to float."""
    try:
        return _F32(float(tok))
    except ValueError:
        m = _NUM.match(tok)
        if not m:
            raise MeshFormatError(f"not a number: {tok!r}") from None
        return _F32(float(m.group(1)))


def _stoi(tok: bytes) -> int:
    """std::stoi: the leading integer of the token."""
    m = _INT.match(tok)
    if not m:
        raise MeshFormatError(f"not an index: {tok!r}")
    return int(m.group(1))


@dataclass
class ObjData:
    """The arrays Mesh's Indexed loader produces (texcoords / normals None when absent)."""

    positions: np.ndarray
    texcoords: np.ndarray | None
    normals: np.ndarray | None
    indices: np.ndarray


def parse_obj(data: bytes | str) -> ObjData:
    """Mesh(std::istream &, Mesh::Load::Indexed): see the module docstring."""
    if isinstance(data, str):
        data = data.encode()
    pos_t, nor_t, uv_t, faces = [], [], [], []
    for line in data.split(b"\n"):
        if not line or line[:1] == b"#" or len(line) < 2:
            continue
        toks = line.strip(b"\r").split()
        if not toks:
            continue
        kind = toks[0]
        if kind == b"v":
            if len(toks) >= 4:
                pos_t.append((_stof(toks[1]), _stof(toks[2]), _stof(toks[3])))
        elif kind == b"vn":
            if len(toks) >= 4:
                nor_t.append((_stof(toks[1]), _stof(toks[2]), _stof(toks[3])))
        elif kind == b"vt":
            if len(toks) >= 3:
                uv_t.append((_stof(toks[1]), _F32(1.0) - _stof(toks[2])))
        elif kind == b"f":
            if len(toks) >= 4:
                faces += toks[1:4]
    if not pos_t:
        return ObjData(np.zeros((0, 3), _F32), None, None, np.zeros(0, np.uint32))
    has_uv, has_n = bool(uv_t), bool(nor_t)
    used: dict[bytes, int] = {}
    indices = np.empty(len(faces), np.uint32)
    pi, ti, ni = [], [], []
    for k, tok in enumerate(faces):
        got = used.get(tok)
        if got is not None:
            indices[k] = got
            continue
        first, last = tok.find(b"/"), tok.rfind(b"/")
        # the reference's substrings: [0, first), [first + 1, first + 1 + last), [last + 1, end)
        # with npos (no slash) wrapping the last two to the whole token
        p = _stoi(tok if first < 0 else tok[:first]) - 1
        pi.append(p)
        if has_uv:
            ti.append(_stoi(tok if first < 0 else tok[first + 1:first + 1 + last]) - 1)
        if has_n:
            ni.append(_stoi(tok if last < 0 else tok[last + 1:]) - 1)
        used[tok] = len(pi) - 1
        indices[k] = len(pi) - 1

    def gather(table, idx, what):
        idx = np.asarray(idx, np.int64)
        arr = np.asarray(table, _F32)
        if len(idx) and (idx.min() < 0 or idx.max() >= len(arr)):
            raise MeshFormatError(f"face {what} index out of range")
        return arr[idx]

    return ObjData(gather(pos_t, pi, "position"), gather(uv_t, ti, "texture coordinate") if has_uv else None,
                   gather(nor_t, ni, "normal") if has_n else None, indices)


# --------------------------------------------------------------------------------------
# single-precision vector helpers in the reference's operation order
# --------------------------------------------------------------------------------------


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - b[..., 1] * a[..., 2],
                     a[..., 2] * b[..., 0] - b[..., 2] * a[..., 0],
                     a[..., 0] * b[..., 1] - b[..., 0] * a[..., 1]], -1)


def _glm_normalize(v):
    """glm::normalize: v * (1 / sqrt(dot(v, v)))."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return v * (_F32(1.0) / np.sqrt(_dot(v, v)))[..., None]


def _mk_normalize(v):
    """mikktspace Normalize: (1 / Length(v)) * v, applied where any component exceeds FLT_MIN."""
    nz = (np.abs(v) > _FLT_MIN).any(-1)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = (_F32(1.0) / np.sqrt(_dot(v, v)))[..., None] * v
    return np.where(nz[..., None], out, v)


def compute_normals(positions: np.ndarray, indices: np.ndarray) -> np.ndarray:
    """Mesh::computeNormals (Mesh.cpp:327-354)."""
    p = np.asarray(positions, _F32)
    f = np.asarray(indices, np.int64).reshape(-1, 3)
    d01 = _glm_normalize(p[f[:, 1]] - p[f[:, 0]])
    d02 = _glm_normalize(p[f[:, 2]] - p[f[:, 0]])
    fn = _cross(d01, d02)
    n = np.zeros_like(p)
    np.add.at(n, f.reshape(-1), np.repeat(fn, 3, axis=0))  # face order per vertex
    return _glm_normalize(n).astype(_F32)


# --------------------------------------------------------------------------------------
# MikkTSpace (default settings) -- per-corner tangent and handedness
# --------------------------------------------------------------------------------------


def mikktspace(positions, normals, texcoords, indices):
    """Per-corner (tangent xyz, sign) of the MikkTSpace algorithm for a triangle list, as the
    reference's callbacks feed it (Mesh.cpp:25-92): (3T, 4) float32."""
    P = np.asarray(positions, _F32)
    N = np.asarray(normals, _F32)
    U = np.asarray(texcoords, _F32)
    idx = np.asarray(indices, np.int64).reshape(-1)
    nt = len(idx) // 3
    ncorner = 3 * nt
    out = np.zeros((ncorner, 4), _F32)
    out[:, 0] = 1.0  # untouched corners keep (1, 0, 0) and the negative handedness
    out[:, 3] = -1.0
    if nt == 0:
        return out
    cp, cn, cu = P[idx], N[idx], U[idx]

    # 1. weld corners with identical position, normal and texture coordinate (-0 == +0)
    key = np.concatenate([cp, cn, cu], 1) + _F32(0.0)
    _, first, inv = np.unique(key.view(np.dtype((np.void, key.dtype.itemsize * 8))).reshape(-1),
                              return_index=True, return_inverse=True)
    weld = first[inv.reshape(-1)].reshape(nt, 3)

    # 2. degenerate triangles (two equal positions) leave the groups
    tp = cp.reshape(nt, 3, 3)
    eq = lambda a, b: (tp[:, a] == tp[:, b]).all(-1)  # noqa: E731
    degen = eq(0, 1) | eq(0, 2) | eq(1, 2)
    good = np.nonzero(~degen)[0]
    G = len(good)

    # 3. per-triangle first-order derivatives (eq. 18-19 of the paper)
    v1, v2, v3 = tp[good, 0], tp[good, 1], tp[good, 2]
    tu = cu.reshape(nt, 3, 2)[good]
    t21x = tu[:, 1, 0] - tu[:, 0, 0]
    t21y = tu[:, 1, 1] - tu[:, 0, 1]
    t31x = tu[:, 2, 0] - tu[:, 0, 0]
    t31y = tu[:, 2, 1] - tu[:, 0, 1]
    d1, d2 = v2 - v1, v3 - v1
    area = t21x * t31y - t21y * t31x
    vos = t31y[:, None] * d1 - t21y[:, None] * d2
    vot = (-t31x)[:, None] * d1 + t21x[:, None] * d2
    orient = area > 0
    nz_area = np.abs(area) > _FLT_MIN
    with np.errstate(divide="ignore", invalid="ignore"):
        len_os = np.sqrt(_dot(vos, vos))
        len_ot = np.sqrt(_dot(vot, vot))
        fs = np.where(orient, _F32(1.0), _F32(-1.0))
        tri_os = np.where((nz_area & (len_os > _FLT_MIN))[:, None], (fs / len_os)[:, None] * vos, _F32(0.0))
        tri_ot = np.where((nz_area & (len_ot > _FLT_MIN))[:, None], (fs / len_ot)[:, None] * vot, _F32(0.0))
        mag_s = np.where(nz_area, len_os / np.abs(area), _F32(0.0))
        mag_t = np.where(nz_area, len_ot / np.abs(area), _F32(0.0))
    any_grp = ~(nz_area & (mag_s > _FLT_MIN) & (mag_t > _FLT_MIN))
    orient = orient.tolist()
    any_grp = any_grp.tolist()
    gw = weld[good].tolist()  # welded corner ids of the good triangles, in order

    # 4. edge adjacency: an edge pairs with the same edge walked the other way
    edges = sorted((min(w[k], w[(k + 1) % 3]), max(w[k], w[(k + 1) % 3]), f) for f, w in enumerate(gw) for k in range(3))
    neigh = [[-1, -1, -1] for _ in range(G)]

    def get_edge(w, a, b):
        if w[0] == a or w[0] == b:
            if w[1] == a or w[1] == b:
                return w[0], w[1], 0
            return w[2], w[0], 2
        return w[1], w[2], 1

    ne = len(edges)
    for i in range(ne):
        a, b, f = edges[i]
        ia0, ia1, ea = get_edge(gw[f], a, b)
        if neigh[f][ea] != -1:
            continue
        j = i + 1
        while j < ne and edges[j][0] == a and edges[j][1] == b:
            t = edges[j][2]
            ib1, ib0, eb = get_edge(gw[t], a, b)
            if ia0 == ib0 and ia1 == ib1 and neigh[t][eb] == -1:
                neigh[f][ea] = t
                neigh[t][eb] = f
                break
            j += 1

    # 5. vertex groups: fans of triangles around a welded corner with one orientation
    assigned = [[-1, -1, -1] for _ in range(G)]
    g_rep, g_orient, g_members = [], [], []
    for f in range(G):
        for i in range(3):
            if any_grp[f] or assigned[f][i] != -1:
                continue
            g = len(g_rep)
            rep = gw[f][i]
            g_rep.append(rep)
            g_orient.append(orient[f])
            members = [f]
            g_members.append(members)
            assigned[f][i] = g
            stack = [neigh[f][(i + 2) % 3], neigh[f][i]]  # left neighbour first
            while stack:
                t = stack.pop()
                if t < 0:
                    continue
                wt = gw[t]
                k = 0 if wt[0] == rep else (1 if wt[1] == rep else 2)
                if assigned[t][k] != -1:
                    continue
                if any_grp[t] and assigned[t][0] == -1 and assigned[t][1] == -1 and assigned[t][2] == -1:
                    orient[t] = g_orient[g]  # the first group to reach it decides
                if orient[t] != g_orient[g]:
                    continue
                members.append(t)
                assigned[t][k] = g
                stack.append(neigh[t][(k + 2) % 3])
                stack.append(neigh[t][k])

    # 6. split each group into subgroups of triangles whose projected directions are not
    #    exactly opposite (the default threshold of 180 degrees: cos > -1), then one tangent
    #    space per distinct subgroup: the angle-weighted average of the projected directions,
    #    members in triangle order
    tpos = tp[good]
    tnor = cn.reshape(nt, 3, 3)[good]
    any_arr = np.asarray(any_grp)

    def projected(fs, ks):
        n = tnor[fs, ks]
        vo = _mk_normalize(tri_os[fs] - _dot(n, tri_os[fs])[:, None] * n)
        vt = _mk_normalize(tri_ot[fs] - _dot(n, tri_ot[fs])[:, None] * n)
        return vo, vt

    def pair_dot(a):
        return (a[:, None, 0] * a[None, :, 0] + a[:, None, 1] * a[None, :, 1]) + a[:, None, 2] * a[None, :, 2]

    sub_members: list[list[int]] = []  # distinct subgroups (sorted triangle lists)
    sub_rep: list[int] = []
    sub_orient: list[bool] = []
    corner_sub: dict[tuple[int, int], int] = {}  # (good triangle, corner) -> subgroup
    for g in range(len(g_rep)):
        rep = g_rep[g]
        mem = sorted(g_members[g])
        ks = [0 if gw[f][0] == rep else (1 if gw[f][1] == rep else 2) for f in mem]
        if len(mem) > 1:
            vo, vt = projected(np.asarray(mem), np.asarray(ks))
            a = any_arr[mem]
            sim = (a[:, None] | a[None, :] | np.eye(len(mem), dtype=bool)
                   | ((pair_dot(vo) > _F32(-1.0)) & (pair_dot(vt) > _F32(-1.0))))
        known: dict[tuple, int] = {}
        for j, (f, k) in enumerate(zip(mem, ks)):
            key = tuple(mem) if len(mem) == 1 or sim[j].all() else tuple(np.asarray(mem)[sim[j]].tolist())
            sid = known.get(key)
            if sid is None:
                sid = known[key] = len(sub_members)
                sub_members.append(list(key))
                sub_rep.append(rep)
                sub_orient.append(g_orient[g])
            corner_sub[(f, k)] = sid
    nsub = len(sub_members)
    rows_s, rows_f, rows_k = [], [], []
    for sid in range(nsub):
        rep = sub_rep[sid]
        for f in sub_members[sid]:
            if any_grp[f]:
                continue
            w = gw[f]
            rows_s.append(sid)
            rows_f.append(f)
            rows_k.append(0 if w[0] == rep else (1 if w[1] == rep else 2))
    s_tan = np.zeros((nsub, 3), _F32)
    if rows_s:
        rs = np.asarray(rows_s)
        rf = np.asarray(rows_f)
        rk = np.asarray(rows_k)
        n = tnor[rf, rk]
        vo, _ = projected(rf, rk)
        p0 = tpos[rf, (rk + 2) % 3]
        p1 = tpos[rf, rk]
        p2 = tpos[rf, (rk + 1) % 3]
        e1, e2 = p0 - p1, p2 - p1
        e1 = _mk_normalize(e1 - _dot(n, e1)[:, None] * n)
        e2 = _mk_normalize(e2 - _dot(n, e2)[:, None] * n)
        cosv = np.clip(_dot(e1, e2), _F32(-1.0), _F32(1.0))
        ang = np.arccos(cosv.astype(np.float64)).astype(_F32)
        np.add.at(s_tan, rs, ang[:, None] * vo)  # sequential, rows in member order
        s_tan = _mk_normalize(s_tan)

    # 7. corners take their subgroup's space; degenerate triangles copy from a good corner
    gi = np.asarray(good)
    for (f, k), sid in corner_sub.items():
        c = 3 * gi[f] + k
        out[c, :3] = s_tan[sid]
        out[c, 3] = 1.0 if sub_orient[sid] else -1.0
    if G < nt:
        firstgood: dict[int, int] = {}
        for f in range(G):
            for k in range(3):
                firstgood.setdefault(gw[f][k], 3 * gi[f] + k)
        for t in np.nonzero(degen)[0]:
            for k in range(3):
                src = firstgood.get(int(weld[t, k]))
                if src is not None:
                    out[3 * t + k] = out[src]
    return out


def tangent_frames(positions, normals, texcoords, indices):
    """Mesh::computeTangentsAndBitangents(force = true) after MikkTSpace: the vertex split
    and the tangent / bitangent finish of Mesh.cpp:397-502. Returns (positions, normals,
    texcoords, tangents, bitangents, indices), float32 / uint32."""
    P = np.asarray(positions, _F32)
    N = np.asarray(normals, _F32)
    nv = len(P)
    U = np.full((nv, 2), 0.5, _F32) if texcoords is None else np.asarray(texcoords, _F32)
    idx = np.asarray(indices, np.int64).reshape(-1).copy()
    if nv == 0 or len(idx) == 0:
        z = np.zeros((nv, 3), _F32)
        return P, N, U, z, z.copy(), idx.astype(np.uint32)
    tg = mikktspace(P, N, U, idx)
    # instances of each vertex in corner order
    order = np.argsort(idx, kind="stable")
    starts = np.searchsorted(idx[order], np.arange(nv + 1))
    new_idx = idx.copy()
    src_vertex, src_corner = [], []
    first_corner = np.full(nv, -1, np.int64)
    tl = tg.tolist()
    for v in range(nv):
        inst = order[starts[v]:starts[v + 1]].tolist()
        if not inst:
            continue
        first_corner[v] = inst[0]
        for r in range(1, len(inst)):
            if tl[inst[r]] == tl[inst[r - 1]]:
                new_idx[inst[r]] = new_idx[inst[r - 1]]
            else:
                new_idx[inst[r]] = nv + len(src_vertex)
                src_vertex.append(v)
                src_corner.append(inst[r])
    sv = np.asarray(src_vertex, np.int64)
    corner_of = np.concatenate([first_corner, np.asarray(src_corner, np.int64)])
    vert_of = np.concatenate([np.arange(nv), sv])
    P2, N2, U2 = P[vert_of], N[vert_of], U[vert_of]
    has = corner_of >= 0
    t4 = np.zeros((len(vert_of), 4), _F32)
    t4[has] = tg[corner_of[has]]
    t = t4[:, :3]
    delta = np.sqrt(_dot(_cross(N2, t), _cross(N2, t)))
    fallback = np.where((np.abs(N2[:, 2]) > _F32(0.01))[:, None], np.array([1, 0, 0], _F32), np.array([0, 0, 1], _F32))
    t = np.where((delta < _F32(0.01))[:, None], fallback, t)
    b = (-t4[:, 3])[:, None] * _cross(N2, t)
    return P2, N2, U2, _glm_normalize(t).astype(_F32), _glm_normalize(b).astype(_F32), new_idx.astype(np.uint32)


def load_obj(data: bytes | str) -> tuple[Mesh, bool]:
    """Resources::getMesh(name, Storage::CPU | Storage::FORCE_FRAME) on the text of an OBJ
    file: the mesh with normals, texture coordinates, tangents and bitangents, and whether
    the file had texture coordinates."""
    obj = parse_obj(data)
    normals = obj.normals if obj.normals is not None else compute_normals(obj.positions, obj.indices)
    p, n, u, t, b, i = tangent_frames(obj.positions, normals, obj.texcoords, obj.indices)
    return Mesh(positions=p, indices=i, normals=n, tangents=t, bitangents=b, texcoords=u), obj.texcoords is not None
