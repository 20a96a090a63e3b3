"""Hierarchy inspection (rt_hierarchy_boxes, rt_ray_levels; RaycasterVisualisation in
rendu_gb300.raycaster): the display geometry of the reference's RaycasterVisualisation for
this library's own hierarchy.

* Every node box is listed once, breadth first with its depth; children lie inside their
  parents; the leaves hold every triangle once and bound it.
* A ray's levels end in the same closest hit as rt_intersect (bit for bit), and every box
  it lists is entered by the ray.
* The meshes are the reference's: 8 corners and 12 edges per box, one mesh per depth, ray
  mesh green on a hit with the hit triangle appended.
"""
import numpy as np
import pytest

from conftest import golden_meshes, load_golden

pytestmark = pytest.mark.gpu


def _rc(R):
    g = load_golden("raycaster_small.npz")
    rc = R.Raycaster(0)
    for pos, idx, m in golden_meshes(g):
        rc.add_mesh(pos, idx, m)
    rc.updateHierarchy()
    return rc, g


def test_all_levels(cuda_lib):
    from rendu_gb300.raycaster import RaycasterVisualisation

    rc, g = _rc(cuda_lib)
    vis = RaycasterVisualisation(rc)
    boxes, info, _ = vis._call("rt_hierarchy_boxes")
    st = rc.stats()
    depth, tris = info[:, 0], info[:, 1]
    assert depth[0] == 0 and (np.diff(depth) >= 0).all()  # breadth first
    assert (tris > 0).sum() == st["leaves"] and tris.sum() == st["triangles"]
    assert (tris == 0).sum() == st["nodes"]  # the root box + every inner child
    assert (boxes[:, :3] <= boxes[:, 3:]).all()
    root = boxes[0]
    assert (boxes[:, :3] >= root[:3] - 1e-3).all() and (boxes[:, 3:] <= root[3:] + 1e-3).all()
    meshes = vis.getAllLevels()
    assert [m["name"] for m in meshes] == [f"Level {d}" for d in range(depth.max() + 1)]
    for d, m in enumerate(meshes):
        k = int((depth == d).sum())
        assert m["positions"].shape == (8 * k, 3) and m["indices"].shape == (36 * k,) and m["colors"].shape == (8 * k, 3)
    # deeper levels are darker (value 0.75 - 0.5 depth^2)
    assert meshes[0]["colors"][0].max() > meshes[-1]["colors"][0].max()


def test_ray_levels_end_in_the_closest_hit(cuda_lib):
    from rendu_gb300.raycaster import RaycasterVisualisation

    rc, g = _rc(cuda_lib)
    vis = RaycasterVisualisation(rc)
    rays = np.ascontiguousarray(g["rays"][:400])
    ref = rc.intersect_batch(rays)
    hits = 0
    for i, ray in enumerate(rays.view(np.float32).reshape(-1, 8)):
        boxes, info, hit = vis._call("rt_ray_levels", rays[i:i + 1].ctypes.data)
        assert hit["prim"] == ref["prim"][i]
        assert hit["t"].view(np.uint32) == ref["t"][i].view(np.uint32)
        if hit["prim"] != 0xFFFFFFFF:
            hits += 1
            assert hit["u"].view(np.uint32) == ref["u"][i].view(np.uint32)
        if len(boxes):
            o, d = ray[:3].astype(np.float64), ray[4:7].astype(np.float64)
            d /= np.linalg.norm(d)
            with np.errstate(divide="ignore", invalid="ignore"):
                t0 = (boxes[:, :3] - o) / d
                t1 = (boxes[:, 3:] - o) / d
            tn = np.nanmax(np.minimum(t0, t1), axis=1)
            tf = np.nanmin(np.maximum(t0, t1), axis=1)
            assert (tn <= tf + 1e-3 * (1 + np.abs(tf))).all(), f"ray {i} lists a box it misses"
    assert hits > 10
    r = rays.view(np.float32).reshape(-1, 8)
    k = int(np.nonzero(ref["prim"] != 0xFFFFFFFF)[0][0])
    meshes, h = vis.getRayLevels(tuple(r[k, :3]), tuple(r[k, 4:7]), float(r[k, 3]), float(r[k, 7]))
    assert h == rc.intersects(tuple(r[k, :3]), tuple(r[k, 4:7]), float(r[k, 3]), float(r[k, 7])) and h.hit
    assert meshes and meshes[0]["name"] == "Level 0"


def test_ray_mesh(cuda_lib, tmp_path):
    from rendu_gb300.raycaster import RaycasterVisualisation, save_line_obj

    rc, g = _rc(cuda_lib)
    vis = RaycasterVisualisation(rc)
    r = g["rays"].view(np.float32).reshape(-1, 8)
    ref = rc.intersect_batch(g["rays"])
    i = int(np.nonzero(ref["prim"] != 0xFFFFFFFF)[0][0])
    j = int(np.nonzero(ref["prim"] == 0xFFFFFFFF)[0][0])
    hit = rc.intersects(tuple(r[i, :3]), tuple(r[i, 4:7]), float(r[i, 3]), float(r[i, 7]))
    assert hit.hit
    m = vis.getRayMesh(r[i, :3], r[i, 4:7], hit)
    assert m["positions"].shape == (5, 3) and list(m["indices"]) == [0, 1, 0, 2, 3, 4]
    assert (m["colors"] == [0, 1, 0]).all()
    # the segment ends on the hit triangle's plane
    a, b, c = m["positions"][2:]
    n = np.cross(b - a, c - a)
    assert abs(np.dot(m["positions"][1] - a, n)) <= 1e-4 * np.linalg.norm(n) * (1 + np.abs(a).max())
    miss_hit = rc.intersects(tuple(r[j, :3]), tuple(r[j, 4:7]), float(r[j, 3]), float(r[j, 7]))
    assert not miss_hit.hit
    miss = vis.getRayMesh(r[j, :3], r[j, 4:7], miss_hit, 2.0)
    assert miss["positions"].shape == (2, 3) and (miss["colors"] == [1, 0, 0]).all()
    path = tmp_path / "bvh.obj"
    levels = vis.getAllLevels()
    save_line_obj(levels + [m], str(path))
    lines = path.read_text().splitlines()
    assert sum(x.startswith("l ") for x in lines) == sum(len(x["indices"]) // 3 for x in levels) + 2
    assert sum(x.startswith("v ") for x in lines) == sum(len(x["positions"]) for x in levels) + 5
