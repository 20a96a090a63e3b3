"""Display geometry of the hierarchy inspection (rendu_gb300.raycaster._box_meshes,
save_line_obj): RaycasterVisualisation::createBVHMeshes's layout -- BoundingBox::getCorners'
corner order, 12 edges as degenerate triangles, one mesh per depth coloured by glm's
hue/saturation/value conversion of (300 d^2, 1, 0.75 - 0.5 d^2). Host code only."""
import numpy as np

from rendu_gb300 import raycaster as R


def test_box_mesh_layout():
    boxes = np.array([[0, 0, 0, 2, 4, 8], [0, 0, 0, 1, 1, 1], [1, 1, 1, 2, 2, 2]], np.float32)
    ms = R._box_meshes(boxes, np.array([0, 1, 1]))
    assert [m["name"] for m in ms] == ["Level 0", "Level 1"]
    corners = ms[0]["positions"]
    # x slowest, z fastest (Bounds.cpp:37-47)
    np.testing.assert_array_equal(corners, [[0, 0, 0], [0, 0, 8], [0, 4, 0], [0, 4, 8], [2, 0, 0], [2, 0, 8],
                                            [2, 4, 0], [2, 4, 8]])
    edges = {tuple(sorted(t[:2])) for t in ms[0]["indices"].reshape(-1, 3)}
    assert len(edges) == 12 and all(bin(a ^ b).count("1") == 1 for a, b in edges)  # box edges only
    assert ms[1]["indices"].max() == 15 and len(ms[1]["indices"]) == 72
    np.testing.assert_allclose(ms[0]["colors"][0], [0.75, 0.0, 0.0])  # depth 0: hue 0, value 0.75
    np.testing.assert_allclose(ms[1]["colors"][0], [0.25, 0.0, 0.25], atol=1e-6)  # depth 1: hue 300, value 0.25
    assert R._box_meshes(np.zeros((0, 6), np.float32), np.zeros(0, np.int32)) == []


def test_hsv_sectors():
    for h, expect in ((0, (1, 0, 0)), (60, (1, 1, 0)), (120, (0, 1, 0)), (180, (0, 1, 1)), (240, (0, 0, 1)),
                      (300, (1, 0, 1)), (30, (1, 0.5, 0))):
        np.testing.assert_allclose(R._hsv_to_rgb(h, 1.0, 1.0), expect, atol=1e-6)
    np.testing.assert_allclose(R._hsv_to_rgb(123, 0.0, 0.4), (0.4, 0.4, 0.4))


def test_line_obj(tmp_path):
    boxes = np.array([[0, 0, 0, 1, 1, 1], [0, 0, 0, 0.5, 0.5, 0.5]], np.float32)
    ms = R._box_meshes(boxes, np.array([0, 1]))
    path = tmp_path / "levels.obj"
    R.save_line_obj(ms, str(path))
    lines = path.read_text().splitlines()
    assert lines[0] == "g Level_0" and "g Level_1" in lines
    assert sum(x.startswith("v ") for x in lines) == 16 and sum(x.startswith("l ") for x in lines) == 24
    ls = [tuple(map(int, x.split()[1:])) for x in lines if x.startswith("l ")]
    assert min(min(x) for x in ls) == 1 and max(max(x) for x in ls) == 16  # 1-based, offset per group
