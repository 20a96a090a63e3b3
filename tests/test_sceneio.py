"""Scene loading (rendu_gb300.sceneio / meshio / imageio) against the reference's own loaders.

The golden fixtures (tests/golden/scene_io.npz, made by tests/golden/make_golden.py
--scene-io) hold what the reference's code returns for the demo scene's files
(tests/golden/scene_demo, made by its make_scene.py) and for seeded synthetic inputs:
  * meshes: the reference's mesh loading (OBJ Indexed loader, computeNormals, its own
    mikktspace.c and the vertex split of computeTangentsAndBitangents);
  * MikkTSpace per-corner output on stress meshes (UV islands, mirrored UVs, degenerate
    triangles, exactly opposite tangents around a pole, constant UVs);
  * textures: stb_image / tinyexr through Image::load, on the demo textures and on PNGs of
    every colour type and bit depth (colour-key and palette transparency, interlacing);
  * transformations: glm's translate * rotate * scale.
Every comparison is bit-exact. Where the reference tree is present the same checks also run
directly against it, on all of its OBJ meshes, PNG and EXR files and scenes.
Host code only: runs without a GPU."""
import glob
import os
import sys
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

DEMO = os.path.join(GOLDEN, "scene_demo")
def _ref_root():
    from oracle.oracle import reference_root

    return reference_root()


REF_RES = os.path.join(_ref_root(), "resources")


def _golden_module():
    ns = {"__name__": "make_golden", "__file__": os.path.join(GOLDEN, "make_golden.py")}
    src = open(os.path.join(GOLDEN, "make_golden.py")).read()
    exec(compile(src, "make_golden.py", "exec"), ns)  # defines the case generators only
    return ns


@pytest.fixture(scope="module")
def golden():
    return load_golden("scene_io.npz")


@pytest.fixture(scope="module")
def lib():
    from rendu_gb300 import build

    build.build()


def _bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                                                 b.view(np.uint32) if b.dtype == np.float32 else b)


def _ref_or_skip():
    from oracle import oracle as O

    if not os.path.isdir(REF_RES) or O.build_ref() is None:
        pytest.skip("reference tree not present")
    return O


# --------------------------------------------------------------------------------------
# the .scene text format
# --------------------------------------------------------------------------------------


def test_decode_tokens():
    from rendu_gb300.sceneio import decode

    text = (" stray: 1 2  # before any root: dropped\n"
            "* object: # a root\n"
            "\tmesh: crate   \n"
            "\tno colon here\n"
            "\ttranslation: 1.0,2.0 , 3.0\n"
            "\ttextures:\n"
            "\t\t- srgb: 0.8,0.8,0.8\n"
            "\t\t- rgb: default_normal\n"
            "\tcube: rgb32cube: sky: deeper\n"
            "*material:\n"
            "\t- orphan: 1\n"
            "\t- child: 2\n"
            "\tname:\n")
    roots = decode(text)
    assert [r.key for r in roots] == ["object", "material"]
    obj = roots[0]
    assert [e.key for e in obj.elements] == ["mesh", "translation", "textures", "cube"]
    assert obj.elements[0].values == ["crate"]
    assert obj.elements[1].values == ["1.0", "2.0", "3.0"]
    tex = obj.elements[2]
    assert [(t.key, t.values) for t in tex.elements] == [("srgb", ["0.8", "0.8", "0.8"]), ("rgb", ["default_normal"])]
    cube = obj.elements[3]
    assert cube.values == [] and cube.elements[0].key == "rgb32cube"
    assert cube.elements[0].elements[0].key == "sky" and cube.elements[0].elements[0].values == ["deeper"]
    mat = roots[1]
    # a '-' line right after a root is an ordinary element (its key keeps the dash); the next
    # '-' line becomes its array element
    assert mat.elements[0].key == "- orphan" and mat.elements[0].elements[0].key == "child"
    assert mat.elements[1].key == "name" and mat.elements[1].values == []


def test_transformations_match_glm(golden):
    from rendu_gb300.sceneio import KeyValues, decode_transformation

    for a, g, t, s, ref in zip(golden["tf_axis"], golden["tf_angle"], golden["tf_trans"], golden["tf_scale"],
                               golden["tf_out"]):
        kv = [KeyValues("orientation", [repr(float(x)) for x in a] + [repr(float(g))]),
              KeyValues("translation", [repr(float(x)) for x in t]), KeyValues("scaling", [repr(float(s))])]
        assert _bits_equal(decode_transformation(kv), ref)
    assert _bits_equal(decode_transformation([]), np.eye(4, dtype=np.float32))


def test_matrix_product_order():
    from rendu_gb300.sceneio import mat_mul

    rng = np.random.default_rng(0)
    a, b = rng.normal(size=(2, 4, 4)).astype(np.float32)
    expect = np.zeros((4, 4), np.float32)
    for i in range(4):
        for j in range(4):
            acc = np.float32(0)
            for k in range(4):
                acc = np.float32(acc + a[i, k] * b[k, j]) if k else np.float32(a[i, k] * b[k, j])
            expect[i, j] = acc
    assert _bits_equal(mat_mul(a, b), expect)


# --------------------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------------------


@pytest.mark.parametrize("name", ["demo_ball", "demo_crate", "demo_floor", "demo_leaf", "demo_lamp"])
def test_obj_meshes_match_reference(golden, name):
    from rendu_gb300 import meshio

    m, had = meshio.load_obj(open(os.path.join(DEMO, name + ".obj"), "rb").read())
    for k in ("positions", "normals", "texcoords", "tangents", "bitangents", "indices"):
        assert _bits_equal(getattr(m, k), golden[f"obj_{name}_{k}"]), k
    assert had == bool(golden[f"obj_{name}_had_uv"])


@pytest.mark.parametrize("name", ["grid_islands", "soup", "pole_fan", "constant_uv"])
def test_mikktspace_matches_reference(golden, name):
    from rendu_gb300 import meshio

    out = meshio.mikktspace(golden[f"mk_{name}_in_pos"], golden[f"mk_{name}_in_nor"], golden[f"mk_{name}_in_uv"],
                            golden[f"mk_{name}_in_idx"])
    assert _bits_equal(out, golden[f"mk_{name}_out"])


def test_obj_token_rules():
    """Face tokens are read with the reference's substring rules: no slash -> the position
    index serves all three; one slash -> the texture index is the substring of length
    first-slash-position after it (so "12/345" reads texture coordinate 34)."""
    from rendu_gb300 import meshio

    v = "\n".join(f"v {i} 0 0" for i in range(40))
    vt = "\n".join(f"vt {i / 400:.4f} 0.5" for i in range(400))
    o = meshio.parse_obj(v + "\n" + vt + "\nf 12/345 2/3 3/4\nf 1 2 3\n# comment\nf 12/345 1 2 9\n")
    assert list(o.indices) == [0, 1, 2, 3, 4, 5, 0, 3, 4]
    np.testing.assert_array_equal(o.positions[:, 0], [11, 1, 2, 0, 1, 2])
    np.testing.assert_array_equal(o.texcoords[:, 0], np.float32([33 / 400, 2 / 400, 3 / 400, 0, 1 / 400, 2 / 400]))
    assert o.normals is None
    with pytest.raises(meshio.MeshFormatError):
        meshio.parse_obj("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n")
    with pytest.raises(meshio.MeshFormatError):
        meshio.parse_obj("v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nf 1//1 2//1 3//1\n")
    assert len(meshio.parse_obj("# nothing\n").positions) == 0


def test_normals_and_frames_when_missing():
    """A mesh without normals gets computeNormals' area-independent face sums; a mesh
    without texture coordinates gets the constant ones and tangents from the fallback."""
    from rendu_gb300 import meshio

    m, had = meshio.load_obj("v 0 0 0\nv 1 0 0\nv 0 0 -1\nv 1 0 -1\nf 1 2 3\nf 2 4 3\n")
    assert not had
    np.testing.assert_allclose(m.normals, np.tile(np.float32([0, 1, 0]), (4, 1)), atol=1e-7)
    np.testing.assert_array_equal(m.texcoords, np.full((4, 2), 0.5, np.float32))
    np.testing.assert_array_equal(m.tangents, np.tile(np.float32([1, 0, 0]), (4, 1)))
    np.testing.assert_allclose(np.abs(m.bitangents), np.tile([0, 0, 1], (4, 1)))


def test_reference_meshes_directly():
    O = _ref_or_skip()
    from rendu_gb300 import meshio

    paths = sorted(glob.glob(os.path.join(REF_RES, "**", "*.obj"), recursive=True))
    assert paths
    for p in paths:
        txt = open(p, "rb").read()
        r = O.ref_mesh_load_obj(txt)
        m, had = meshio.load_obj(txt)
        for k in ("positions", "normals", "texcoords", "tangents", "bitangents", "indices"):
            assert _bits_equal(getattr(m, k), r[k]), (p, k)
        assert had == r["had_uv"]


def test_random_meshes_against_reference_mikktspace():
    O = _ref_or_skip()
    from rendu_gb300 import meshio

    rng = np.random.default_rng(11)
    for trial in range(20):
        nv = int(rng.integers(4, 80))
        p = rng.normal(size=(nv, 3)).astype(np.float32)
        if trial % 3 == 0:
            p[rng.integers(0, nv, nv // 4)] = p[0]  # coincident positions -> degenerate triangles
        n = (p / np.linalg.norm(p, axis=1, keepdims=True)).astype(np.float32)
        u = rng.uniform(0, 1, (nv, 2)).astype(np.float32)
        if trial % 4 == 1:
            u = np.round(u * 2) / 2  # many equal UVs -> UV-degenerate triangles
        t = rng.integers(0, nv, (int(rng.integers(1, 3 * nv)), 3))
        t = t[(t[:, 0] != t[:, 1]) & (t[:, 1] != t[:, 2]) & (t[:, 0] != t[:, 2])].reshape(-1).astype(np.uint32)
        if len(t) == 0:
            continue
        assert _bits_equal(meshio.mikktspace(p, n, u, t), O.ref_mikktspace(p, n, u, t)), trial


# --------------------------------------------------------------------------------------
# textures
# --------------------------------------------------------------------------------------


def _assert_jpeg_close(a, b, what):
    """JPEG samples: the inverse DCT, chroma upsampling and colour conversion are exact here
    and fixed-point in stb_image, so samples may differ by a few 1/255 steps."""
    assert a.shape == b.shape, what
    d = np.abs(a.astype(np.float64) - b) * 255.0
    assert d.max() <= 3.01 and d.mean() < 0.1 and (d > 1.01).mean() < 0.05, (what, d.max(), d.mean())


def test_demo_textures_match_reference(golden, lib):
    from rendu_gb300 import imageio

    files = sorted(glob.glob(os.path.join(DEMO, "*.png")) + glob.glob(os.path.join(DEMO, "*.exr"))
                   + glob.glob(os.path.join(DEMO, "*.jpg")))
    assert len(files) == 12
    for path in files:
        ref = golden[f"img_{os.path.basename(path)}"]
        if path.endswith(".jpg"):
            _assert_jpeg_close(imageio.load_image(path, 4), ref, path)
        else:
            assert _bits_equal(imageio.load_image(path, 4), ref), path


def test_jpeg_errors(lib):
    from rendu_gb300 import imageio

    data = open(os.path.join(DEMO, "demo_crate_color.jpg"), "rb").read()
    img = imageio.decode_jpeg(data, 3)
    assert img.shape == (58, 46, 3)
    np.testing.assert_array_equal(imageio.decode_jpeg(data, 4)[..., 3], 1.0)
    grey = imageio.decode_jpeg(data, 1)[..., 0]
    rgb255 = np.rint(img * 255).astype(np.int32)
    expect = (rgb255[..., 0] * 77 + rgb255[..., 1] * 150 + rgb255[..., 2] * 29) >> 8
    np.testing.assert_array_equal(np.rint(grey * 255).astype(np.int32), expect)
    for bad in (data[:40], data[:2] + b"\xff\xc9\x00\x0b" + bytes(9) + data[2:], b"\xff\xd8\xff\xd9"):
        with pytest.raises(imageio.ImageFormatError, match="JPEG"):
            imageio.decode_jpeg(bad)
    # a truncated entropy-coded segment decodes to something, without reading out of bounds
    out = imageio.decode_jpeg(data[: len(data) - 200] + b"\xff\xd9")
    assert out.shape == (58, 46, 4)


def test_png_variants_match_stb(golden, lib):
    from rendu_gb300 import imageio

    sys.path.insert(0, DEMO)
    import make_scene as MS

    ns = _golden_module()
    with tempfile.TemporaryDirectory() as d:
        for name, samples, kw in ns["png_variants"]():
            path = os.path.join(d, name + ".png")
            MS.write_png(path, samples, **kw)
            for ch in (3, 4):
                assert _bits_equal(imageio.load_image(path, ch), golden[f"png_{name}_{ch}"]), (name, ch)


def test_image_flip_and_errors(lib, tmp_path):
    from rendu_gb300 import imageio

    img = imageio.load_image(os.path.join(DEMO, "demo_checker.png"), 4)
    np.testing.assert_array_equal(imageio.load_image(os.path.join(DEMO, "demo_checker.png"), 4, flip=True), img[::-1])
    bad = tmp_path / "x.jpg"
    bad.write_bytes(b"\xff\xd8\xff\xe0rest")
    with pytest.raises(imageio.ImageFormatError, match="x.jpg"):
        imageio.load_image(str(bad))
    data = bytearray(open(os.path.join(DEMO, "demo_checker.png"), "rb").read())
    with pytest.raises(imageio.ImageFormatError):
        imageio.decode_png(bytes(data[:60]))


def test_reference_images_directly(lib):
    O = _ref_or_skip()
    from rendu_gb300 import imageio

    paths = sorted(glob.glob(os.path.join(REF_RES, "**", "*.png"), recursive=True)
                   + glob.glob(os.path.join(REF_RES, "**", "*.exr"), recursive=True))
    assert paths
    for p in paths:
        assert _bits_equal(imageio.load_image(p, 4), O.ref_load_image(p, 4, max_pixels=1 << 24)), p
    jpegs = sorted(glob.glob(os.path.join(REF_RES, "**", "*.jpg"), recursive=True))
    assert jpegs  # progressive and sequential, 4:2:0 and 4:4:4, grey
    for p in jpegs:
        _assert_jpeg_close(imageio.load_image(p, 4), O.ref_load_image(p, 4, max_pixels=1 << 24), p)


# --------------------------------------------------------------------------------------
# whole scenes
# --------------------------------------------------------------------------------------


def test_demo_scene_structure(lib):
    from rendu_gb300 import sceneio

    ls = sceneio.load_scene(os.path.join(DEMO, "demo.scene"))
    sc = ls.scene
    # objects ordered by material type: the four Regular ones in file order, then Emissive
    assert ls.object_names == ["demo_floor", "demo_ball", "demo_crate", "demo_leaf", "demo_lamp"]
    assert [sc.materials[o["material"]]["type"] for o in sc.objects] == [1, 1, 1, 1, 8]
    assert [sc.materials[o["material"]]["masked"] for o in sc.objects] == [False, False, False, True, False]
    # skipuvs: the crate's mesh has no texture coordinates; the lamp keeps the constant ones
    has_uv = [sc.meshes[o["mesh"]].texcoords is not None for o in sc.objects]
    assert has_uv == [True, True, False, True, True]
    np.testing.assert_array_equal(sc.meshes[sc.objects[4]["mesh"]].texcoords, np.full((4, 2), 0.5, np.float32))
    # the scene transformation premultiplies every object's own
    from rendu_gb300.sceneio import KeyValues, decode_transformation, mat_mul

    scene_m = decode_transformation([KeyValues("orientation", ["0.0", "1.0", "0.0", "0.3"]),
                                     KeyValues("translation", ["0.0", "-0.1", "0.0"])])
    ball = decode_transformation([KeyValues("translation", ["-0.5", "0.5", "0.0"]), KeyValues("scaling", ["0.5"])])
    np.testing.assert_array_equal(sc.objects[1]["model"], mat_mul(scene_m, ball))
    # lights in file order, spot cone halved, directions normalised
    assert [l["type"] for l in sc.lights] == [0, 2, 1]
    spot = sc.lights[1]
    assert spot["inner"] == pytest.approx(0.4) and spot["outer"] == pytest.approx(0.6) and not spot["shadows"]
    assert np.linalg.norm(spot["direction"]) == pytest.approx(1.0, abs=1e-6)
    assert sc.lights[0]["radius"] == 4.0 and sc.lights[0]["shadows"]
    # cube-map background: six faces, rows flipped
    assert sc.background["mode"] == 2 and len(set(sc.background["tex"])) == 6
    from rendu_gb300 import imageio

    face = sc.textures[sc.background["tex"][3]]
    np.testing.assert_array_equal(face, imageio.load_image(os.path.join(DEMO, "demo_sky_py.exr"), 4)[::-1])
    # constant-colour textures: 8 x 8 RGBA, alpha 1 when not given
    ball_mat = sc.materials[sc.objects[1]["material"]]
    np.testing.assert_array_equal(sc.textures[ball_mat["tex"][0]], np.broadcast_to(np.float32([0.8, 0.3, 0.2, 1.0]),
                                                                                    (8, 8, 4)))
    assert ls.camera["fov"] == pytest.approx(1.1) and ls.planes == pytest.approx((0.01, 50.0))


def test_scene_errors(lib, tmp_path):
    from rendu_gb300 import sceneio

    base = open(os.path.join(DEMO, "demo.scene")).read()
    cases = {
        "missing material": base.replace("material: ball_mat", "material: nothing"),
        "unable to load mesh": base.replace("mesh: demo_ball", "mesh: no_such_mesh"),
        "unknown block": base + "\n* teapot:\n\tsize: 1\n",
        "unable to find texture": base.replace("srgb: demo_checker", "srgb: no_such_texture"),
        "planes": base.replace("planes: 0.01 50.0", "planes: 5.0 1.0"),
        "unknown material type": base.replace("type: Emissive", "type: Glowing"),
    }
    for msg, text in cases.items():
        p = tmp_path / "bad.scene"
        p.write_text(text)
        with pytest.raises(sceneio.SceneError, match=msg):
            sceneio.load_scene(str(p), resources=[DEMO])
    with pytest.raises(sceneio.SceneError, match="unable to find scene"):
        sceneio.load_scene("no_such_scene", resources=[DEMO])
    # by name through the resources index
    assert sceneio.load_scene("demo", resources=[DEMO]).name == "demo"


def test_reference_scenes_load(lib):
    _ref_or_skip()
    from rendu_gb300 import imageio, sceneio

    roots = [os.path.join(REF_RES, "common"), os.path.join(REF_RES, "pbrdemo")]
    ls = sceneio.load_scene("cornellbox", resources=roots)
    sc = ls.scene
    assert len(sc.objects) == 8 and sc.triangle_count == 32 and len(sc.lights) == 1
    assert ls.camera["eye"] == pytest.approx((0.0, 1.0, 2.5)) and ls.camera["fov"] == pytest.approx(1.3)
    assert all(sc.meshes[o["mesh"]].texcoords is None for o in sc.objects)  # every object skips UVs
    assert sc.background == {"mode": 0, "color": (0.0, 0.0, 0.0), "tex": (0,) * 6}
    counts = {"furnace-test": 22, "parameter-spheres": 22, "boxes": 443, "multi-probes": 3, "cornellbox-emissive": 7,
              "cornellbox-cutout": 7, "cornellbox-parallax": 3, "cornellbox-reflections": 8, "cornellbox-textured": 8,
              "cornellbox-transparent": 7, "gallery-materials": 52}
    for name, objects in counts.items():
        assert len(sceneio.load_scene(name, resources=roots).scene.objects) == objects, name
    cut = sceneio.load_scene("cornellbox-cutout", resources=roots).scene
    assert any(m["masked"] for m in cut.materials) and [l["type"] for l in cut.lights] == [2, 2]
    assert sceneio.load_scene("cornellbox-reflections", resources=roots).scene.background["mode"] == 3
    del imageio


def test_cli_arguments():
    from rendu_gb300.__main__ import _parse

    a = _parse(["--scene", "cornellbox", "--size", "320", "200", "--samples", "6", "--render"])
    assert a.size == [320, 200] and a.samples == 6 and a.depth == 5 and a.render and a.resources == []
