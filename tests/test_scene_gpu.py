"""Scenes loaded from the reference's file format, rendered on the GPU.

* The demo scene (tests/golden/scene_demo: its own meshes, PNG / EXR textures, cube-map
  background, point / spot / directional lights, a masked and an emissive material, an
  object that skips UVs, a scene-wide transformation) rendered by the device path tracer
  against the C restatement on the same random stream.
* The command-line render (python -m rendu_gb300): the image it writes equals the image
  rendered through the API and saved with save_image, for PNG and EXR outputs.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from render_stats import rel_rmse

pytestmark = pytest.mark.gpu

DEMO_SCENE = os.path.join(GOLDEN, "scene_demo", "demo.scene")


def test_demo_scene_matches_port_on_the_same_random_stream(cuda_lib, port_lib):
    from rendu_gb300 import sceneio

    ls = sceneio.load_scene(DEMO_SCENE)
    sc = ls.scene
    w, h, spp, depth = 64, 48, 16, 5
    cam = dict(ls.camera, ratio=w / h)
    gpu = cuda_lib.PathTracer(sc)
    img = np.zeros((h, w, 3), np.float32)
    gpu.render(cam, spp, depth, img, seed=21)
    port = port_lib.PortPathTracer(sc)
    ref = port.render(cam, spp, depth, w, h, seed=21)
    assert np.isfinite(img).all() and img.mean() > 0.05
    rel = np.abs(img - ref) / (np.abs(ref) + 1e-2)
    assert np.mean(rel < 1e-3) > 0.95, f"only {np.mean(rel < 1e-3):.3f} of values agree to 1e-3"
    assert rel_rmse(img, ref) < 0.05
    st = gpu.last_stats()
    assert st["primary_rays"] == w * h * spp == int(port.rays[0])
    assert abs(st["shadow_rays"] - int(port.rays[2])) <= 0.01 * port.rays[2] + 10
    gpu.close()


def test_command_line_render(cuda_lib, tmp_path):
    from rendu_gb300 import sceneio
    from rendu_gb300.__main__ import main
    from rendu_gb300.pathtracer import PathTracer, save_image

    w, h = 48, 32
    png = str(tmp_path / "cli.png")
    exr = str(tmp_path / "cli.exr")
    assert main(["--scene", DEMO_SCENE, "--samples", "3", "--depth", "4", "--size", str(w), str(h), "--output", png,
                 "--seed", "5", "--render"]) == 0
    assert main(["--scene", DEMO_SCENE, "--samples", "4", "--depth", "4", "--size", str(w), str(h), "--output", exr,
                 "--seed", "5"]) == 0
    ls = sceneio.load_scene(DEMO_SCENE)
    tracer = PathTracer(ls.scene)
    img = np.zeros((h, w, 3), np.float32)
    tracer.render(dict(ls.camera, ratio=float(np.float32(w) / np.float32(h))), 4, 4, img, seed=5)  # 3 -> 4 spp
    tracer.close()
    api_png = str(tmp_path / "api.png")
    api_exr = str(tmp_path / "api.exr")
    save_image(img, api_png, tonemap=True)
    save_image(img, api_exr, tonemap=False)
    assert open(png, "rb").read() == open(api_png, "rb").read()
    assert open(exr, "rb").read() == open(api_exr, "rb").read()
    assert main(["--scene", "no_such_scene", "--output", str(tmp_path / "x.png")]) == 1
