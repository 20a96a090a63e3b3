"""Batched rendering (pt_batch_render): many jobs of different scenes, resolutions, sample
counts and depths in shared waves replayed from one CUDA graph. Every job's image must be
exactly the image pt_render gives for that job alone (same random stream, same summation
order), for any tuning; the autotuner writes its cache."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(R, small=True):
    from rendu_gb300 import scenes as S

    wl = S.batch_workload(seed=11, jobs=6, tri_range=(2_000, 30_000), res_range=(24, 72), spp_range=(1, 32),
                          depth_range=(2, 6))
    wl.append({"scene": S.feature_scene(5), "width": 40, "height": 32, "samples": 8, "depth": 4, "seed": 9})
    out = []
    for j in wl:
        tr = R.PathTracer(j["scene"])
        cam = dict(j["scene"].camera, ratio=j["width"] / j["height"])
        out.append({"tracer": tr, "camera": cam, "samples": j["samples"], "depth": j["depth"], "seed": j["seed"],
                    "image": np.zeros((j["height"], j["width"], 3), np.float32)})
    return out


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_equals_individual_renders(cuda_lib, mode):
    jobs = _jobs(cuda_lib)
    single = []
    for j in jobs:
        img = np.zeros_like(j["image"])
        j["tracer"].render(j["camera"], j["samples"], j["depth"], img, seed=j["seed"], mode=mode)
        single.append(img)
    br = cuda_lib.BatchRenderer(0)
    for tuning in (None, {"wave_paths": 1 << 12, "tile_pixels": 97, "max_samples": 2},
                   {"wave_paths": 1 << 20, "tile_pixels": 1 << 16, "max_samples": 64}):
        for j in jobs:
            j["image"][:] = 0.0
        st = br.render(jobs, mode=mode, tuning=tuning)
        for j, ref in zip(jobs, single):
            assert np.array_equal(j["image"], ref), f"job differs under tuning {tuning}"
        assert st["primary_rays"] == sum(j["image"].shape[0] * j["image"].shape[1] *
                                         2 ** round(np.log2(j["samples"])) for j in jobs)


def test_batch_device_images_and_accumulation(cuda_lib):
    import torch

    jobs = _jobs(cuda_lib)[:3]
    br = cuda_lib.BatchRenderer(0)
    host = []
    for j in jobs:
        j["image"][:] = 1.0
    br.render(jobs)
    host = [j["image"].copy() for j in jobs]
    for j in jobs:
        j["image"] = torch.ones(j["image"].shape, dtype=torch.float32, device="cuda")
    br.render(jobs)
    torch.cuda.synchronize()
    for j, h in zip(jobs, host):
        assert np.array_equal(j["image"].cpu().numpy(), h)


def test_autotune_writes_cache_and_is_used(cuda_lib, tmp_path):
    jobs = _jobs(cuda_lib)[:4]
    br = cuda_lib.BatchRenderer(0)
    path = str(tmp_path / "tuning.json")
    t = br.autotune(jobs, cache_path=path)
    assert os.path.exists(path)
    cached = json.load(open(path))
    assert cached["wave_paths"] == t["wave_paths"] and cached["tile_pixels"] == t["tile_pixels"]
    os.environ["RENDU_GB300_TUNING"] = path
    try:
        for j in jobs:
            j["image"][:] = 0.0
        br.render(jobs)  # picks up the cached tuning
    finally:
        del os.environ["RENDU_GB300_TUNING"]
    for j in jobs:
        assert np.isfinite(j["image"]).all() and j["image"].mean() > 0
