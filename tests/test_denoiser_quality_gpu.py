"""What the learned denoiser gains over the plain path tracer: a short training on pairs the
path tracer renders (one scene of the large workload's type), then on a view of a held-out
scene the denoised image must have a lower relative RMSE against a high-sample render than
plain path tracing given the same wall time (the render plus the denoising)."""
import pytest

pytestmark = pytest.mark.gpu


def test_denoiser_beats_plain_path_tracing_at_equal_time(cuda_lib):
    import torch

    from rendu_gb300 import denoiser as D
    from rendu_gb300 import scenes as S

    tr = cuda_lib.PathTracer(S.denoiser_scene(20261301, instances=30))
    feats, targets = D.render_pairs(tr, S.random_cameras(20261301, 24), 128, 128, spp_in=[8, 32, 128],
                                    spp_ref=lambda s: 8 * s, seed=5)
    tr.close()
    net = D.Denoiser(seed=3)
    losses = D.train(net, feats, targets, 800, batch=8, crop=64, lr=1e-3, seed=2, log_every=200)
    assert losses[-1][1] < losses[0][1]

    held = cuda_lib.PathTracer(S.denoiser_scene(20261302, instances=30))
    cam = S.random_cameras(20261302, 1)[0]
    w = h = 128
    truth = torch.zeros((h, w, 3), device="cuda")
    held.render(dict(cam, ratio=1.0), 4096, 5, truth, seed=9, mode=1, fp64=True)
    curve = D.progressive_curves(held, cam, w, h, (16, 32, 64, 128, 256, 512, 1024), truth, denoiser=net, seed=40)
    held.close()
    for p in curve[:3]:  # 16, 32, 64 samples + denoising vs plain path tracing with the same time
        t_den = p["render_s"] + p["denoise_ms"] / 1e3
        rival = next((q for q in curve if q["render_s"] >= t_den), curve[-1])
        assert p["denoised"] < rival["plain"], (p, rival)
        assert p["denoised"] < 0.8 * p["plain"]
