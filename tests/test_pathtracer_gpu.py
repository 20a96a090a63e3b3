"""Parity of the sm_103a path tracer with the reference.

* Material functions against the reference's golden vectors (same uniforms in).
* Whole renders against the C restatement driven by the SAME Philox stream: the two
  differ only where float rounding (FMA contraction, transcendental ulps) flips a
  decision, so nearly every pixel agrees to ~1e-4.
* Whole renders against the reference's own renders at equal spp, statistically.
* Exact answers: background-only and emitter-only views, the accumulate-and-normalise
  contract, sample-count rounding, depth 0, 4-component images, device images.
"""
import numpy as np
import pytest

from conftest import load_golden
from render_stats import assert_same_distribution, rel_rmse

pytestmark = pytest.mark.gpu


def _scene(name):
    from rendu_gb300 import scenes as S

    return {"cornell": lambda: S.cornell_scene(20261203), "cornell_lit": lambda: S.cornell_scene(20261203, True),
            "mixed": lambda: S.feature_scene(20261203),
            "instanced": lambda: S.instanced_scene(20261206)}[name]()


def test_material_matches_reference(cuda_lib):
    from rendu_gb300 import pathtracer as P

    g = load_golden("material_ggx.npz")
    ev = P.material_eval(g["eval_in"])
    # Transcendentals (powf) may differ by an ulp from the host C library; cases where the
    # GGX D term cancels (roughness 0.045 -> alpha 0.002, NdotH ~ 1) amplify that.
    close = np.isclose(ev, g["eval_out"], rtol=2e-5, atol=1e-6)
    assert close.mean() > 0.998, f"{(~close).sum()} of {close.size} values differ"
    np.testing.assert_allclose(ev, g["eval_out"], rtol=2e-3, atol=1e-5)
    sm = P.material_sample(g["sample_in"], g["sample_uniforms"])
    close = np.isclose(sm, g["sample_out"], rtol=2e-4, atol=2e-5).all(axis=1)
    assert close.mean() > 0.999, f"{(~close).sum()} of {len(close)} samples differ"


@pytest.mark.parametrize("name,spp,depth", [("cornell", 16, 5), ("cornell_lit", 8, 5), ("mixed", 8, 4),
                                            ("instanced", 4, 8)])
def test_render_matches_port_on_the_same_random_stream(cuda_lib, port_lib, name, spp, depth):
    sc = _scene(name)
    w, h = 64, 48
    cam = dict(sc.camera, ratio=w / h)
    gpu = cuda_lib.PathTracer(sc)
    img = np.zeros((h, w, 3), np.float32)
    gpu.render(cam, spp, depth, img, seed=99)
    port = port_lib.PortPathTracer(sc)
    ref = port.render(cam, spp, depth, w, h, seed=99)
    rel = np.abs(img - ref) / (np.abs(ref) + 1e-2)
    assert np.isfinite(img).all()
    assert np.mean(rel < 1e-3) > 0.97, f"only {np.mean(rel < 1e-3):.3f} of values agree to 1e-3"
    assert rel_rmse(img, ref) < 0.05
    st = gpu.last_stats()
    assert st["primary_rays"] == w * h * spp == int(port.rays[0])
    assert abs(st["bounce_rays"] - int(port.rays[1])) <= 0.01 * port.rays[1] + 10
    assert abs(st["shadow_rays"] - int(port.rays[2])) <= 0.01 * port.rays[2] + 10


@pytest.mark.parametrize("name", ["cornell", "cornell_lit", "mixed", "instanced"])
def test_render_matches_reference_statistically(cuda_lib, name):
    """Against two renders of the reference's own PathTracer. "instanced" is the large
    workload's scene itself (2,049,210 triangles in 205 meshes under a clustered hierarchy,
    deep traversal stacks, the cube-map sky with the sun disc) at 160x90, 64 spp, depth 8."""
    g = load_golden("renders.npz")
    w, h, spp, depth = (int(x) for x in g[f"{name}_cfg"])
    sc = _scene(name)
    img = np.zeros((h, w, 3), np.float32)
    cuda_lib.PathTracer(sc).render(dict(sc.camera, ratio=w / h), spp, depth, img, seed=7)
    assert_same_distribution(img, g[f"{name}_a"], g[f"{name}_b"])


def _flat_scene(emissive_color=None, bg=(0.25, 0.5, 0.75)):
    from rendu_gb300 import scenes as S

    sc = S.Scene()
    if emissive_color is not None:
        m = sc.add_mesh(S.quad_mesh((-50, -50, -1), (100, 0, 0), (0, 100, 0)))
        sc.add_object(m, sc.add_material(emissive_color, emissive=True))
    else:  # geometry behind the camera only
        m = sc.add_mesh(S.quad_mesh((-1, -1, 5), (2, 0, 0), (0, 2, 0)))
        sc.add_object(m, sc.add_material((0.5, 0.5, 0.5)))
    sc.background = {"mode": 0, "color": bg, "tex": (0,) * 6}
    sc.camera = {"eye": (0, 0, 1), "center": (0, 0, 0), "up": (0, 1, 0), "fov": 1.0, "ratio": 1.0}
    return sc


def test_exact_background_and_emitter_views(cuda_lib):
    img = np.zeros((8, 8, 3), np.float32)
    cuda_lib.PathTracer(_flat_scene()).render(_flat_scene().camera, 4, 3, img)
    assert np.all(img == np.array([0.25, 0.5, 0.75], np.float32))
    img = np.zeros((8, 8, 3), np.float32)
    sc = _flat_scene(emissive_color=(2.0, 7.0, 0.5))
    cuda_lib.PathTracer(sc).render(sc.camera, 4, 3, img)
    # Emission seen directly, each sample clamped at 5 (PathTracer.cpp:288).
    assert np.all(img == np.array([2.0, 5.0, 0.5], np.float32))


def test_accumulate_normalise_rounding_and_depth(cuda_lib):
    sc = _flat_scene()
    tr = cuda_lib.PathTracer(sc)
    # The image is accumulated into, then the whole is divided by spp.
    img = np.full((4, 4, 3), 2.0, np.float32)
    tr.render(sc.camera, 4, 2, img)
    np.testing.assert_allclose(img, np.broadcast_to((2.0 + 4 * np.array([0.25, 0.5, 0.75])) / 4, img.shape), rtol=1e-6)
    # Sample counts round to the nearest power of two in log2 (PathTracer.cpp:169-173).
    for samples, spp in [(3, 4), (5, 4), (6, 8), (1, 1), (12, 16)]:
        img = np.zeros((2, 2, 3), np.float32)
        tr.render(sc.camera, samples, 2, img)
        assert tr.last_stats()["primary_rays"] == 4 * spp
    # depth 0: no ray is cast, the image is only normalised.
    img = np.full((2, 2, 3), 8.0, np.float32)
    tr.render(sc.camera, 4, 0, img)
    assert np.all(img == 2.0) and tr.last_stats()["rays"] == 0


def test_four_component_and_device_images(cuda_lib):
    import torch

    sc = _scene("cornell")
    tr = cuda_lib.PathTracer(sc)
    host = np.zeros((12, 16, 3), np.float32)
    tr.render(dict(sc.camera, ratio=16 / 12), 4, 3, host, seed=3)
    four = np.zeros((12, 16, 4), np.float32)
    four[..., 3] = 0.125
    tr.render(dict(sc.camera, ratio=16 / 12), 4, 3, four, seed=3)
    assert np.array_equal(four[..., :3], host) and np.all(four[..., 3] == 0.125)
    dev = torch.zeros((12, 16, 3), dtype=torch.float32, device="cuda")
    tr.render(dict(sc.camera, ratio=16 / 12), 4, 3, dev, seed=3)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)


def test_argument_errors(cuda_lib):
    sc = _scene("cornell")
    tr = cuda_lib.PathTracer(sc)
    with pytest.raises(cuda_lib.RenduError):
        tr.render(sc.camera, 0, 3, np.zeros((2, 2, 3), np.float32))
    with pytest.raises(cuda_lib.RenduError):
        tr.render(sc.camera, 4, 3, np.zeros((2, 2, 2), np.float32))


def _ext_scene(name):
    from rendu_gb300 import scenes as S

    if name == "open_env":
        return S.constant_environment(S.open_cornell_scene(20261203), (0.8, 0.9, 1.0))
    if name == "instanced_small":
        return S.instanced_scene(20261206, instances=24, subdivisions=3)
    return _scene(name)


@pytest.mark.parametrize("name,spp,depth", [("cornell_lit", 8, 5), ("open_env", 8, 5), ("instanced_small", 4, 6),
                                            ("instanced", 2, 8)])
def test_extended_render_matches_port_on_the_same_random_stream(cuda_lib, port_lib, name, spp, depth):
    sc = _ext_scene(name)
    w, h = 64, 48
    cam = dict(sc.camera, ratio=w / h)
    gpu = cuda_lib.PathTracer(sc)
    img = np.zeros((h, w, 3), np.float32)
    gpu.render(cam, spp, depth, img, seed=5, mode=1, clamp=0.0)
    ref = port_lib.PortPathTracer(sc).render(cam, spp, depth, w, h, seed=5, mode=1, clamp=0.0)
    rel = np.abs(img - ref) / (np.abs(ref) + 1e-2)
    assert np.isfinite(img).all()
    assert np.mean(rel < 1e-3) > 0.95, f"only {np.mean(rel < 1e-3):.3f} of values agree to 1e-3"


def test_extended_estimator_converges_to_reference_estimator(cuda_lib):
    sc = _ext_scene("open_env")
    tr = cuda_lib.PathTracer(sc)
    imgs = []
    for seed, mode in ((1, 0), (2, 0), (3, 1)):
        img = np.zeros((32, 32, 3), np.float32)
        tr.render(sc.camera, 1024, 5, img, seed=seed, mode=mode, clamp=0.0)
        imgs.append(img)
    assert_same_distribution(imgs[2], imgs[0], imgs[1], factor=1.3)


def test_optional_buffers_survive_graph_reuse(cuda_lib):
    """The wave engine replays one captured graph across calls. A render with feature
    buffers after a call that re-captured it without them (the first double-precision
    accumulation allocates and forces a new capture), and a double-precision render after
    a capture made without one, both still get their buffers."""
    from rendu_gb300 import scenes as S

    sc = S.cornell_scene(3)
    tr = cuda_lib.PathTracer(sc)
    img = np.zeros((24, 24, 3), np.float32)
    aov = np.zeros((24, 24, 8), np.float32)
    tr.render(sc.camera, 2, 3, img, seed=1, aov=aov)
    ref_img, ref_aov = img.copy(), aov.copy()
    img64 = np.zeros_like(img)
    tr.render(sc.camera, 2, 3, img64, seed=1, fp64=True)
    np.testing.assert_allclose(img64, ref_img, rtol=1e-6, atol=1e-7)
    img[:] = 0
    aov2 = np.zeros_like(aov)
    tr.render(sc.camera, 2, 3, img, seed=1, aov=aov2)
    np.testing.assert_array_equal(aov2, ref_aov)
    np.testing.assert_array_equal(img, ref_img)
    # A different depth re-captures during a render without either option ...
    tmp = np.zeros_like(img)
    tr.render(sc.camera, 2, 4, tmp, seed=1)
    # ... and both options still work at that depth afterwards.
    a = np.zeros_like(img)
    tr.render(sc.camera, 2, 4, a, seed=1, fp64=True)
    np.testing.assert_allclose(a, tmp, rtol=1e-6, atol=1e-7)
    aov3 = np.zeros_like(aov)
    b = np.zeros_like(img)
    tr.render(sc.camera, 2, 4, b, seed=1, aov=aov3)
    np.testing.assert_array_equal(aov3, ref_aov)


def test_feature_buffers_and_fp64_accumulation(cuda_lib):
    """First-hit features: a camera-facing quad of one linear albedo gives that albedo, the
    normal facing the camera and the hit distance at every pixel; double-precision
    accumulation gives the same image up to float rounding."""
    from rendu_gb300 import scenes as S

    sc = S.Scene()
    m = sc.add_mesh(S.quad_mesh((-50, -50, -2), (100, 0, 0), (0, 100, 0)))
    sc.add_object(m, sc.add_material((0.5, 0.25, 0.75), rough=1.0))
    sc.lights.append({"type": 1, "color": (1.0, 1.0, 1.0), "direction": (0.0, 0.0, -1.0), "shadows": False})
    sc.camera = {"eye": (0, 0, 1), "center": (0, 0, 0), "up": (0, 1, 0), "fov": 1.0, "ratio": 1.0}
    tr = cuda_lib.PathTracer(sc)
    img = np.zeros((16, 16, 3), np.float32)
    aov = np.zeros((16, 16, 8), np.float32)
    tr.render(sc.camera, 4, 2, img, seed=1, aov=aov)
    np.testing.assert_allclose(aov[..., 0:3], np.broadcast_to(np.float32([0.5, 0.25, 0.75]) ** np.float32(2.2),
                                                              (16, 16, 3)), rtol=1e-5)
    np.testing.assert_allclose(aov[..., 3:6], np.broadcast_to(np.float32([0, 0, 1]), (16, 16, 3)), atol=1e-5)
    # Distance: 3 along the axis, 3 |d| / |d.z| off-axis for the pixel-centre direction d
    # (the per-sample jitter moves it by well under 3% inside a pixel at this resolution).
    t = np.tan(0.5) * ((np.arange(16) + 0.5) / 16 * 2 - 1)
    dist = 3.0 * np.sqrt(1.0 + t[None, :] ** 2 + t[:, None] ** 2)
    np.testing.assert_allclose(aov[..., 6], dist, rtol=3e-2)
    # Every sample of a pixel carries the same radiance here: no spread, a zero standard error
    lum = img @ np.float32([0.2126, 0.7152, 0.0722])
    assert (aov[..., 7] <= 1e-3 * lum + 1e-7).all()
    img64 = np.zeros_like(img)
    tr.render(sc.camera, 4, 2, img64, seed=1, fp64=True)
    np.testing.assert_allclose(img64, img, rtol=1e-6, atol=1e-7)


def test_standard_error_channel_matches_the_spread_of_independent_renders(cuda_lib):
    """The feature buffer's standard error of the mean luminance against the spread of two
    independent renders a and b: E[(L_a - L_b)^2] = Var(L_a) + Var(L_b). The channel is the
    spread of the samples as if they were independent, sqrt((E[L^2] - E[L]^2) / n); with
    n / (n - 1) it is unbiased for independent samples, and the stratified sub-pixel positions
    (PathTracer.cpp:57-84) make the true variance of a pixel's mean somewhat smaller, so it
    is a close upper estimate."""
    from rendu_gb300 import scenes as S

    sc = S.cornell_scene(20261203, True)
    tr = cuda_lib.PathTracer(sc)
    w = np.float32([0.2126, 0.7152, 0.0722])
    out = []
    for seed in (1, 2):
        img = np.zeros((96, 96, 3), np.float32)
        aov = np.zeros((96, 96, 8), np.float32)
        tr.render(sc.camera, 16, 4, img, seed=seed, aov=aov)
        out.append((img @ w, aov[..., 7]))
    (la, sa), (lb, sb) = out
    spread = np.mean((la.astype(np.float64) - lb) ** 2)
    predicted = np.mean(sa.astype(np.float64) ** 2 + sb.astype(np.float64) ** 2) * 16 / 15
    assert predicted > 0 and 0.7 < spread / predicted < 1.05, (spread, predicted)


def test_sky_table_and_eval_match_port_and_reference(cuda_lib, port_lib):
    """ATMOSPHERE (MaterialSky): the device table equals the C restatement's (and so the
    reference's stored table) up to expf's last bit around half-precision ties; the device
    sky matches the reference's MaterialSky::eval within float ulps."""
    from rendu_gb300 import pathtracer as P

    g = load_golden("sky.npz")
    t = P.sky_table()
    tp = port_lib.port_sky_table(512, 256)
    assert (t == tp).mean() > 0.999
    np.testing.assert_allclose(t, tp, rtol=2 ** -10, atol=2 ** -24)
    out = P.sky_eval(g["cases"])
    np.testing.assert_allclose(out, port_lib.port_sky_eval(tp, g["cases"]), rtol=2e-4, atol=1e-6)
    np.testing.assert_allclose(out, g["eval_out"], rtol=2e-3, atol=1e-6)
    # a caller-supplied table is used as given
    flat = np.full((4, 8, 4), 0.5, np.float32)
    np.testing.assert_allclose(P.sky_eval(g["cases"][:64], table=flat),
                               port_lib.port_sky_eval(flat, g["cases"][:64]), rtol=2e-4, atol=1e-6)


@pytest.mark.parametrize("spp,depth", [(8, 4)])
def test_atmosphere_render_matches_port_on_the_same_random_stream(cuda_lib, port_lib, spp, depth):
    from rendu_gb300 import scenes as S

    sc = S.atmosphere(S.open_cornell_scene(20261203), sun=(0.4, 0.7, 0.5))
    w, h = 64, 48
    cam = dict(sc.camera, ratio=w / h)
    img = np.zeros((h, w, 3), np.float32)
    cuda_lib.PathTracer(sc).render(cam, spp, depth, img, seed=7)
    ref = port_lib.PortPathTracer(sc).render(cam, spp, depth, w, h, seed=7)
    rel = np.abs(img - ref) / (np.abs(ref) + 1e-2)
    assert np.isfinite(img).all() and img.max() > 0
    assert np.mean(rel < 1e-3) > 0.97, f"only {np.mean(rel < 1e-3):.3f} of values agree to 1e-3"
