"""The denoiser's sm_103a kernels against the CPU restatement (oracle/denoiser.py): every
convolution tile configuration forward and backward (BF16 operands, FP32 accumulation),
the whole U-Net's loss and gradients, Adam, and inference with padding, through the C-ABI."""
import numpy as np
import pytest

from oracle import denoiser as OD

pytestmark = pytest.mark.gpu


def _bf16(a):
    """numpy values -> CUDA bfloat16 tensor holding their round-to-nearest-even rounding."""
    import torch

    bits = OD.bf16_bits(a).view(np.int16)
    return torch.from_numpy(np.ascontiguousarray(bits)).view(torch.bfloat16).cuda()


def _f32(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _np(t):
    import torch

    torch.cuda.synchronize()
    return t.float().cpu().numpy()


# (c0, up0, c1, cout): every layer shape of the U-Net, the dgrad shapes (cout = a layer's
# input channels: 80, 112, 160, 224), and small / masked tiles.
CONV_CASES = [(16, 0, 0, 32), (32, 0, 0, 32), (32, 0, 0, 48), (48, 0, 0, 48), (48, 0, 0, 64), (64, 0, 0, 96),
              (96, 0, 0, 128), (128, 0, 0, 128), (128, 1, 96, 96), (96, 1, 64, 64), (64, 1, 48, 48), (48, 1, 32, 32),
              (32, 0, 0, 16), (32, 0, 0, 80), (64, 0, 0, 112), (64, 0, 0, 160), (96, 0, 0, 224), (8, 0, 8, 8)]


# Image sizes: 22 pixels wide (tiles of 32 x 4 pixels), 150 wide (row tiles, the second one
# partly outside the image) and 400 wide (row tiles inside the row as well as at its ends).
SIZES = [(18, 22), (6, 150), (4, 400)]


def _case(rng, c0, up0, c1, cout, b=2, h=18, w=22):
    x0 = OD.bf16_round(rng.normal(size=(b, h >> up0, w >> up0, c0)))
    x1 = OD.bf16_round(rng.normal(size=(b, h, w, c1))) if c1 else None
    x = OD.upsample2(x0) if up0 else x0
    if c1:
        x = np.concatenate([x, x1], -1)
    return x0, x1, x


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("c0,up0,c1,cout", CONV_CASES)
def test_conv_forward_matches_oracle(cuda_lib, c0, up0, c1, cout, h, w):
    from rendu_gb300 import denoiser as D

    rng = np.random.default_rng(c0 * 1000 + cout + up0 + w)
    x0, x1, x = _case(rng, c0, up0, c1, cout, h=h, w=w)
    w = OD.bf16_round(rng.normal(size=(9, c0 + c1, cout)) * 0.1)
    bias = rng.normal(size=cout).astype(np.float32)
    ref = OD.conv3x3(x, w, bias)
    bound = OD.conv3x3(np.abs(x), np.abs(w)) + np.abs(bias)
    out = _np(D.conv3x3(_bf16(x0), _bf16(w), cout, x1=_bf16(x1) if c1 else None, up0=bool(up0), bias=_f32(bias)))
    # FP32 accumulation of exact BF16 products: error well below 1e-5 of the sum of |terms|.
    assert np.all(np.abs(out - ref) <= 1e-5 * bound + 1e-7), np.abs(out - ref).max()
    # Fused ReLU + BF16 store: within one BF16 rounding of the exact value.
    outb = _np(D.conv3x3(_bf16(x0), _bf16(w), cout, x1=_bf16(x1) if c1 else None, up0=bool(up0), bias=_f32(bias),
                         relu=True, out_fp32=False))
    r = np.maximum(ref, 0.0)
    assert np.all(np.abs(outb - r) <= 2 ** -8 * np.abs(r) + 1e-5 * bound + 1e-7)


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("c0,up0,c1,cout", CONV_CASES)
def test_conv_backward_matches_oracle(cuda_lib, c0, up0, c1, cout, h, w):
    from rendu_gb300 import denoiser as D

    rng = np.random.default_rng(7 + c0 * 1000 + cout + up0 + w)
    x0, x1, x = _case(rng, c0, up0, c1, cout, h=h, w=w)
    wf = (rng.normal(size=(9, c0 + c1, cout)) * 0.1).astype(np.float32)
    gy = OD.bf16_round(rng.normal(size=x.shape[:3] + (cout,)))
    dx, dw = D.conv3x3_backward(_bf16(x0), _f32(wf), _bf16(gy), x1=_bf16(x1) if c1 else None, up0=bool(up0))
    wb = OD.bf16_round(wf)
    ref_dx = OD.conv3x3_dgrad(gy, wb)
    bound_dx = OD.conv3x3_dgrad(np.abs(gy), np.abs(wb))
    assert np.all(np.abs(_np(dx) - ref_dx) <= 1e-5 * bound_dx + 1e-7)
    ref_dw = OD.conv3x3_wgrad(x, gy)
    bound_dw = OD.conv3x3_wgrad(np.abs(x), np.abs(gy))
    assert np.all(np.abs(_np(dw) - ref_dw) <= 1e-5 * bound_dw + 1e-7)


@pytest.mark.parametrize("b,h,w", [(3, 10, 6), (1, 2, 2), (2, 64, 96)])
def test_conv_odd_shapes(cuda_lib, b, h, w):
    """Images narrower than a pipeline stage (the weight-gradient gather wraps rows many
    times per stage) and larger ones spanning many pixel chunks."""
    from rendu_gb300 import denoiser as D

    rng = np.random.default_rng(b * 100 + h + w)
    c0, cout = 48, 64
    x0 = OD.bf16_round(rng.normal(size=(b, h, w, c0)))
    wf = (rng.normal(size=(9, c0, cout)) * 0.1).astype(np.float32)
    gy = OD.bf16_round(rng.normal(size=(b, h, w, cout)))
    out = _np(D.conv3x3(_bf16(x0), _bf16(wf), cout))
    ref = OD.conv3x3(x0, OD.bf16_round(wf))
    assert np.all(np.abs(out - ref) <= 1e-5 * OD.conv3x3(np.abs(x0), np.abs(OD.bf16_round(wf))) + 1e-7)
    dx, dw = D.conv3x3_backward(_bf16(x0), _f32(wf), _bf16(gy))
    ref_dw = OD.conv3x3_wgrad(x0, gy)
    assert np.all(np.abs(_np(dw) - ref_dw) <= 1e-5 * OD.conv3x3_wgrad(np.abs(x0), np.abs(gy)) + 1e-7)
    ref_dx = OD.conv3x3_dgrad(gy, OD.bf16_round(wf))
    assert np.all(np.abs(_np(dx) - ref_dx) <= 1e-5 * OD.conv3x3_dgrad(np.abs(gy), np.abs(OD.bf16_round(wf))) + 1e-7)


def _features(rng, b, h, w):
    n = rng.normal(size=(b, h, w, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.concatenate([rng.exponential(0.5, (b, h, w, 3)), rng.uniform(0, 1, (b, h, w, 3)), n,
                           rng.uniform(0, 6, (b, h, w, 1)), rng.exponential(0.05, (b, h, w, 1))], -1).astype(np.float32)


def test_network_structure_matches_oracle(cuda_lib):
    from rendu_gb300.denoiser import Denoiser

    d = Denoiser()
    net = OD.UNet()
    assert d.layers() == net.layers
    assert d.param_count == net.param_count


def test_network_gradients_match_oracle(cuda_lib):
    from rendu_gb300.denoiser import Denoiser

    rng = np.random.default_rng(11)
    d = Denoiser(seed=5)
    params = d.get_params()
    feats = _features(rng, 2, 64, 80)
    # Radiance away from zero (the loss divides by output + 0.01, so near-black outputs would
    # weigh the comparison towards a few pixels' BF16 rounding) and targets away from the
    # near-identity output, so that the gradient is large against that rounding.
    feats[..., :3] += 0.5
    x_log = np.log1p(feats[..., :3].astype(np.float64))
    target = np.expm1(x_log + np.array([0.5, -0.3, 0.5])).astype(np.float32)
    loss = d.backward(feats, target)
    grads = d.get_grads()
    net = OD.UNet()
    ref_loss, ref = net.backward(params, feats, target)
    # The relative squared error divides by (output + 0.01): outputs near zero magnify the
    # BF16 rounding of the activations more than the old log-space loss did.
    assert abs(loss - ref_loss) <= 3e-3 * ref_loss
    errs = []
    for k, l in enumerate(net.layers):
        cin = l["cin0"] + l["cin1"]
        for off, n in ((l["weight_offset"], 9 * cin * l["cout"]), (l["bias_offset"], l["cout"])):
            g, r = grads[off:off + n], ref[off:off + n]
            errs.append((k, off == l["bias_offset"], np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)))
    # BF16 activations and output gradients: the two sides round a few values to adjacent
    # BF16 numbers, which the chain of 19 layers spreads into a small relative difference,
    # largest at the coarsest level (fewest pixels to average it out).
    worst = sorted(errs, key=lambda e: -e[2])[:6]
    assert worst[0][2] < 3e-2 and np.median([e for _, _, e in errs]) < 1e-2, worst


def test_adam_matches_oracle(cuda_lib):
    from rendu_gb300.denoiser import Denoiser

    rng = np.random.default_rng(12)
    d = Denoiser(seed=6)
    feats = _features(rng, 1, 32, 32)
    target = rng.exponential(0.5, (1, 32, 32, 3)).astype(np.float32)
    p = d.get_params().astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for step, lr in ((1, 1e-3), (2, 5e-4)):
        d.backward(feats, target)
        g = d.get_grads().astype(np.float64)
        d.adam_step(lr)
        p, m, v = OD.adam(p, g, m, v, step, lr)
        np.testing.assert_allclose(d.get_params(), p, rtol=0, atol=2e-6)


def test_denoise_pads_and_matches_oracle(cuda_lib):
    """An image whose sides are not multiples of 16 is edge-padded, denoised and cropped;
    host and device pointers give identical results."""
    import torch

    from rendu_gb300.denoiser import Denoiser

    rng = np.random.default_rng(13)
    d = Denoiser(seed=7)
    feats = _features(rng, 2, 37, 45)
    out = d.denoise(feats)
    assert out.shape == (2, 37, 45, 3)
    net = OD.UNet()
    acts, y = net.forward(d.get_params(), OD.pad16(feats))
    ref = OD.output(OD.pad16(feats), y)[:, :37, :45]
    diff = np.abs(np.log1p(out) - np.log1p(ref))
    assert diff.max() < 0.05 and diff.mean() < 2e-3, (diff.max(), diff.mean())
    dev = d.denoise(torch.from_numpy(feats).cuda())
    np.testing.assert_array_equal(_np(dev), out)


def test_training_step_is_deterministic_and_lowers_loss(cuda_lib):
    from rendu_gb300.denoiser import Denoiser

    rng = np.random.default_rng(14)
    feats = _features(rng, 4, 32, 32)
    target = np.ascontiguousarray(feats[..., :3] * 0.5)
    runs = []
    for _ in range(2):
        d = Denoiser(seed=8)
        losses = [d.train_step(feats, target, 2e-3) for _ in range(120)]
        runs.append((losses, d.get_params()))
    assert runs[0][0] == runs[1][0]
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    assert runs[0][0][-1] < 0.75 * runs[0][0][0], runs[0][0][::20]


def test_invalid_arguments_are_rejected(cuda_lib):
    from rendu_gb300 import RenduError
    from rendu_gb300.denoiser import Denoiser

    d = Denoiser()
    f = np.zeros((1, 20, 32, 11), np.float32)
    t = np.zeros((1, 20, 32, 3), np.float32)
    with pytest.raises(RenduError, match="multiples of 16"):
        d.train_step(f, t, 1e-3)
    with pytest.raises(RenduError, match="parameter count"):
        d.set_params(np.zeros(3, np.float32))
    with pytest.raises(RenduError, match="learning rate"):
        d.adam_step(float("nan"))


def test_captured_steps_match_eager(cuda_lib):
    """dn_train_step and dn_denoise run eagerly on a new shape, capture a CUDA graph on the
    next call and replay it after: every call gives what the eager dn_backward +
    dn_adam_step sequence gives, bit for bit."""
    from rendu_gb300.denoiser import Denoiser

    rng = np.random.default_rng(15)
    feats = _features(rng, 2, 48, 32)
    target = rng.exponential(0.5, (2, 48, 32, 3)).astype(np.float32)
    a, b = Denoiser(seed=9), Denoiser(seed=9)
    for lr in (1e-3, 1e-3, 5e-4, 5e-4, 5e-4):
        la = a.train_step(feats, target, lr)
        lb = b.backward(feats, target)
        b.adam_step(lr)
        assert la == lb
    np.testing.assert_array_equal(a.get_params(), b.get_params())
    f2 = _features(rng, 1, 40, 56)
    outs = [a.denoise(f2) for _ in range(4)]
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
