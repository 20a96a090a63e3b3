"""The denoiser's CPU restatement (oracle/denoiser.py) against PyTorch autograd in float64:
the convolution and its two gradients, the pooling / upsampling adjoints, and the whole
U-Net's loss gradient. The reference has no learned denoiser; these checks pin the oracle
that the GPU tests then hold the sm_103a kernels to."""
import numpy as np
import pytest

from oracle import denoiser as OD

torch = pytest.importorskip("torch")
F = torch.nn.functional


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64))


def _torch_weight(w):
    """[tap][cin][cout] -> conv2d's (cout, cin, 3, 3), tap = 3 ky + kx."""
    w = np.asarray(w, np.float64)
    return _t(w.reshape(3, 3, w.shape[1], w.shape[2]).transpose(3, 2, 0, 1))


def _nchw(x):
    return _t(x).permute(0, 3, 1, 2)


def test_conv_and_gradients_match_autograd():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 7, 9, 5))
    w = rng.normal(size=(9, 5, 6))
    b = rng.normal(size=6)
    g = rng.normal(size=(2, 7, 9, 6))
    xt = _nchw(x).requires_grad_(True)
    wt = _torch_weight(w).requires_grad_(True)
    yt = F.conv2d(xt, wt, _t(b), padding=1)
    np.testing.assert_allclose(OD.conv3x3(x, w, b), yt.permute(0, 2, 3, 1).detach().numpy(), rtol=1e-12, atol=1e-12)
    yt.backward(_nchw(g))
    np.testing.assert_allclose(OD.conv3x3_dgrad(g, w), xt.grad.permute(0, 2, 3, 1).numpy(), rtol=1e-12, atol=1e-11)
    dw = wt.grad.numpy().transpose(2, 3, 1, 0).reshape(9, 5, 6)
    np.testing.assert_allclose(OD.conv3x3_wgrad(x, g), dw, rtol=1e-12, atol=1e-11)


def test_pool_and_upsample_adjoints():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 8, 6, 3))
    g = rng.normal(size=(2, 16, 12, 3))
    # <up(x), g> = <x, up^T(g)>
    assert np.isclose((OD.upsample2(x) * g).sum(), (x * OD.upsample2_adjoint(g)).sum())
    # pooling gradient = autograd's (no ties with continuous values)
    xt = _nchw(x).requires_grad_(True)
    yt = F.max_pool2d(xt, 2)
    gy = rng.normal(size=(2, 4, 3, 3))
    yt.backward(_nchw(gy))
    y = OD.pool2(x)
    np.testing.assert_array_equal(y, yt.permute(0, 2, 3, 1).detach().numpy())
    np.testing.assert_allclose(OD.pool2_back(x, y, gy), xt.grad.permute(0, 2, 3, 1).numpy())
    # ties go to the first maximal input of the window (row-major)
    z = np.zeros((1, 2, 2, 1))
    gz = OD.pool2_back(z, OD.pool2(z), np.ones((1, 1, 1, 1)))
    assert gz[0, 0, 0, 0] == 1 and gz.sum() == 1


def _torch_unet(net, params, x_in):
    acts = {0: _nchw(x_in)}
    ws = []
    for op in net.ops:
        if op[0] == "pool":
            acts[op[2]] = F.max_pool2d(acts[op[1]], 2)
            continue
        _, k, s0, s1, out = op
        l = net.layers[k]
        w, b = net.weights(params, k)
        wt = _torch_weight(w).requires_grad_(True)
        bt = _t(b).requires_grad_(True)
        ws.append((wt, bt))
        a = F.interpolate(acts[s0], scale_factor=2, mode="nearest") if l["up0"] else acts[s0]
        if s1 is not None:
            a = torch.cat([a, acts[s1]], dim=1)
        z = F.conv2d(a, wt, bt, padding=1)
        acts[out] = F.relu(z) if l["relu"] else z
    return acts[net.ops[-1][4]], ws


def test_unet_backward_matches_autograd():
    """Without bfloat16 rounding the oracle's hand-written backward equals autograd."""
    rng = np.random.default_rng(3)
    net = OD.UNet()
    params = np.zeros(net.param_count, np.float32)
    for k, l in enumerate(net.layers):
        cin = l["cin0"] + l["cin1"]
        params[l["weight_offset"]:l["weight_offset"] + 9 * cin * l["cout"]] = \
            rng.normal(0, np.sqrt(2 / (9 * cin)), 9 * cin * l["cout"])
        params[l["bias_offset"]:l["bias_offset"] + l["cout"]] = rng.normal(0, 0.05, l["cout"])
    feats = np.concatenate([rng.exponential(0.5, (2, 32, 32, 3)), rng.uniform(0, 1, (2, 32, 32, 3)),
                            rng.normal(size=(2, 32, 32, 3)), rng.uniform(0, 4, (2, 32, 32, 1)),
                            rng.exponential(0.05, (2, 32, 32, 1))], -1).astype(np.float32)
    target = rng.exponential(0.5, (2, 32, 32, 3)).astype(np.float32)
    loss, grads = net.backward(params, feats, target, bf16=False)

    x_in = OD.prepare(feats).astype(np.float64)
    y, ws = _torch_unet(net, params, x_in)
    # output = max(exp(log(1 + radiance) + y) - 1, 0) from the float32 radiance; relative
    # squared error with the denominator held constant
    pred = torch.clamp(torch.expm1(torch.log1p(_nchw(feats[..., :3]).clamp(min=0.0)) + y[:, :3]), min=0.0)
    lt = (((pred - _nchw(target)) / (pred.detach() + 0.01)) ** 2).mean()
    lt.backward()
    assert np.isclose(loss, lt.item(), rtol=1e-12)
    for k, (wt, bt) in enumerate(ws):
        l = net.layers[k]
        cin = l["cin0"] + l["cin1"]
        gw = wt.grad.numpy().transpose(2, 3, 1, 0).reshape(-1)
        np.testing.assert_allclose(grads[l["weight_offset"]:l["weight_offset"] + 9 * cin * l["cout"]], gw,
                                   rtol=1e-8, atol=1e-12)
        np.testing.assert_allclose(grads[l["bias_offset"]:l["bias_offset"] + l["cout"]], bt.grad.numpy(),
                                   rtol=1e-8, atol=1e-12)


def test_bf16_rounding_is_round_to_nearest_even():
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e38], np.float32)
    r = OD.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 and r[4] == -2.5
    assert np.isfinite(r[5])
    t = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(r, t)
