"""CPU restatement of the learned denoiser -- ORACLE, test infrastructure only.

The reference renderer has no learned denoiser (its only image filter is the real-time
bilateral blur, src/engine/processing/BilateralBlur.cpp:7-11), so there is nothing of the
reference to pin here: this module restates, in float64 numpy, the network the product
runs on the GPU (rendu_gb300/csrc/dn_api.cu, dn_kernels.cu) so that its kernels can be
checked operation by operation:

* ``conv3x3`` / ``conv3x3_dgrad`` / ``conv3x3_wgrad``: 3x3 convolution, zero padding,
  weights [tap][cin][cout] with tap = 3 (dy + 1) + (dx + 1);
* ``upsample2`` / ``upsample2_adjoint``, ``pool2`` / ``pool2_back`` (first maximal input
  of each window in row-major order);
* ``UNet``: the 5-level U-Net with its forward and backward passes, rounding activations
  and output gradients to bfloat16 exactly where the GPU stores them as bfloat16
  (``bf16=False`` turns the rounding off, for checks against autograd);
* ``adam``: one Adam step (Kingma & Ba 2015).

Only tests/, the smoke check and bench.py's CPU leg use it.
"""
from __future__ import annotations

import numpy as np

LEVEL_CHANNELS = (32, 48, 64, 96, 128)
IN_CHANNELS = 16
OUT_CHANNELS = 16
FEATURES = 11


def bf16_round(a) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def bf16_bits(a) -> np.ndarray:
    """bfloat16 bit patterns (uint16) of the rounded values."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def _taps(x):
    """(B, H, W, C) -> (B, H, W, 9, C): x[y + dy, x + dx] for tap = 3 (dy + 1) + (dx + 1),
    zero outside the image."""
    b, h, w, c = x.shape
    xp = np.zeros((b, h + 2, w + 2, c), x.dtype)
    xp[:, 1:-1, 1:-1] = x
    return np.stack([xp[:, 1 + dy:1 + dy + h, 1 + dx:1 + dx + w] for dy in (-1, 0, 1) for dx in (-1, 0, 1)], axis=3)


def conv3x3(x, w, bias=None):
    """x (B, H, W, Cin), w (9, Cin, Cout) -> (B, H, W, Cout) in float64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    b, h, wd, c = x.shape
    out = _taps(x).reshape(b * h * wd, 9 * c) @ w.reshape(9 * c, -1)
    if bias is not None:
        out = out + np.asarray(bias, np.float64)
    return out.reshape(b, h, wd, -1)


def conv3x3_dgrad(g, w):
    """Gradient with respect to the input: dx[p, ci] = sum_{tap, co} g[p - off(tap), co] w[tap][ci][co]
    = conv3x3(g, w flipped in space and transposed)."""
    w = np.asarray(w, np.float64)
    wt = np.ascontiguousarray(w[::-1].transpose(0, 2, 1))
    return conv3x3(g, wt)


def conv3x3_wgrad(x, g):
    """dw[tap][ci][co] = sum_p x[p + off(tap), ci] g[p, co]."""
    x = np.asarray(x, np.float64)
    g = np.asarray(g, np.float64)
    b, h, w, c = x.shape
    t = _taps(x).reshape(b * h * w, 9 * c)
    return (t.T @ g.reshape(b * h * w, -1)).reshape(9, c, -1)


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_adjoint(g):
    b, h, w, c = g.shape
    return g.reshape(b, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def pool2(x):
    b, h, w, c = x.shape
    return x.reshape(b, h // 2, 2, w // 2, 2, c).max(axis=(2, 4))


def pool2_back(x, y, gy):
    """Each pooled gradient goes to the first input of its 2x2 window (order (0,0), (0,1),
    (1,0), (1,1)) equal to the window's maximum."""
    b, h, w, c = x.shape
    win = x.reshape(b, h // 2, 2, w // 2, 2, c).transpose(0, 1, 3, 2, 4, 5).reshape(b, h // 2, w // 2, 4, c)
    first = np.argmax(win == y[:, :, :, None, :], axis=3)
    onehot = (np.arange(4)[None, None, None, :, None] == first[:, :, :, None, :]) * gy[:, :, :, None, :]
    return onehot.reshape(b, h // 2, w // 2, 2, 2, c).transpose(0, 1, 3, 2, 4, 5).reshape(b, h, w, c)


def prepare(features):
    """Features {radiance rgb, albedo rgb, normal xyz, distance, standard error} -> 16 input
    channels: log(1 + radiance), albedo, normal / 2 + 1/2, distance / (1 + distance),
    e / (1 + e) with the relative standard error e = se / (luminance + 0.01), log(1 + se),
    zeros."""
    f = np.asarray(features, np.float32)
    out = np.zeros(f.shape[:-1] + (IN_CHANNELS,), np.float32)
    out[..., 0:3] = np.log1p(np.maximum(f[..., 0:3], 0.0))
    out[..., 3:6] = f[..., 3:6]
    out[..., 6:9] = f[..., 6:9] * 0.5 + 0.5
    d = np.maximum(f[..., 9], 0.0)
    out[..., 9] = d / (1.0 + d)
    se = np.maximum(f[..., 10], 0.0)
    lum = np.maximum(0.2126 * f[..., 0] + 0.7152 * f[..., 1] + 0.0722 * f[..., 2], 0.0)
    e = se / (lum + 0.01)
    out[..., 10] = e / (1.0 + e)
    out[..., 11] = np.log1p(se)
    return out


def output(features, y):
    """Radiance max(exp(log(1 + input) + y) - 1, 0) from the float32 input radiance."""
    r = np.maximum(np.asarray(features, np.float64)[..., 0:3], 0.0)
    return np.maximum(np.expm1(np.log1p(r) + np.asarray(y, np.float64)[..., 0:3]), 0.0)


def pad16(features):
    """Edge-replicate (B, H, W, C) up to multiples of 16 in H and W."""
    b, h, w, c = features.shape
    hp, wp = -(-h // 16) * 16, -(-w // 16) * 16
    return np.pad(features, ((0, 0), (0, hp - h), (0, wp - w), (0, 0)), mode="edge")


class UNet:
    """The denoiser's layer graph: (cin0, cin1, cout, up0, relu, level) per convolution,
    and the flat parameter layout (weights [9][cin][cout] then bias [cout] per layer)."""

    def __init__(self):
        self.layers = []
        self.ops = []  # ("conv", layer index, src0, src1, out) | ("pool", src, out)
        self.tensors = []  # (level, channels)
        off = 0

        def tensor(level, ch):
            self.tensors.append((level, ch))
            return len(self.tensors) - 1

        def conv(s0, up0, s1, cout, relu):
            nonlocal off
            cin0 = self.tensors[s0][1]
            cin1 = self.tensors[s1][1] if s1 is not None else 0
            level = self.tensors[s0][0] - (1 if up0 else 0)
            out = tensor(level, cout)
            woff = off
            off += 9 * (cin0 + cin1) * cout
            boff = off
            off += cout
            self.layers.append(dict(cin0=cin0, cin1=cin1, cout=cout, up0=int(up0), relu=int(relu), level=level,
                                    weight_offset=woff, bias_offset=boff))
            self.ops.append(("conv", len(self.layers) - 1, s0, s1, out))
            return out

        def pool(s):
            out = tensor(self.tensors[s][0] + 1, self.tensors[s][1])
            self.ops.append(("pool", s, out))
            return out

        cur = tensor(0, IN_CHANNELS)
        skip = []
        for lvl, ch in enumerate(LEVEL_CHANNELS):
            if lvl:
                cur = pool(cur)
            cur = conv(cur, False, None, ch, True)
            cur = conv(cur, False, None, ch, True)
            skip.append(cur)
        for lvl in range(len(LEVEL_CHANNELS) - 2, -1, -1):
            cur = conv(cur, True, skip[lvl], LEVEL_CHANNELS[lvl], True)
            cur = conv(cur, False, None, LEVEL_CHANNELS[lvl], True)
        conv(cur, False, None, OUT_CHANNELS, False)
        self.param_count = off

    def weights(self, params, k):
        l = self.layers[k]
        cin = l["cin0"] + l["cin1"]
        w = params[l["weight_offset"]:l["weight_offset"] + 9 * cin * l["cout"]].reshape(9, cin, l["cout"])
        b = params[l["bias_offset"]:l["bias_offset"] + l["cout"]]
        return w, b

    def _input(self, acts, s0, s1, up0):
        a = upsample2(acts[s0]) if up0 else acts[s0]
        return a if s1 is None else np.concatenate([a, acts[s1]], axis=-1)

    def forward(self, params, features, bf16=True):
        """features (B, H, W, 11), H and W multiples of 16 -> (acts, output (B, H, W, 16)).
        Activations are rounded to bfloat16 where the GPU stores them so; the output stays
        float32 (FP32 on the GPU)."""
        rnd = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
        params = np.asarray(params, np.float32)
        acts = {0: rnd(prepare(features))}
        for op in self.ops:
            if op[0] == "pool":
                acts[op[2]] = pool2(acts[op[1]])
                continue
            _, k, s0, s1, out = op
            l = self.layers[k]
            w, b = self.weights(params, k)
            z = conv3x3(self._input(acts, s0, s1, l["up0"]), rnd(w), b)
            if l["relu"]:
                z = np.maximum(z, 0.0)
            last = k == len(self.layers) - 1
            acts[out] = (z.astype(np.float32) if bf16 else z) if last else rnd(z)
        return acts, acts[self.ops[-1][4]]

    @staticmethod
    def loss_and_grad(features, y, target):
        """Relative squared error mean(((x - t) / (x' + 0.01))^2) of the output
        x = output(features, y) against the target t, x' = x held constant in the gradient;
        returns (loss, dL/dy) with dL/dy = 2 (x - t) / (x' + 0.01)^2 (x + 1) where x > 0."""
        x = output(features, y)
        t = np.asarray(target, np.float64)
        den = x + 0.01
        q = (x - t) / den
        n = q.size
        g = np.zeros(y.shape, np.float64)
        g[..., :3] = np.where(x > 0.0, 2.0 * q / den * (x + 1.0), 0.0) / n
        return float((q * q).mean()), g

    def backward(self, params, features, target, bf16=True):
        """(loss, flat gradient) of one batch, following the GPU's order of operations."""
        rnd = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
        params = np.asarray(params, np.float32)
        acts, y = self.forward(params, features, bf16)
        loss, gy = self.loss_and_grad(features, y, target)
        grads = np.zeros(self.param_count, np.float64)
        g = {self.ops[-1][4]: gy}
        for op in reversed(self.ops):
            if op[0] == "pool":
                _, s, out = op
                g[s] = g[s] + pool2_back(acts[s], acts[out], g[out])
                continue
            _, k, s0, s1, out = op
            l = self.layers[k]
            go = g[out]
            if l["relu"]:
                go = np.where(acts[out] > 0, go, 0.0)
            gb = rnd(go)
            x = self._input(acts, s0, s1, l["up0"])
            cin = l["cin0"] + l["cin1"]
            grads[l["weight_offset"]:l["weight_offset"] + 9 * cin * l["cout"]] = conv3x3_wgrad(x, gb).reshape(-1)
            grads[l["bias_offset"]:l["bias_offset"] + l["cout"]] = go.reshape(-1, l["cout"]).sum(axis=0)
            if s0 == 0:
                continue
            w, _ = self.weights(params, k)
            gx = conv3x3_dgrad(gb, rnd(w))
            g0 = gx[..., :l["cin0"]]
            g[s0] = upsample2_adjoint(g0) if l["up0"] else g0
            if s1 is not None:
                g[s1] = gx[..., l["cin0"]:]
        return loss, grads


def adam(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns new (params, m, v)."""
    m = b1 * m + (1 - b1) * grads
    v = b2 * v + (1 - b2) * grads * grads
    p = params - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v

