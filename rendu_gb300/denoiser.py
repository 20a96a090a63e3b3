"""Learned denoiser over the C-ABI ``dn_*`` entry points.

A 5-level U-Net (3x3 convolutions with 32, 48, 64, 96 and 128 channels, BF16 activations,
FP32 accumulation on the tensor cores) that maps a few-sample render plus its first-hit
feature buffers (albedo, normal, distance, standard error: ``PathTracer.render(..., aov=...)``) to a
converged image. The reference has no learned denoiser; this module completes the
renderer with one that is trained here on the path tracer's own output.

Arrays are float32 NHWC: features (B, H, W, 11) = radiance rgb, albedo rgb, normal xyz,
distance, standard error of the mean luminance; images (B, H, W, 3). Host numpy arrays or CUDA tensors (all of one kind per call).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

FEATURES = L.DN_FEATURES
# Network input channels that carry data (of the 16 the first layer reads): log radiance,
# albedo, normal, distance, relative standard error, log standard error.
INPUT_CHANNELS = 12


def _is_cuda(a) -> bool:
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


def _ptr(a):
    if _is_cuda(a):
        import torch

        if not a.is_contiguous() or a.dtype != torch.float32:
            raise TypeError("CUDA tensors must be contiguous float32")
        return C.c_void_p(a.data_ptr())
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
        raise TypeError("arrays must be C-contiguous float32")
    return C.c_void_p(a.ctypes.data)


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _nhwc(a, channels):
    shape = tuple(a.shape)
    if len(shape) == 3:
        shape = (1,) + shape
    if len(shape) != 4 or shape[3] != channels:
        raise ValueError(f"expected (B, H, W, {channels}) or (H, W, {channels}), got {tuple(a.shape)}")
    return shape


def rel_rmse(x, ref, eps: float = 1e-2) -> float:
    """Relative RMSE, sqrt(mean(((x - ref) / (ref + eps))^2)), over every pixel and channel."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean(((x - ref) / (ref + eps)) ** 2)))


def features_from_render(image, aov) -> np.ndarray:
    """Stack a render (H, W, >=3) and its feature buffer (H, W, 8) into (H, W, 11)."""
    return np.ascontiguousarray(np.concatenate([np.asarray(image)[..., :3], np.asarray(aov)], axis=-1), np.float32)


class Denoiser:
    """The U-Net on one device. ``denoise`` runs inference; ``train_step`` one Adam step on
    a batch of (features, converged target) crops whose sides are multiples of 16."""

    def __init__(self, device: int = 0, seed: int | None = None):
        h = C.c_void_p()
        L.call("dn_create", C.byref(h), int(device))
        self._h = h
        self.device = device
        if seed is not None:
            L.call("dn_init", self._h, int(seed))

    # ---- structure and parameters ------------------------------------------------------------
    def layers(self) -> list[dict]:
        n = C.c_uint32()
        L.call("dn_layer_count", self._h, C.byref(n))
        out = []
        for i in range(n.value):
            d = L.dn_layer()
            L.call("dn_layer_info", self._h, i, C.byref(d))
            out.append({k: getattr(d, k) for k, _ in d._fields_})
        return out

    @property
    def param_count(self) -> int:
        n = C.c_size_t()
        L.call("dn_param_count", self._h, C.byref(n))
        return n.value

    def get_params(self) -> np.ndarray:
        out = np.empty(self.param_count, np.float32)
        L.call("dn_get_params", self._h, out.ctypes.data, out.size)
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, np.float32).reshape(-1)
        L.call("dn_set_params", self._h, p.ctypes.data, p.size)

    def get_grads(self) -> np.ndarray:
        out = np.empty(self.param_count, np.float32)
        L.call("dn_get_grads", self._h, out.ctypes.data, out.size)
        return out

    def read_grads(self, out) -> None:
        """Copy the last gradients into ``out`` (param_count float32: a CUDA tensor, ordered on
        the current stream, or a host array)."""
        dev = _is_cuda(out)
        L.call("dn_read_grads", self._h, _ptr(out), self.param_count, _stream() if dev else None,
               L.RT_FLAG_DEVICE_PTRS if dev else 0)

    def write_grads(self, src) -> None:
        """Replace the gradients that the next ``adam_step`` applies with ``src``."""
        dev = _is_cuda(src)
        L.call("dn_write_grads", self._h, _ptr(src), self.param_count, _stream() if dev else None,
               L.RT_FLAG_DEVICE_PTRS if dev else 0)

    def init(self, seed: int) -> None:
        L.call("dn_init", self._h, int(seed))

    def save(self, path: str) -> None:
        np.save(path, self.get_params())

    def load(self, path: str) -> None:
        self.set_params(np.load(path))

    def flops(self, height: int, width: int, batch: int = 1, channels=None) -> float:
        """Multiply-add FLOPs of one forward pass (2 x MACs of every convolution) at the
        padded size the network runs at. ``channels`` = (first layer's inputs, last layer's
        outputs) counts only the channels that carry data (INPUT_CHANNELS and 3) instead of
        the 16 each is padded to."""
        hp, wp = -(-height // 16) * 16, -(-width // 16) * 16
        layers = self.layers()
        total = 0.0
        for k, l in enumerate(layers):
            px = batch * (hp >> l["level"]) * (wp >> l["level"])
            cin, cout = l["cin0"] + l["cin1"], l["cout"]
            if channels is not None and k == 0:
                cin = channels[0]
            if channels is not None and k == len(layers) - 1:
                cout = channels[1]
            total += 2.0 * px * 9 * cin * cout
        return total

    # ---- compute -----------------------------------------------------------------------------
    def denoise(self, features, out=None):
        """features (B, H, W, 11) or (H, W, 11) -> radiance of the same leading shape x 3."""
        b, h, w, _ = _nhwc(features, FEATURES)
        dev = _is_cuda(features)
        if out is None:
            if dev:
                import torch

                out = torch.empty(tuple(features.shape[:-1]) + (3,), dtype=torch.float32, device=features.device)
            else:
                out = np.empty(tuple(features.shape[:-1]) + (3,), np.float32)
        L.call("dn_denoise", self._h, _ptr(features), w, h, b, _ptr(out), _stream() if dev else None,
               L.RT_FLAG_DEVICE_PTRS if dev else 0)
        return out

    def backward(self, features, target, read_loss: bool = True):
        """Loss and gradients of one batch (kept on the device; ``get_grads`` reads them)."""
        b, h, w, _ = _nhwc(features, FEATURES)
        dev = _is_cuda(features)
        loss = C.c_float()
        L.call("dn_backward", self._h, _ptr(features), _ptr(target), w, h, b, C.byref(loss) if read_loss else None,
               _stream() if dev else None, L.RT_FLAG_DEVICE_PTRS if dev else 0)
        return loss.value if read_loss else None

    def adam_step(self, lr: float) -> None:
        L.call("dn_adam_step", self._h, float(lr), _stream() if _torch_cuda() else None)

    def train_step(self, features, target, lr: float, read_loss: bool = True):
        b, h, w, _ = _nhwc(features, FEATURES)
        dev = _is_cuda(features)
        loss = C.c_float()
        L.call("dn_train_step", self._h, _ptr(features), _ptr(target), w, h, b, float(lr),
               C.byref(loss) if read_loss else None, _stream() if dev else None, L.RT_FLAG_DEVICE_PTRS if dev else 0)
        return loss.value if read_loss else None

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().dn_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_pairs(tracer, cameras, width: int, height: int, spp_in=4, spp_ref=1024, depth: int = 5, mode: int = 1,
                 clamp: float = 5.0, seed: int = 0):
    """Denoiser inputs and targets rendered by the path tracer itself: for each camera, the
    features of a ``spp_in``-sample render (radiance + first-hit albedo, normal, distance and
    the standard error of the mean luminance; a sequence of sample counts is cycled through
    the cameras) and, when ``spp_ref`` is not 0, an independent render accumulated in double
    precision with ``spp_ref`` samples (an int, or a function of the input's sample count).
    Returns CUDA tensors (N, H, W, 11) and (N, H, W, 3) (targets None without spp_ref)."""
    import torch

    n = len(cameras)
    dev = torch.device("cuda", tracer.device)
    feats = torch.empty((n, height, width, FEATURES), dtype=torch.float32, device=dev)
    targets = torch.empty((n, height, width, 3), dtype=torch.float32, device=dev) if spp_ref else None
    img = torch.empty((height, width, 3), dtype=torch.float32, device=dev)
    aov = torch.empty((height, width, 8), dtype=torch.float32, device=dev)
    for k, cam in enumerate(cameras):
        cam = dict(cam, ratio=width / height)
        img.zero_()
        spp = spp_in[k % len(spp_in)] if isinstance(spp_in, (list, tuple)) else spp_in
        tracer.render(cam, spp, depth, img, seed=seed + 2 * k, mode=mode, clamp=clamp, aov=aov)
        feats[k, ..., :3] = img
        feats[k, ..., 3:] = aov
        if spp_ref:
            img.zero_()
            ref = spp_ref(spp) if callable(spp_ref) else spp_ref
            tracer.render(cam, ref, depth, img, seed=seed + 2 * k + 1, mode=mode, clamp=clamp, fp64=True)
            targets[k] = img
    return feats, targets


def rel_rmse_t(x, ref, eps: float = 1e-2) -> float:
    """rel_rmse on CUDA tensors (float64 arithmetic)."""
    d = (x.double() - ref.double()) / (ref.double() + eps)
    return float(d.square().mean().sqrt())


def progressive_curves(tracer, camera, width: int, height: int, spp_levels, truth, denoiser=None, depth: int = 5,
                       mode: int = 1, clamp: float = 5.0, seed: int = 0):
    """Plain path tracing and path tracing + denoiser at equal sample counts on one view, as
    the sample count doubles: renders of ``spp_levels[0]`` and then of each level's
    difference to the previous one are added up (independent random streams), so that the
    image at level N costs the render time of N samples per pixel; the features (first-hit
    buffers and the standard error) are combined the same way. At every level: the plain
    image's relative RMSE against ``truth`` (H, W, 3 CUDA tensor) and the cumulative device
    render time, and with ``denoiser`` the denoised image's error and the denoising time
    (CUDA events). Returns [{spp, render_s, plain, denoised, denoise_ms}]."""
    import torch

    dev = torch.device("cuda", tracer.device)
    w = torch.tensor([0.2126, 0.7152, 0.0722], dtype=torch.float64, device=dev)
    rad = torch.zeros((height, width, 3), dtype=torch.float64, device=dev)
    feat = torch.zeros((height, width, 7), dtype=torch.float64, device=dev)
    s1 = torch.zeros((height, width), dtype=torch.float64, device=dev)
    s2 = torch.zeros((height, width), dtype=torch.float64, device=dev)
    img = torch.empty((height, width, 3), dtype=torch.float32, device=dev)
    aov = torch.empty((height, width, 8), dtype=torch.float32, device=dev)
    f = torch.empty((1, height, width, FEATURES), dtype=torch.float32, device=dev)
    out = torch.empty((1, height, width, 3), dtype=torch.float32, device=dev)
    cam = dict(camera, ratio=width / height)
    total, render_s, curve = 0, 0.0, []
    for k, level in enumerate(spp_levels):
        n = level - total
        img.zero_()
        tracer.render(cam, n, depth, img, seed=seed + k, mode=mode, clamp=clamp, fp64=True, aov=aov)
        render_s += tracer.last_stats()["device_ms"] / 1e3
        m = img.double() @ w  # mean luminance of this render
        se = aov[..., 7].double()
        rad += n * img.double()
        feat += n * aov[..., :7].double()
        s1 += n * m
        s2 += n * (n * se.square() + m.square())  # n E[L^2] = n (n se^2 + m^2)
        total = level
        point = {"spp": level, "render_s": render_s, "plain": rel_rmse_t(rad / total, truth)}
        if denoiser is not None:
            f[0, ..., :3] = (rad / total).float()
            f[0, ..., 3:10] = (feat / total).float()
            mean = s1 / total
            f[0, ..., 10] = ((s2 / total - mean.square()).clamp(min=0.0) / total).sqrt().float()
            denoiser.denoise(f, out)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                denoiser.denoise(f, out)
            e1.record()
            torch.cuda.synchronize()
            point["denoise_ms"] = e0.elapsed_time(e1) / 3
            point["denoised"] = rel_rmse_t(out[0], truth)
        curve.append(point)
    return curve


def time_to(points, threshold: float):
    """Seconds to reach a relative RMSE of ``threshold`` along [(seconds, error)], interpolated
    log-log between the two measured points around it; None when no measured point reaches
    it."""
    pts = sorted(points)
    if pts and pts[0][1] <= threshold:
        return pts[0][0]
    for (t0, e0), (t1, e1) in zip(pts, pts[1:]):
        if e0 > threshold >= e1:
            a = (np.log(threshold) - np.log(e0)) / (np.log(e1) - np.log(e0))
            return float(np.exp(np.log(t0) + a * (np.log(t1) - np.log(t0))))
    return None


def train_step_dp(net, features, target, lr: float, group=None, read_loss: bool = True):
    """One data-parallel training step, run by every process of ``group``
    (torch.distributed) on its own share of the batch: its loss and gradients
    (``net.backward``), their mean over the processes (one all_reduce of the flat
    gradient; with equal shares that is the gradient of the whole batch, whose loss is a
    mean over pixels), then the same Adam step everywhere, so the processes' parameters stay
    identical. CUDA tensors travel through NCCL on the device; with gloo, or host arrays,
    through host memory. Returns the mean loss over the processes (or None)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    loss = net.backward(features, target, read_loss=read_loss)
    dev = _is_cuda(features)
    on_device = dev and dist.get_backend(group) == "nccl"
    g = torch.empty(net.param_count + 1, dtype=torch.float32, device=features.device if dev else "cpu")
    if dev:
        net.read_grads(g[:-1])
    else:
        net.read_grads(g[:-1].numpy())
    g[-1] = float(loss) if read_loss else 0.0
    buf = g if (on_device or not dev) else g.cpu()
    dist.all_reduce(buf, group=group)
    buf /= world
    if buf is not g:
        g.copy_(buf)
    if dev:
        net.write_grads(g[:-1])
    else:
        net.write_grads(g[:-1].numpy())
    net.adam_step(lr)
    return float(buf[-1]) if read_loss else None


def train(denoiser, feats, targets, steps: int, batch: int = 8, crop: int = 64, lr: float = 2e-3, seed: int = 0,
          log_every: int = 0):
    """Adam on random ``crop`` x ``crop`` crops of (feats, targets) -- CUDA tensors as
    render_pairs returns them -- each crop flipped and transposed at random, with a
    cosine-decayed learning rate. Crops are gathered on the device; only the logged losses
    (every ``log_every`` steps) synchronise. Returns [(step, loss)]."""
    import math

    import torch

    n, h, w, _ = feats.shape
    if crop % 16 or crop > min(h, w):
        raise ValueError("crop must be a multiple of 16 no larger than the images")
    gen = torch.Generator(device=feats.device)
    gen.manual_seed(int(seed))
    ar = torch.arange(crop, device=feats.device)
    losses = []
    for s in range(steps):
        i = torch.randint(0, n, (batch,), generator=gen, device=feats.device)
        y = torch.randint(0, h - crop + 1, (batch,), generator=gen, device=feats.device)
        x = torch.randint(0, w - crop + 1, (batch,), generator=gen, device=feats.device)
        flip = torch.randint(0, 8, (batch,), generator=gen, device=feats.device)
        ry = torch.where((flip & 1).bool()[:, None], crop - 1 - ar, ar)
        rx = torch.where((flip & 2).bool()[:, None], crop - 1 - ar, ar)
        rows, cols = (y[:, None] + ry)[:, :, None], (x[:, None] + rx)[:, None, :]
        tr = (flip & 4).bool()[:, None, None]
        rows, cols = torch.where(tr, rows.transpose(1, 2), rows), torch.where(tr, cols.transpose(1, 2), cols)
        bi = i[:, None, None]
        f = feats[bi, rows, cols].contiguous()
        t = targets[bi, rows, cols].contiguous()
        lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
        read = bool(log_every) and (s % log_every == 0 or s == steps - 1)
        loss = denoiser.train_step(f, t, lr_s, read_loss=read)
        if read:
            losses.append((s, loss))
    return losses


def _torch_cuda() -> bool:
    try:
        import torch

        return torch.cuda.is_available() and torch.cuda.is_initialized()
    except Exception:
        return False


def conv3x3(x0, weights, cout: int, x1=None, up0: bool = False, bias=None, relu: bool = False, out_fp32=True):
    """One dn_conv3x3 layer on CUDA tensors: x0 (B, H>>up0, W>>up0, c0) and x1 (B, H, W, c1)
    bfloat16, weights bfloat16 (9, c0 + c1, cout), bias float32 (cout,) or None."""
    import torch

    b, h0, w0, c0 = x0.shape
    h, w = (2 * h0, 2 * w0) if up0 else (h0, w0)
    c1 = 0 if x1 is None else x1.shape[3]
    out = torch.empty((b, h, w, cout), dtype=torch.float32 if out_fp32 else torch.bfloat16, device=x0.device)
    L.call("dn_conv3x3", C.c_void_p(x0.data_ptr()), c0, int(up0), C.c_void_p(x1.data_ptr()) if x1 is not None else None,
           c1, b, h, w, C.c_void_p(weights.data_ptr()), C.c_void_p(bias.data_ptr()) if bias is not None else None, cout,
           int(relu), C.c_void_p(out.data_ptr()), int(out_fp32), _stream())
    return out


def conv3x3_backward(x0, weights_f32, gy, x1=None, up0: bool = False, want_dx=True, want_dw=True):
    """dn_conv3x3_backward on CUDA tensors: returns (dx (B, H, W, c0 + c1) float32 or None,
    dw (9, c0 + c1, cout) float32 or None) for the bfloat16 output gradient gy."""
    import torch

    b, h, w, cout = gy.shape
    c0 = x0.shape[3]
    c1 = 0 if x1 is None else x1.shape[3]
    dx = torch.empty((b, h, w, c0 + c1), dtype=torch.float32, device=gy.device) if want_dx else None
    dw = torch.empty((9, c0 + c1, cout), dtype=torch.float32, device=gy.device) if want_dw else None
    L.call("dn_conv3x3_backward", C.c_void_p(x0.data_ptr()), c0, int(up0),
           C.c_void_p(x1.data_ptr()) if x1 is not None else None, c1, b, h, w, C.c_void_p(weights_f32.data_ptr()),
           cout, C.c_void_p(gy.data_ptr()), C.c_void_p(dx.data_ptr()) if dx is not None else None,
           C.c_void_p(dw.data_ptr()) if dw is not None else None, _stream())
    return dx, dw
