"""Data-parallel denoiser training (denoiser.train_step_dp): every process computes the loss
and gradients of its share of a batch, one all_reduce averages the flat gradient, and every
process applies the same Adam step.

* CPU (gloo, world size 2 and 3): the host logic, with a stand-in network whose loss and
  gradients come from the float64 restatement of the U-Net (oracle/denoiser.py): the
  averaged gradient equals the gradient of the whole batch, the mean loss its loss, and the
  processes end with identical parameters.
* GPU (gloo, two processes on one device; their kernels never wait on each other): the
  library's gradients of two half batches, averaged, match the gradient of the whole batch
  to float32 summation-order rounding, and both processes hold bit-identical parameters
  after two steps."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _OracleNet:
    """The Denoiser methods train_step_dp uses, computed by the float64 restatement."""

    def __init__(self, params):
        from oracle import denoiser as O

        self.O = O
        self.u = O.UNet()
        self.param_count = self.u.param_count
        self.p = np.asarray(params, np.float64).copy()
        self.m = np.zeros_like(self.p)
        self.v = np.zeros_like(self.p)
        self.step = 0
        self.g = None
        self.applied = []  # the gradients each Adam step used

    def backward(self, features, target, read_loss=True):
        loss, g = self.u.backward(self.p, features, target, bf16=False)
        self.g = g.astype(np.float32)
        return loss

    def read_grads(self, out):
        out[...] = self.g

    def write_grads(self, src):
        self.g = np.array(src, np.float32)

    def adam_step(self, lr):
        self.step += 1
        self.applied.append(self.g.copy())
        self.p, self.m, self.v = self.O.adam(self.p, self.g.astype(np.float64), self.m, self.v, self.step, lr)


def _batch(n, size, seed):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, 2.0, (n, size, size, 11)).astype(np.float32)
    t = rng.uniform(0.0, 2.0, (n, size, size, 3)).astype(np.float32)
    return f, t


def _params(seed):
    from oracle import denoiser as O

    rng = np.random.default_rng(seed)
    return rng.normal(0.0, 0.05, O.UNet().param_count)


def _cpu_worker(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from rendu_gb300.denoiser import train_step_dp

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    f, t = _batch(world, 16, 7)
    net = _OracleNet(_params(3))
    loss = train_step_dp(net, f[rank:rank + 1], t[rank:rank + 1], 1e-3)
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), p=net.p, g=net.applied[0], loss=loss)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_dp_step_equals_whole_batch_step_on_gloo(tmp_path, world):
    import torch.multiprocessing as mp

    mp.start_processes(_cpu_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    f, t = _batch(world, 16, 7)
    ref = _OracleNet(_params(3))
    ref_loss = ref.backward(f, t)
    outs = [np.load(tmp_path / f"r{r}.npz") for r in range(world)]
    for o in outs:
        assert np.array_equal(o["p"], outs[0]["p"])  # every process holds the same parameters
        assert abs(float(o["loss"]) - ref_loss) <= 1e-6 * abs(ref_loss)  # carried in float32
    g = outs[0]["g"]
    scale = np.abs(ref.g).max()
    assert np.allclose(g, ref.g, rtol=1e-5, atol=1e-6 * scale)


def _gpu_worker(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    from rendu_gb300 import denoiser as D

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    f, t = _batch(4, 64, 11)
    net = D.Denoiser(seed=3)
    fs = torch.from_numpy(f[2 * rank:2 * rank + 2]).cuda()
    ts = torch.from_numpy(t[2 * rank:2 * rank + 2]).cuda()
    grads = []
    for step in range(2):
        loss = D.train_step_dp(net, fs, ts, 1e-3)
        g = torch.empty(net.param_count, dtype=torch.float32, device="cuda")
        net.read_grads(g)  # the averaged gradient the step applied
        grads.append(g.cpu().numpy())
    torch.cuda.synchronize()
    np.savez(os.path.join(out_dir, f"g{rank}.npz"), p=net.get_params(), g0=grads[0], g1=grads[1], loss=loss)
    net.close()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_dp_gradients_match_whole_batch_on_gpu(cuda_lib, tmp_path):
    import torch
    import torch.multiprocessing as mp

    from rendu_gb300 import denoiser as D

    mp.start_processes(_gpu_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    f, t = _batch(4, 64, 11)
    net = D.Denoiser(seed=3)
    net.backward(torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda())
    ref = net.get_grads()
    net.close()
    a, b = np.load(tmp_path / "g0.npz"), np.load(tmp_path / "g1.npz")
    assert np.array_equal(a["p"], b["p"])  # identical parameters on both processes
    assert np.array_equal(a["g1"], b["g1"])
    scale = np.abs(ref).max()
    assert np.allclose(a["g0"], ref, rtol=1e-3, atol=1e-5 * scale)
    assert np.isfinite(a["loss"])
