"""PathTracer::render split over processes (one per GPU): interleaved pixel tiles per rank and
one sum of the images over the ranks (pathtracer.render_split, pt_render_options.ranks).

* CPU (gloo, world size 2 and 3): the host logic -- each rank renders only its tiles through
  a stand-in tracer that writes the C restatement's image on the owned tiles and zeros
  elsewhere, as the library documents; all_reduce and reduce-to-root assemble exactly the
  one-process image.
* GPU (gloo, world size 2, both ranks on cuda:0; the ranks' kernels never wait on each
  other): the library's split renders, summed, equal the one-process render bit for bit, for
  the reference and the extended estimator, with double-precision accumulation."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _PortTracer:
    """Renders like PathTracer.render with a rank split, from a precomputed full image."""

    def __init__(self, full):
        self.full = full

    def render(self, camera, samples, depth, image, seed=0, mode=0, clamp=5.0, fp64=False, ranks=1, rank=0):
        from rendu_gb300.pathtracer import rank_tile_mask

        own = rank_tile_mask(image.shape[0], image.shape[1], ranks, rank)
        image[...] = 0.0
        image[own] = self.full[own]
        return image


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cpu_worker(rank, world, port, full, out_dir, use_reduce):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from rendu_gb300.pathtracer import render_split

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    img = np.full_like(full, 7.0)  # the caller's image; every pixel is rewritten
    render_split(_PortTracer(full), {}, 4, 3, img, dst=0 if use_reduce else None)
    if rank == 0 or not use_reduce:
        np.save(os.path.join(out_dir, f"r{rank}.npy"), img)
    dist.destroy_process_group()


@pytest.mark.parametrize("world,use_reduce", [(2, False), (3, True)])
def test_split_assembly_on_gloo(tmp_path, port_lib, world, use_reduce):
    import torch.multiprocessing as mp

    from oracle import oracle as O
    from rendu_gb300 import scenes as S
    from rendu_gb300.pathtracer import rank_tile_mask

    sc = S.cornell_scene(20261203, True)
    w, h = 96, 100  # 9,600 pixels: three tiles, the last one partial
    cam = dict(sc.camera, ratio=w / h)
    full = O.PortPathTracer(sc).render(cam, 4, 3, w, h, seed=11).astype(np.float32)
    masks = [rank_tile_mask(h, w, world, r) for r in range(world)]
    assert np.array_equal(np.sum(masks, 0), np.ones((h, w)))  # the tiles cover the image once
    mp.start_processes(_cpu_worker, args=(world, _free_port(), full, str(tmp_path), use_reduce), nprocs=world,
                       start_method="spawn")
    for r in range(world if not use_reduce else 1):
        got = np.load(tmp_path / f"r{r}.npy")
        assert np.array_equal(got.view(np.uint32), full.view(np.uint32))


def _gpu_worker(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import rendu_gb300 as R
    from rendu_gb300 import scenes as S
    from rendu_gb300.pathtracer import render_split

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    for name, sc, mode in (("cornell", S.cornell_scene(20261203, True), 0),
                           ("instanced", S.instanced_scene(20261206, instances=24, subdivisions=3), 1)):
        w, h = 200, 150
        cam = dict(sc.camera, ratio=w / h)
        tr = R.PathTracer(sc)
        img = torch.full((h, w, 4), 0.25, dtype=torch.float32, device="cuda")  # accumulated into, alpha kept
        render_split(tr, cam, 8, 4, img, seed=3, mode=mode, fp64=(mode == 1))
        torch.cuda.synchronize()
        np.save(os.path.join(out_dir, f"{name}_r{rank}.npy"), img.cpu().numpy())
        tr.close()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_split_render_equals_one_process_render(cuda_lib, tmp_path):
    import torch
    import torch.multiprocessing as mp

    from rendu_gb300 import scenes as S

    mp.start_processes(_gpu_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, start_method="spawn")
    for name, sc, mode in (("cornell", S.cornell_scene(20261203, True), 0),
                           ("instanced", S.instanced_scene(20261206, instances=24, subdivisions=3), 1)):
        w, h = 200, 150
        cam = dict(sc.camera, ratio=w / h)
        tr = cuda_lib.PathTracer(sc)
        ref = torch.full((h, w, 4), 0.25, dtype=torch.float32, device="cuda")
        tr.render(cam, 8, 4, ref, seed=3, mode=mode, fp64=(mode == 1))
        ref = ref.cpu().numpy()
        tr.close()
        assert ref[..., :3].mean() > 0.0
        for r in range(2):
            got = np.load(tmp_path / f"{name}_r{r}.npy")
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"{name}: rank {r} differs"
