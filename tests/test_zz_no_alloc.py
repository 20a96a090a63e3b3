"""rt_visible_noalloc: the visibility query for callers that cannot allocate device memory
(cudaMalloc forbidden or too slow where they run). Its scratch is a static device array
shared by every call, so this test checks two calls in a row -- the second one sees the
first one's leftovers in the scratch -- against the allocating entry point rt_visible.

Kept in a file collected last so that a failure here stops a `-x` run only after every
other test has run; it passes alone in a fresh process as well as after the others."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_meshes, load_golden

pytestmark = pytest.mark.gpu


def _noalloc():
    import rendu_gb300._lib as L

    f = L.lib().rt_visible_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_visible_noalloc_matches_rt_visible_on_two_calls(cuda_lib):
    import torch

    g = load_golden("raycaster_small.npz")
    rc = cuda_lib.Raycaster(0)
    for pos, idx, m in golden_meshes(g):
        rc.add_mesh(pos, idx, m)
    rc.updateHierarchy()
    rng = np.random.default_rng(77)
    rays = g["rays"]
    pick = rng.integers(0, len(rays), 60000)
    far = rays[pick, 0:3] + rng.uniform(0.05, 6.0, (len(pick), 1)) * rays[pick, 4:7] / np.linalg.norm(
        rays[pick, 4:7], axis=1, keepdims=True)
    second = np.concatenate([rays[pick, 0:3], far], 1).astype(np.float32)
    fn = _noalloc()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for segs in (g["segs"], second):  # 2,000 then 60,000 segments through the same scratch
        expected = rc.visible_batch(segs)
        d_segs = torch.from_numpy(np.ascontiguousarray(segs)).cuda()
        d_out = torch.full((len(segs),), 7, dtype=torch.uint8, device="cuda")
        assert fn(C.c_void_p(rc.handle), C.c_void_p(d_segs.data_ptr()), len(segs), C.c_void_p(d_out.data_ptr()),
                  stream) == 0
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), expected)
    assert np.array_equal(rc.visible_batch(g["segs"]), g["visible"])  # and the reference's own answer


def test_visible_noalloc_rejects_batches_beyond_its_scratch(cuda_lib):
    import rendu_gb300._lib as L

    rc = cuda_lib.Raycaster(0)
    rc.add_mesh(np.eye(3, dtype=np.float32), np.array([0, 1, 2], np.uint32))
    rc.updateHierarchy()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    code = _noalloc()(C.c_void_p(rc.handle), dummy, 262144 + 1, dummy, None)
    assert code == L.RT_ERR_ARG
    assert b"at most 262144" in L.lib().rt_last_error()
