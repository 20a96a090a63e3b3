"""Failure paths on the GPU, made to happen without faulting it.

The reference logs and returns on failure (PathTracer.cpp:162-168); here a bounded device
loop or a capped stack sets a status word and the call returns a status code:
* a traversal stack capped below what the hierarchy needs (rt_set_traversal_stack) ->
  RT_ERR_OVERFLOW, from the host-buffer call itself, and from rt_get_status after the
  asynchronous device-pointer and allocation-free calls;
* a shadow ray that has to pass more than 256 alpha-masked surfaces (the bound of the walk
  that restates PathTracer::checkVisibility, PathTracer.cpp:124-157) -> RT_ERR_TIMEOUT.
After each failure the same context or scene answers normally again."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _deep_raycaster(R, S):
    """A 327,680-triangle sphere and rays from inside it: closest-hit walks that push more
    than 2 stack entries."""
    mesh = S.icosphere_mesh(7, seed=5)
    rc = R.Raycaster(0)
    rc.add_mesh(mesh.positions, mesh.indices)
    rc.updateHierarchy()
    rng = np.random.default_rng(9)
    n = 1 << 16
    d = rng.normal(size=(n, 3)).astype(np.float32)
    o = (rng.uniform(-0.3, 0.3, (n, 3))).astype(np.float32)
    rays = np.concatenate([o, np.full((n, 1), 1e-4, np.float32), d, np.full((n, 1), 1e8, np.float32)], 1)
    return rc, rays


def test_capped_stack_reports_overflow_on_every_path(cuda_lib):
    import torch

    import rendu_gb300 as R
    import rendu_gb300._lib as L
    from rendu_gb300 import scenes as S

    rc, rays = _deep_raycaster(R, S)
    good = rc.intersect_batch(rays)
    assert (good["prim"] != L.RT_NO_HIT).all()  # every ray from inside hits the sphere
    assert rc.status() == L.RT_OK

    rc.set_traversal_stack(1)  # the 2-entry kernels
    with pytest.raises(L.RenduError) as e:
        rc.intersect_batch(rays)
    assert e.value.code == L.RT_ERR_OVERFLOW
    # Any-hit walks stop at their first hit, so they may or may not need the deep entries;
    # either way the call answers with a status, not a fault.
    try:
        rc.intersect_any_batch(rays)
    except L.RenduError as err:
        assert err.code == L.RT_ERR_OVERFLOW

    # Device pointers: the call returns at once; rt_get_status reports the overflow once.
    d_rays = torch.from_numpy(rays).cuda()
    rc.intersect_batch(d_rays)
    assert rc.status() == L.RT_ERR_OVERFLOW
    assert rc.status() == L.RT_OK

    # The allocation-free visibility query reports through the same word.
    segs = np.concatenate([rays[:, 0:3], rays[:, 0:3] + 4.0 * rays[:, 4:7]], 1).astype(np.float32)
    d_segs = torch.from_numpy(segs).cuda()
    d_vis = torch.empty(len(segs), dtype=torch.uint8, device="cuda")
    f = L.lib().rt_visible_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert f(C.c_void_p(rc.handle), C.c_void_p(d_segs.data_ptr()), len(segs), C.c_void_p(d_vis.data_ptr()),
             stream) == L.RT_OK
    assert rc.status() == L.RT_ERR_OVERFLOW

    # Back to the automatic bound: same answers as before, no status.
    rc.set_traversal_stack(0)
    again = rc.intersect_batch(rays)
    assert np.array_equal(again["prim"], good["prim"])
    assert np.array_equal(again["t"].view(np.uint32), good["t"].view(np.uint32))
    assert f(C.c_void_p(rc.handle), C.c_void_p(d_segs.data_ptr()), len(segs), C.c_void_p(d_vis.data_ptr()),
             stream) == L.RT_OK
    assert rc.status() == L.RT_OK
    assert np.array_equal(d_vis.cpu().numpy(), rc.visible_batch(segs))
    rc.close()


def test_set_traversal_stack_rejects_more_than_256(cuda_lib):
    import rendu_gb300 as R
    import rendu_gb300._lib as L

    rc = R.Raycaster(0)
    with pytest.raises(L.RenduError) as e:
        rc.set_traversal_stack(257)
    assert e.value.code == L.RT_ERR_ARG
    rc.close()


def _quad_stack_scene(S, layers: int):
    """A floor, `layers` fully transparent alpha-masked quads stacked above it and a point
    light above the stack: every shadow ray from the floor walks through all the layers."""
    sc = S.Scene()
    floor = sc.add_mesh(S.quad_mesh((-1, 0, 1), (2, 0, 0), (0, 0, -2)))
    sc.add_object(floor, sc.add_material((0.6, 0.6, 0.6)))
    pos, idx, uv = [], [], []
    for k in range(layers):
        y = 1.0 + k / layers
        base = len(pos)
        pos += [(-2, y, 2), (2, y, 2), (2, y, -2), (-2, y, -2)]
        uv += [(0, 0), (1, 0), (1, 1), (0, 1)]
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    stack = S.Mesh(np.array(pos, np.float32), np.array(idx, np.uint32), texcoords=np.array(uv, np.float32))
    clear = sc.add_texture(S.constant_texture([1.0, 1.0, 1.0, 0.0]))
    sc.add_object(sc.add_mesh(stack), sc.add_material(None, masked=True, albedo_tex=clear))
    sc.lights.append({"type": 0, "color": (5.0, 5.0, 5.0), "position": (0.0, 3.0, 0.0), "direction": (0, -1, 0),
                      "radius": 10.0, "inner": 0.5, "outer": 0.8, "shadows": True})
    sc.camera = {"eye": (0.0, 0.6, 0.0), "center": (0.0, 0.0, -0.01), "up": (0.0, 0.0, -1.0), "fov": 1.0,
                 "ratio": 1.0}
    return sc


def test_shadow_walk_through_too_many_cut_outs_times_out(cuda_lib):
    import rendu_gb300 as R
    import rendu_gb300._lib as L
    from rendu_gb300 import scenes as S

    ok = _quad_stack_scene(S, 200)  # within the 256-step bound: lit, no error
    tr = R.PathTracer(ok)
    img = np.zeros((32, 32, 3), np.float32)
    tr.render(ok.camera, 1, 1, img, seed=1)
    assert img.mean() > 0.0
    tr.close()

    bad = _quad_stack_scene(S, 300)
    tr = R.PathTracer(bad)
    img = np.zeros((32, 32, 3), np.float32)
    with pytest.raises(L.RenduError) as e:
        tr.render(bad.camera, 1, 1, img, seed=1)
    assert e.value.code == L.RT_ERR_TIMEOUT
    # The scene and the GPU still answer: a render without the light's shadow walk works.
    bad.lights[0]["shadows"] = False
    tr.close()
    tr = R.PathTracer(bad)
    img = np.zeros((32, 32, 3), np.float32)
    tr.render(bad.camera, 1, 1, img, seed=1)
    assert np.isfinite(img).all() and img.mean() > 0.0
    tr.close()


def test_misaligned_device_buffers_are_rejected(cuda_lib):
    """The traversal reads rays and writes hits as 16-byte vectors: device pointers that are
    not 16-byte aligned are refused before anything is launched."""
    import torch

    import rendu_gb300 as R
    import rendu_gb300._lib as L
    from rendu_gb300 import scenes as S

    mesh = S.icosphere_mesh(2, seed=1)
    rc = R.Raycaster(0)
    rc.add_mesh(mesh.positions, mesh.indices)
    rc.updateHierarchy()
    raw = torch.zeros(8 * 64 + 4, dtype=torch.float32, device="cuda")
    hits = torch.zeros(4 * 64 + 4, dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib = L.lib()
    for name, out in (("rt_intersect", hits), ("rt_intersect_any", hits)):
        f = getattr(lib, name)
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_uint32]
        code = f(C.c_void_p(rc.handle), C.c_void_p(raw.data_ptr() + 4), 64, C.c_void_p(out.data_ptr()), stream,
                 L.RT_FLAG_DEVICE_PTRS)
        assert code == L.RT_ERR_ARG, name
    f = lib.rt_intersect
    code = f(C.c_void_p(rc.handle), C.c_void_p(raw.data_ptr()), 64, C.c_void_p(hits.data_ptr() + 4), stream,
             L.RT_FLAG_DEVICE_PTRS)
    assert code == L.RT_ERR_ARG
    # aligned buffers still work
    assert f(C.c_void_p(rc.handle), C.c_void_p(raw.data_ptr()), 64, C.c_void_p(hits.data_ptr()), stream,
             L.RT_FLAG_DEVICE_PTRS) == L.RT_OK
    torch.cuda.synchronize()
    assert rc.status() == L.RT_OK
    rc.close()
