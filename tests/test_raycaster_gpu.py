"""Parity of the sm_103a raycaster with the reference (golden fixtures) and with the C
restatement at larger sizes. Bar: hit/miss and triangle id bit-exact except exact distance
ties; distances and barycentrics bit-exact (the per-triangle test is the reference's
arithmetic)."""
import numpy as np
import pytest

from conftest import golden_meshes, load_golden

pytestmark = pytest.mark.gpu
NO_HIT = 0xFFFFFFFF


def _gpu_from_meshes(R, meshes):
    rc = R.Raycaster(0)
    for pos, idx, m in meshes:
        rc.add_mesh(pos, idx, m)
    rc.updateHierarchy()
    return rc


def _port_from_meshes(O, meshes):
    p = O.PortRaycaster()
    for pos, idx, m in meshes:
        p.add_mesh(pos, idx, m)
    p.build()
    return p


def _assert_closest_equal(h, ref_prim, ref_t, ref_u, ref_v, rays, port):
    """t bit-exact everywhere; ids equal unless both triangles give the same t."""
    bad = np.nonzero(h["t"].view(np.uint32) != ref_t.view(np.uint32))[0]
    assert len(bad) == 0, (f"{len(bad)} distances differ, e.g. rays {bad[:5].tolist()}: gpu t/prim "
                           f"{h['t'][bad[:5]].tolist()} {h['prim'][bad[:5]].tolist()} vs "
                           f"{ref_t[bad[:5]].tolist()} {ref_prim[bad[:5]].tolist()}")
    diff = np.nonzero(h["prim"] != ref_prim)[0]
    for i in diff:
        r_a, a = port.test_triangle(rays[i], h["prim"][i])
        r_b, b = port.test_triangle(rays[i], ref_prim[i])
        assert r_a == 1 and r_b == 1 and a["t"] == b["t"], f"ray {i}: id differs without a tie"
    same = h["prim"] == ref_prim
    assert np.array_equal(h["u"][same].view(np.uint32), ref_u[same].view(np.uint32))
    assert np.array_equal(h["v"][same].view(np.uint32), ref_v[same].view(np.uint32))
    return len(diff)


def test_closest_matches_reference_golden(cuda_lib, port_lib):
    g = load_golden("raycaster_small.npz")
    meshes = golden_meshes(g)
    rc = _gpu_from_meshes(cuda_lib, meshes)
    h = rc.intersect_batch(g["rays"])
    ties = _assert_closest_equal(h, g["hit_prim"], g["hit_t"], g["hit_u"], g["hit_v"], g["rays"],
                                 _port_from_meshes(port_lib, meshes))
    assert ties <= len(h) // 1000


def test_closest_equals_brute_force(cuda_lib, port_lib):
    """With the (t, id) order both the GPU and the exhaustive checker are deterministic."""
    g = load_golden("raycaster_small.npz")
    meshes = golden_meshes(g)
    rc = _gpu_from_meshes(cuda_lib, meshes)
    h = rc.intersect_batch(g["rays"])
    b = _port_from_meshes(port_lib, meshes).brute(g["rays"])
    assert np.array_equal(h["prim"], b["prim"])
    assert np.array_equal(h["t"].view(np.uint32), b["t"].view(np.uint32))


def test_any_and_visible_match_reference_golden(cuda_lib):
    g = load_golden("raycaster_small.npz")
    rc = _gpu_from_meshes(cuda_lib, golden_meshes(g))
    assert np.array_equal(rc.intersect_any_batch(g["rays"]), g["any"])
    assert np.array_equal(rc.visible_batch(g["segs"]), g["visible"])


def test_hit_record_mapping_matches_reference(cuda_lib):
    """prim -> (meshId, localId) as in Raycaster::Hit; interpolateAttribute weights."""
    g = load_golden("raycaster_small.npz")
    meshes = golden_meshes(g)
    rc = _gpu_from_meshes(cuda_lib, meshes)
    offs = np.cumsum([0] + [len(i) // 3 for _, i, _ in meshes])
    for k in np.nonzero(g["hit_prim"] != NO_HIT)[0][:200]:
        o = g["rays"][k]
        hit = rc.intersects(o[0:3], o[4:7], float(o[3]), float(o[7]))
        assert hit.hit
        mesh = int(np.searchsorted(offs, g["hit_prim"][k], side="right") - 1)
        if hit.meshId == mesh:
            assert hit.localId == 3 * (int(g["hit_prim"][k]) - offs[mesh])
        assert hit.w == pytest.approx(1.0 - hit.u - hit.v, abs=1e-6)


def test_device_pointer_path_equals_host_path(cuda_lib):
    import torch

    g = load_golden("raycaster_small.npz")
    rc = _gpu_from_meshes(cuda_lib, golden_meshes(g))
    hh = rc.intersect_batch(g["rays"])
    d_rays = torch.from_numpy(g["rays"]).cuda()
    dh = rc.intersect_batch(d_rays)
    da = rc.intersect_any_batch(d_rays)
    torch.cuda.synchronize()
    dh = dh.cpu().numpy()
    assert np.array_equal(dh.view(np.uint32)[:, 3], hh["prim"])
    assert np.array_equal(dh[:, 0].view(np.uint32), hh["t"].view(np.uint32))
    assert np.array_equal(da.cpu().numpy(), g["any"])


@pytest.mark.parametrize("subdiv,n", [(6, 1 << 20)])
def test_large_mesh_matches_port(cuda_lib, port_lib, subdiv, n):
    from rendu_gb300 import scenes as S

    mesh = S.icosphere_mesh(subdiv, seed=31)
    rays = S.random_rays(n, mesh.positions.min(0), mesh.positions.max(0), seed=32, scale=1.6)
    meshes = [(mesh.positions, mesh.indices, S.translation((0.1, 0.2, -0.3)) @ S.rotation_y(0.4))]
    rc = _gpu_from_meshes(cuda_lib, meshes)
    port = _port_from_meshes(port_lib, meshes)
    h = rc.intersect_batch(rays)
    p = port.intersect(rays)
    ties = _assert_closest_equal(h, p["prim"], p["t"], p["u"], p["v"], rays, port)
    assert ties <= n // 10000
    assert np.array_equal(rc.intersect_any_batch(rays), port.intersect_any(rays))


def test_full_size_raycaster_properties(cuda_lib, port_lib):
    """Raycaster workload at full size (1,310,720 triangles, 16,777,216 rays): the any-hit
    answer equals 'closest hit exists' on every ray, hits lie in their windows, and a
    200k-ray sample matches the C restatement."""
    import torch

    from rendu_gb300 import scenes as S

    mesh, rays = S.raycaster_workload()
    rc = _gpu_from_meshes(cuda_lib, [(mesh.positions, mesh.indices, None)])
    d_rays = torch.from_numpy(rays).cuda()
    dh = rc.intersect_batch(d_rays)
    da = rc.intersect_any_batch(d_rays)
    torch.cuda.synchronize()
    prim = dh[:, 3].contiguous().view(torch.int32)
    hit = prim != -1
    assert torch.equal(hit.to(torch.uint8), da)
    t = dh[:, 0]
    assert bool(((t > d_rays[:, 3]) | ~hit).all())
    assert bool(((t < d_rays[:, 7]) | ~hit).all())
    sample = np.random.default_rng(3).choice(len(rays), 200000, replace=False)
    port = _port_from_meshes(port_lib, [(mesh.positions, mesh.indices, None)])
    p = port.intersect(rays[sample])
    hs = dh[torch.from_numpy(sample).cuda()].cpu().numpy()
    assert np.array_equal(hs[:, 0].view(np.uint32), p["t"].view(np.uint32))
    diff = hs.view(np.uint32)[:, 3] != p["prim"]
    assert diff.sum() <= 20


def test_host_buffer_pipeline_equals_device_path(cuda_lib):
    """The pipelined host-buffer path (chunks of up to 2M records, the last three halving,
    two traversal streams) at 16,777,216 rays gives the device path's answers bit for bit,
    with pinned and with pageable buffers, for closest hit, any hit and visibility; and a
    ray count that is no multiple of the chunk size splits correctly too."""
    import torch

    from rendu_gb300 import _lib as L
    from rendu_gb300 import scenes as S

    mesh, rays = S.raycaster_workload()
    rc = _gpu_from_meshes(cuda_lib, [(mesh.positions, mesh.indices, None)])
    d_rays = torch.from_numpy(rays).cuda()
    dh = rc.intersect_batch(d_rays).cpu().numpy()
    da = rc.intersect_any_batch(d_rays).cpu().numpy()
    pinned = torch.from_numpy(rays).pin_memory().numpy()
    for host in (rays, pinned):
        h = rc.intersect_batch(host)
        assert np.array_equal(h.view(np.uint32).reshape(-1, 4), dh.view(np.uint32))
        assert np.array_equal(rc.intersect_any_batch(host), da)
    m = len(rays) - 12345
    h = rc.intersect_batch(rays[:m])
    assert np.array_equal(h.view(np.uint32).reshape(-1, 4), dh[:m].view(np.uint32))
    segs = np.concatenate([rays[:, 0:3], rays[:, 0:3] + 3.0 * rays[:, 4:7]], 1).astype(np.float32)
    d_vis = torch.empty(len(segs), dtype=torch.uint8, device="cuda")
    d_segs = torch.from_numpy(segs).cuda()
    L.call("rt_visible", rc._h, d_segs.data_ptr(), len(segs), d_vis.data_ptr(), None, L.RT_FLAG_DEVICE_PTRS)
    torch.cuda.synchronize()
    assert np.array_equal(rc.visible_batch(segs), d_vis.cpu().numpy())


def test_edge_cases(cuda_lib):
    R = cuda_lib
    # Empty raycaster: every query misses.
    rc = R.Raycaster(0)
    rc.updateHierarchy()
    rays = np.array([[0, 0, -2, 1e-4, 0, 0, 1, 1e8]], np.float32)
    assert rc.intersect_batch(rays)["prim"][0] == NO_HIT
    assert rc.intersect_any_batch(rays)[0] == 0
    # One triangle; rays through its interior, edge, vertex, outside; windows.
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    rc = R.Raycaster(0)
    rc.add_mesh(tri, np.array([0, 1, 2], np.uint32))
    rc.updateHierarchy()
    rays = np.array([
        [0.2, 0.2, -1, 1e-4, 0, 0, 1, 1e8],   # hit at t=1
        [0.2, 0.2, -1, 1e-4, 0, 0, -1, 1e8],  # pointing away
        [0.2, 0.2, -1, 1e-4, 0, 0, 1, 0.5],   # window ends before
        [0.2, 0.2, -1, 2.0, 0, 0, 1, 1e8],    # window starts after
        [2.0, 2.0, -1, 1e-4, 0, 0, 1, 1e8],   # outside
        [0.0, 0.0, -1, 1e-4, 0, 0, 1, 1e8],   # vertex
        [0.5, 0.5, -1, 1e-4, 0, 0, 1, 1e8],   # hypotenuse
        [0.2, 0.2, -1, 1e-4, 0, 0, 0, 1e8],   # zero direction
        [0.2, 0.2, -1, 1e-4, 0, 0, 2.5, 1e8],  # unnormalised direction
        [0.2, 0.2, 0, 1e-4, 1, 0, 0, 1e8],    # in the triangle's plane
    ], np.float32)
    h = rc.intersect_batch(rays)
    got = (h["prim"] != NO_HIT).tolist()
    assert got == [True, False, False, False, False, True, True, False, True, False]
    assert h["t"][0] == np.float32(1.0) and h["t"][8] == np.float32(1.0)
    assert (rc.intersect_any_batch(rays) == np.array(got, np.uint8)).all()
    # Degenerate (zero-area) triangles never hit.
    rc = R.Raycaster(0)
    rc.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float32), np.array([0, 1, 2], np.uint32))
    rc.updateHierarchy()
    assert rc.intersect_batch(np.array([[1, 0, -1, 1e-4, 0, 0, 1, 1e8]], np.float32))["prim"][0] == NO_HIT


def test_errors_are_reported(cuda_lib):
    R = cuda_lib
    rc = R.Raycaster(0)
    with pytest.raises(R.RenduError) as e:
        rc.add_mesh(np.zeros((3, 3), np.float32), np.array([0, 1, 5], np.uint32))
    assert e.value.code == 1
    with pytest.raises(R.RenduError) as e:
        rc.add_mesh(np.zeros((3, 3), np.float32), np.array([0, 1], np.uint32))
    assert e.value.code == 1
    rc.add_mesh(np.eye(3, dtype=np.float32), np.array([0, 1, 2], np.uint32))
    with pytest.raises(R.RenduError) as e:
        rc.intersect_batch(np.zeros((1, 8), np.float32))
    assert e.value.code == 5  # before updateHierarchy
    rc.updateHierarchy()
    rc.intersect_batch(np.zeros((1, 8), np.float32))
    rc.add_mesh(np.eye(3, dtype=np.float32), np.array([0, 1, 2], np.uint32))
    with pytest.raises(R.RenduError):
        rc.intersect_batch(np.zeros((1, 8), np.float32))  # meshes added since the build


def test_many_meshes_and_stats(cuda_lib, port_lib):
    """200 transformed instances (the large path-tracer scene's shape): per-mesh roots in
    the reference, one hierarchy here; answers identical."""
    from rendu_gb300 import scenes as S

    rng = np.random.default_rng(8)
    sph = S.icosphere_mesh(2, seed=4)
    box = S.box_mesh()
    meshes = []
    for k in range(200):
        m = S.translation(rng.uniform(-10, 10, 3)) @ S.rotation_y(rng.uniform(0, 6.28)) @ S.scaling(rng.uniform(0.3, 1.5))
        src = sph if k % 2 else box
        meshes.append((src.positions, src.indices, m))
    rc = _gpu_from_meshes(cuda_lib, meshes)
    port = _port_from_meshes(port_lib, meshes)
    rays = S.random_rays(200000, (-11, -11, -11), (11, 11, 11), seed=9, scale=1.0)
    h = rc.intersect_batch(rays)
    p = port.intersect(rays)
    _assert_closest_equal(h, p["prim"], p["t"], p["u"], p["v"], rays, port)
    st = rc.stats()
    assert st["meshes"] == 200 and st["triangles"] == 100 * (320 + 12)
    assert 0 < st["nodes"] < st["triangles"] and st["leaves"] > 0


def test_hit_info_batch_gives_reference_mesh_and_local_ids(cuda_lib):
    """rt_hit_info: Raycaster::Hit's meshId and localId (Raycaster.cpp:177-179) for a whole
    batch, host and device buffers, with an empty mesh between non-empty ones."""
    import torch

    g = load_golden("raycaster_small.npz")
    meshes = golden_meshes(g)
    empty = (np.zeros((0, 3), np.float32), np.zeros(0, np.uint32), None)
    meshes = meshes[:2] + [empty] + meshes[2:]
    rc = _gpu_from_meshes(cuda_lib, meshes)
    h = rc.intersect_batch(g["rays"])
    assert np.array_equal(h["prim"], g["hit_prim"])
    mesh_ids, local_ids = rc.hit_info(h)
    sizes = [len(i) // 3 for _, i, _ in meshes]
    offs = np.cumsum([0] + sizes)
    hit = g["hit_prim"] != NO_HIT
    want_mesh = np.searchsorted(offs, g["hit_prim"][hit], side="right") - 1
    # The golden ids are global over the reference's four meshes; the empty mesh shifts the
    # later mesh ids by one and leaves the triangle numbering unchanged.
    assert np.array_equal(mesh_ids[hit], want_mesh)
    assert np.array_equal(local_ids[hit], 3 * (g["hit_prim"][hit] - offs[want_mesh]))
    assert (mesh_ids[~hit] == NO_HIT).all() and (local_ids[~hit] == NO_HIT).all()
    assert 2 not in set(mesh_ids[hit].tolist())
    for k in np.nonzero(hit)[0][:50]:
        assert rc.prim_info(int(h["prim"][k])) == (mesh_ids[k], local_ids[k])
    d_hits = rc.intersect_batch(torch.from_numpy(g["rays"]).cuda())
    dm, dl = rc.hit_info(d_hits)
    torch.cuda.synchronize()
    assert np.array_equal(dm.cpu().numpy().view(np.uint32), mesh_ids)
    assert np.array_equal(dl.cpu().numpy().view(np.uint32), local_ids)


def test_coincident_triangles_across_meshes(cuda_lib, port_lib):
    """Thousands of identical triangles in several meshes: the clustering build merges one
    pair per round and falls back to the radix tree after 512 rounds. The build succeeds
    and the answers equal the C restatement's (ties go to the smaller triangle id)."""
    from rendu_gb300 import scenes as S

    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    pos = np.tile(tri, (1500, 1))
    idx = np.arange(len(pos), dtype=np.uint32)
    other = S.icosphere_mesh(2, seed=3)
    meshes = [(pos, idx, None), (pos, idx, S.translation((0.0, 0.0, 0.5))), (other.positions, other.indices,
                                                                            S.translation((2.0, 0.0, 0.0)))]
    rc = _gpu_from_meshes(cuda_lib, meshes)
    port = _port_from_meshes(port_lib, meshes)
    rng = np.random.default_rng(12)
    n = 20000
    o = np.stack([rng.uniform(-0.5, 3.5, n), rng.uniform(-0.5, 1.5, n), np.full(n, 3.0)], 1)
    d = np.stack([rng.uniform(-0.2, 0.2, n), rng.uniform(-0.2, 0.2, n), -np.ones(n)], 1)
    rays = np.concatenate([o, np.full((n, 1), 1e-4), d, np.full((n, 1), 1e8)], 1).astype(np.float32)
    h = rc.intersect_batch(rays)
    p = port.intersect(rays)
    _assert_closest_equal(h, p["prim"], p["t"], p["u"], p["v"], rays, port)
    assert (h["prim"] != NO_HIT).sum() > n // 10
    assert np.array_equal(rc.intersect_any_batch(rays), port.intersect_any(rays))
    # Raycaster::visible's window (1e-4, |p1 - p0|) along p1 - p0, in float32 step by step.
    p0 = rays[:, 0:3]
    p1 = (p0 + np.float32(5.0) * rays[:, 4:7]).astype(np.float32)
    dv = (p1 - p0).astype(np.float32)
    ln = np.sqrt((dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1]) + dv[:, 2] * dv[:, 2]).astype(np.float32)
    seg_rays = np.concatenate([p0, np.full((n, 1), 1e-4, np.float32), dv, ln[:, None]], 1).astype(np.float32)
    assert np.array_equal(rc.visible_batch(np.concatenate([p0, p1], 1)), 1 - port.intersect_any(seg_rays))
