"""The C restatement (oracle/port) against the reference's own outputs.

The golden fixtures were produced by the reference's Raycaster compiled from its sources
(tests/golden/make_golden.py); the restatement must reproduce them bit for bit. Where the
reference tree is present, the restatement is also compared with the compiled reference
directly on fresh random inputs.
"""
import numpy as np
import pytest

from conftest import golden_meshes, load_golden


def _port_from_golden(O, g):
    p = O.PortRaycaster()
    for pos, idx, m in golden_meshes(g):
        p.add_mesh(pos, idx, m)
    p.build()
    return p


def _seg_rays(segs):
    """Raycaster::visible (Raycaster.cpp:226-230) as rays: d = p1 - p0, window (1e-4, |d|),
    glm::length = sqrt((x*x + y*y) + z*z) in float32."""
    s = segs.astype(np.float32)
    d = (s[:, 3:6] - s[:, 0:3]).astype(np.float32)
    dd = ((d[:, 0] * d[:, 0]).astype(np.float32) + (d[:, 1] * d[:, 1]).astype(np.float32)).astype(np.float32)
    dd = (dd + (d[:, 2] * d[:, 2]).astype(np.float32)).astype(np.float32)
    r = np.zeros((len(s), 8), np.float32)
    r[:, 0:3] = s[:, 0:3]
    r[:, 3] = np.float32(1e-4)
    r[:, 4:7] = d
    r[:, 7] = np.sqrt(dd)
    return r


def test_port_closest_matches_reference_golden(port_lib):
    g = load_golden("raycaster_small.npz")
    p = _port_from_golden(port_lib, g)
    h = p.intersect(g["rays"], threads=4)
    assert np.array_equal(h["prim"], g["hit_prim"])
    assert np.array_equal(h["t"].view(np.uint32), g["hit_t"].view(np.uint32))
    assert np.array_equal(h["u"].view(np.uint32), g["hit_u"].view(np.uint32))
    assert np.array_equal(h["v"].view(np.uint32), g["hit_v"].view(np.uint32))


def test_port_any_and_visible_match_reference_golden(port_lib):
    g = load_golden("raycaster_small.npz")
    p = _port_from_golden(port_lib, g)
    assert np.array_equal(p.intersect_any(g["rays"], threads=4), g["any"])
    vis = 1 - p.intersect_any(_seg_rays(g["segs"]), threads=4)
    assert np.array_equal(vis, g["visible"])


def test_brute_force_agrees_with_reference_golden(port_lib):
    """The hierarchy-free checker finds the reference's closest distance on every ray; the
    triangle id differs only on exact distance ties."""
    g = load_golden("raycaster_small.npz")
    p = _port_from_golden(port_lib, g)
    b = p.brute(g["rays"], threads=4)
    assert np.array_equal(b["t"].view(np.uint32), g["hit_t"].view(np.uint32))
    diff = np.nonzero(b["prim"] != g["hit_prim"])[0]
    for i in diff:
        r1, h1 = p.test_triangle(g["rays"][i], g["hit_prim"][i])
        assert r1 == 1 and h1["t"] == b["t"][i], "a differing id must be an exact tie"


def test_port_hits_are_geometrically_consistent(port_lib):
    g = load_golden("raycaster_small.npz")
    hit = g["hit_prim"] != 0xFFFFFFFF
    assert hit.mean() > 0.25
    u, v = g["hit_u"][hit], g["hit_v"][hit]
    assert (u >= 0).all() and (u <= 1).all() and (v >= 0).all() and (u + v <= 1.0 + 1e-6).all()
    assert (g["hit_t"][hit] > g["rays"][hit, 3]).all()
    assert (g["hit_t"][hit] < g["rays"][hit, 7]).all()
    assert (g["hit_t"][~hit] == np.finfo(np.float32).max).all()


def test_port_matches_compiled_reference_on_fresh_inputs(port_lib):
    O = port_lib
    if O.build_ref() is None:
        pytest.skip("reference tree not present")
    from rendu_gb300 import scenes as S

    mesh = S.icosphere_mesh(5, seed=99)
    rays = S.random_rays(60000, mesh.positions.min(0), mesh.positions.max(0), seed=5, scale=1.5)
    m = S.translation((0.2, -0.1, 0.3)) @ S.rotation_y(1.1)
    p = O.PortRaycaster()
    r = O.RefRaycaster()
    for x in (p, r):
        x.add_mesh(mesh.positions, mesh.indices, m)
        x.add_mesh(S.box_mesh().positions, S.box_mesh().indices)
        x.build()
    hp, hr = p.intersect(rays), r.intersect(rays)
    assert np.array_equal(hp["prim"], hr["prim"])
    assert np.array_equal(hp["t"].view(np.uint32), hr["t"].view(np.uint32))
    assert np.array_equal(p.intersect_any(rays), r.intersect_any(rays))


def test_port_many_meshes_match_reference(port_lib):
    """200 transformed instances: one root per mesh in both (Raycaster.cpp:64-69)."""
    O = port_lib
    if O.build_ref() is None:
        pytest.skip("reference tree not present")
    from rendu_gb300 import scenes as S

    rng = np.random.default_rng(8)
    sph, box = S.icosphere_mesh(2, seed=4), S.box_mesh()
    p, r = O.PortRaycaster(), O.RefRaycaster()
    for k in range(200):
        m = S.translation(rng.uniform(-10, 10, 3)) @ S.rotation_y(rng.uniform(0, 6.28)) @ S.scaling(rng.uniform(0.3, 1.5))
        src = sph if k % 2 else box
        for x in (p, r):
            x.add_mesh(src.positions, src.indices, m)
    p.build()
    r.build()
    rays = S.random_rays(50000, (-11, -11, -11), (11, 11, 11), seed=9, scale=1.0)
    hp, hr = p.intersect(rays), r.intersect(rays)
    assert np.array_equal(hp["prim"], hr["prim"])
    assert np.array_equal(hp["t"].view(np.uint32), hr["t"].view(np.uint32))
