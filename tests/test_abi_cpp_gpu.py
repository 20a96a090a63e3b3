"""The reference-side C++ binding, compiled and run on the GPU: a plain C++17 program that
includes only include/rendu_gb300.h declares the reference's Raycaster class (the members of
Raycaster.hpp:51-97: addMesh, updateHierarchy, intersects, intersectsAny, visible, Hit with
meshId/localId) over the C-ABI, with small stand-ins for glm::vec3/mat4 and Mesh. It adds the
golden meshes with their model matrices, answers the golden rays one by one through
intersects / intersectsAny / visible and all at once through the batched members, and the
test compares every answer with what the compiled reference returned."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_meshes, load_golden

pytestmark = pytest.mark.gpu

PROGRAM = r"""
#include "rendu_gb300.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

// Minimal stand-ins for the reference's glm types and Mesh (Mesh.hpp:126-132).
struct vec3 { float x, y, z; };
struct mat4 { float m[16]; };  // column-major, as glm
struct Mesh { std::vector<vec3> positions; std::vector<uint32_t> indices; };

// The reference's Raycaster (Raycaster.hpp:16-113) with its members routed to the library.
class Raycaster {
public:
    struct Hit {
        bool hit = false;
        float dist = 3.402823466e+38f, u = 0.f, v = 0.f, w = 0.f;
        unsigned long localId = 0, meshId = 0;
        Hit() = default;
        Hit(float d, float uu, float vv, unsigned long lid, unsigned long mid)
            : hit(true), dist(d), u(uu), v(vv), w(1.0f - uu - vv), localId(lid), meshId(mid) {}
    };
    Raycaster() { ok_ = rt_create(&ctx_, 0) == RT_OK; }
    ~Raycaster() { rt_destroy(ctx_); }
    Raycaster(const Raycaster &) = delete;
    Raycaster &operator=(const Raycaster &) = delete;
    bool ok() const { return ok_; }
    void addMesh(const Mesh &mesh, const mat4 &model) {
        uint32_t id = 0;
        ok_ &= rt_add_mesh(ctx_, &mesh.positions[0].x, mesh.positions.size(), mesh.indices.data(),
                           mesh.indices.size(), model.m, &id) == RT_OK;
    }
    void updateHierarchy() { ok_ &= rt_update_hierarchy(ctx_) == RT_OK; }
    Hit intersects(const vec3 &o, const vec3 &d, float mini = 0.0001f, float maxi = 1e8f) const {
        const rt_ray r{o.x, o.y, o.z, mini, d.x, d.y, d.z, maxi};
        rt_hit h;
        if (rt_intersect(ctx_, &r, 1, &h, nullptr, 0) != RT_OK || h.prim == RT_NO_HIT) return Hit();
        uint32_t meshId = 0, localId = 0;
        rt_prim_info(ctx_, h.prim, &meshId, &localId);
        return Hit(h.t, h.u, h.v, localId, meshId);
    }
    bool intersectsAny(const vec3 &o, const vec3 &d, float mini = 0.0001f, float maxi = 1e8f) const {
        const rt_ray r{o.x, o.y, o.z, mini, d.x, d.y, d.z, maxi};
        uint8_t occ = 0;
        rt_intersect_any(ctx_, &r, 1, &occ, nullptr, 0);
        return occ != 0;
    }
    bool visible(const vec3 &p0, const vec3 &p1) const {
        const float seg[6] = {p0.x, p0.y, p0.z, p1.x, p1.y, p1.z};
        uint8_t vis = 0;
        rt_visible(ctx_, seg, 1, &vis, nullptr, 0);
        return vis != 0;
    }
    // Batched members (the fast path).
    int intersects(const rt_ray *rays, size_t n, rt_hit *hits, uint32_t *meshIds, uint32_t *localIds) const {
        const int r = rt_intersect(ctx_, rays, n, hits, nullptr, 0);
        return r != RT_OK ? r : rt_hit_info(ctx_, hits, n, meshIds, localIds, nullptr, 0);
    }
    int intersectsAny(const rt_ray *rays, size_t n, uint8_t *occluded) const {
        return rt_intersect_any(ctx_, rays, n, occluded, nullptr, 0);
    }
private:
    rt_ctx *ctx_ = nullptr;
    bool ok_ = false;
};

template <class T> static std::vector<T> load(const char *dir, const char *name) {
    std::ifstream f(std::string(dir) + "/" + name, std::ios::binary | std::ios::ate);
    std::vector<T> v(size_t(f.tellg()) / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char *>(v.data()), v.size() * sizeof(T));
    return v;
}
template <class T> static void save(const char *dir, const char *name, const std::vector<T> &v) {
    std::ofstream f(std::string(dir) + "/" + name, std::ios::binary);
    f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    const char *dir = argv[1];
    const int meshes = std::atoi(argv[2]);
    Raycaster rc;
    if (!rc.ok()) { std::printf("create: %s\n", rt_last_error()); return 3; }
    for (int k = 0; k < meshes; ++k) {
        char pn[32], in[32], mn[32];
        std::snprintf(pn, sizeof pn, "pos%d.bin", k);
        std::snprintf(in, sizeof in, "idx%d.bin", k);
        std::snprintf(mn, sizeof mn, "model%d.bin", k);
        Mesh m;
        m.positions = load<vec3>(dir, pn);
        m.indices = load<uint32_t>(dir, in);
        const std::vector<float> mm = load<float>(dir, mn);
        mat4 model;
        for (int i = 0; i < 16; ++i) model.m[i] = mm[i];
        rc.addMesh(m, model);
    }
    rc.updateHierarchy();
    if (!rc.ok()) { std::printf("build: %s\n", rt_last_error()); return 4; }
    const std::vector<rt_ray> rays = load<rt_ray>(dir, "rays.bin");
    const std::vector<float> segs = load<float>(dir, "segs.bin");
    const size_t n = rays.size(), ns = segs.size() / 6;
    // One by one, through the reference's signatures.
    std::vector<float> t1(n), u1(n), v1(n);
    std::vector<uint32_t> mesh1(n), local1(n);
    std::vector<uint8_t> any1(n), vis1(ns);
    for (size_t i = 0; i < n; ++i) {
        const rt_ray &r = rays[i];
        const Raycaster::Hit h = rc.intersects({r.ox, r.oy, r.oz}, {r.dx, r.dy, r.dz}, r.tmin, r.tmax);
        t1[i] = h.dist; u1[i] = h.u; v1[i] = h.v;
        mesh1[i] = h.hit ? uint32_t(h.meshId) : RT_NO_HIT;
        local1[i] = h.hit ? uint32_t(h.localId) : RT_NO_HIT;
        any1[i] = rc.intersectsAny({r.ox, r.oy, r.oz}, {r.dx, r.dy, r.dz}, r.tmin, r.tmax) ? 1 : 0;
    }
    for (size_t i = 0; i < ns; ++i) {
        const float *s = &segs[6 * i];
        vis1[i] = rc.visible({s[0], s[1], s[2]}, {s[3], s[4], s[5]}) ? 1 : 0;
    }
    // All at once.
    std::vector<rt_hit> hits(n);
    std::vector<uint32_t> meshb(n), localb(n);
    std::vector<uint8_t> anyb(n);
    if (rc.intersects(rays.data(), n, hits.data(), meshb.data(), localb.data()) != RT_OK) return 5;
    if (rc.intersectsAny(rays.data(), n, anyb.data()) != RT_OK) return 6;
    save(dir, "t1.bin", t1); save(dir, "u1.bin", u1); save(dir, "v1.bin", v1);
    save(dir, "mesh1.bin", mesh1); save(dir, "local1.bin", local1);
    save(dir, "any1.bin", any1); save(dir, "vis1.bin", vis1);
    save(dir, "hits.bin", hits); save(dir, "meshb.bin", meshb); save(dir, "localb.bin", localb);
    save(dir, "anyb.bin", anyb);
    std::printf("ok %zu rays %zu segments\n", n, ns);
    return 0;
}
"""


def test_cpp_raycaster_class_matches_reference_golden(cuda_lib, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from rendu_gb300 import build

    lib = build.build()
    g = load_golden("raycaster_small.npz")
    meshes = golden_meshes(g)
    for k, (pos, idx, m) in enumerate(meshes):
        np.ascontiguousarray(pos, np.float32).tofile(tmp_path / f"pos{k}.bin")
        np.ascontiguousarray(idx, np.uint32).tofile(tmp_path / f"idx{k}.bin")
        model = np.eye(4, dtype=np.float32) if m is None else np.asarray(m, np.float32)
        np.ascontiguousarray(model.T).reshape(16).tofile(tmp_path / f"model{k}.bin")  # column-major
    n = 3000  # the one-by-one calls cost a device round trip each
    rays = np.ascontiguousarray(g["rays"][:n], np.float32)
    rays.tofile(tmp_path / "rays.bin")
    np.ascontiguousarray(g["segs"], np.float32).tofile(tmp_path / "segs.bin")
    src = tmp_path / "raycaster_binding.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "raycaster_binding"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", str(src),
                    "-o", str(exe), f"-L{libdir}", "-lrendu_gb300", f"-Wl,-rpath,{libdir}"], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe), str(tmp_path), str(len(meshes))], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)

    def rd(name, dt):
        return np.fromfile(tmp_path / name, dt)

    prim = g["hit_prim"][:n]
    hit = prim != 0xFFFFFFFF
    offs = np.cumsum([0] + [len(i) // 3 for _, i, _ in meshes])
    want_mesh = np.where(hit, np.searchsorted(offs, prim, side="right") - 1, 0xFFFFFFFF).astype(np.uint32)
    want_local = np.where(hit, 3 * (prim - offs[np.minimum(want_mesh, len(meshes) - 1)]), 0xFFFFFFFF).astype(np.uint32)
    # one by one
    t1 = rd("t1.bin", np.float32)
    assert np.array_equal(t1[hit].view(np.uint32), g["hit_t"][:n][hit].view(np.uint32))
    assert np.array_equal(rd("u1.bin", np.float32)[hit].view(np.uint32), g["hit_u"][:n][hit].view(np.uint32))
    assert np.array_equal(rd("v1.bin", np.float32)[hit].view(np.uint32), g["hit_v"][:n][hit].view(np.uint32))
    assert np.array_equal(rd("mesh1.bin", np.uint32), want_mesh)
    assert np.array_equal(rd("local1.bin", np.uint32), want_local)
    assert np.array_equal(rd("any1.bin", np.uint8), g["any"][:n])
    assert np.array_equal(rd("vis1.bin", np.uint8), g["visible"])
    # batched
    hits = rd("hits.bin", np.uint32).reshape(-1, 4)
    assert np.array_equal(hits[:, 3], prim)
    assert np.array_equal(hits[hit, 0], g["hit_t"][:n][hit].view(np.uint32))
    assert np.array_equal(rd("meshb.bin", np.uint32), want_mesh)
    assert np.array_equal(rd("localb.bin", np.uint32), want_local)
    assert np.array_equal(rd("anyb.bin", np.uint8), g["any"][:n])
