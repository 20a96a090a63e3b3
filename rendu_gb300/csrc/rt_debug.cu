// Hierarchy inspection for debugging and display: the geometry behind the reference's
// RaycasterVisualisation (src/engine/raycaster/RaycasterVisualisation.cpp:9-157 of
// kosua20/Rendu) -- the boxes of every node with its depth (getAllLevels), and the boxes a
// given ray enters with its closest hit (getRayLevels). The hierarchy shown is this
// library's own (a 4-wide LBVH, see rt_build.cu), copied back to the host; the ray walk
// is a host restatement of the device traversal (rt_traverse.cuh): same nearest-first
// order, same fused slab test, same Moller-Trumbore arithmetic, so its hit equals
// rt_intersect's. Host code.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "rt_context.hpp"

namespace {

using rgb::BvhNode;
using rgb::BvhTri;
using rgb::f3;

struct HostHierarchy {
    std::vector<BvhNode> nodes;
    std::vector<BvhTri> tris;
};

int fetch(const rt_ctx *ctx, HostHierarchy &h, bool with_tris) {
    if (!ctx->built || ctx->dirty) {
        rgb::set_error("the hierarchy is not built (call rt_update_hierarchy)");
        return RT_ERR_STATE;
    }
    RT_CUDA_TRY(cudaSetDevice(ctx->device));
    h.nodes.resize(ctx->n_inner);
    if (ctx->n_inner)
        RT_CUDA_TRY(cudaMemcpy(h.nodes.data(), ctx->d_nodes.ptr, ctx->n_inner * sizeof(BvhNode), cudaMemcpyDeviceToHost));
    if (with_tris) {
        h.tris.resize(ctx->n_tris);
        if (ctx->n_tris)
            RT_CUDA_TRY(cudaMemcpy(h.tris.data(), ctx->d_tris.ptr, ctx->n_tris * sizeof(BvhTri), cudaMemcpyDeviceToHost));
    }
    return RT_OK;
}

void child_box(const BvhNode &n, int c, float *b) {
    const float *lx = &n.lox.x, *hx = &n.hix.x, *ly = &n.loy.x, *hy = &n.hiy.x, *lz = &n.loz.x, *hz = &n.hiz.x;
    b[0] = lx[c], b[1] = ly[c], b[2] = lz[c], b[3] = hx[c], b[4] = hy[c], b[5] = hz[c];
}

struct Emit {
    float *boxes;
    int32_t *info;
    size_t cap, count = 0;
    void push(const float *b, int depth, int tris) {
        if (count < cap) {
            if (boxes) std::memcpy(boxes + 6 * count, b, 6 * sizeof(float));
            if (info) info[2 * count] = depth, info[2 * count + 1] = tris;
        }
        ++count;
    }
};

// Host copies of the device arithmetic (rt_traverse.cuh): IEEE single precision with no
// contraction, fused multiply-add only where the device uses fmaf.
struct HostRay {
    f3 o, d, inv, oinv;
    float tmin, tmax;
    bool valid;
};

inline float hdot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline f3 hcross(f3 x, f3 y) { return f3{x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
inline f3 hsub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }

HostRay host_ray(const rt_ray &in) {
    HostRay s;
    s.o = f3{in.ox, in.oy, in.oz};
    s.tmin = in.tmin;
    s.tmax = in.tmax;
    const f3 v{in.dx, in.dy, in.dz};
    const float k = 1.0f / std::sqrt(hdot(v, v));
    s.d = f3{v.x * k, v.y * k, v.z * k};
    auto floor20 = [](float x) { return std::fabs(x) < 1e-20f ? std::copysign(1e-20f, x) : x; };
    s.inv = f3{1.0f / floor20(s.d.x), 1.0f / floor20(s.d.y), 1.0f / floor20(s.d.z)};
    s.oinv = f3{s.o.x * s.inv.x, s.o.y * s.inv.y, s.o.z * s.inv.z};
    s.valid = (s.d.x == s.d.x) && (s.d.y == s.d.y) && (s.d.z == s.d.z) && (s.tmin < s.tmax);
    return s;
}

float host_slab(const HostRay &r, const float *b, float lo_t, float hi_t) {
    const float tx0 = std::fma(b[0], r.inv.x, -r.oinv.x), tx1 = std::fma(b[3], r.inv.x, -r.oinv.x);
    const float ty0 = std::fma(b[1], r.inv.y, -r.oinv.y), ty1 = std::fma(b[4], r.inv.y, -r.oinv.y);
    const float tz0 = std::fma(b[2], r.inv.z, -r.oinv.z), tz1 = std::fma(b[5], r.inv.z, -r.oinv.z);
    const float tn = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)), std::fmax(std::fmin(tz0, tz1), lo_t));
    const float tf = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmin(std::fmax(tz0, tz1), hi_t));
    return tn <= tf ? tn : INFINITY;
}

bool host_mt(const HostRay &r, const BvhTri &tri, float &t, float &u, float &v) {
    const f3 v01{tri.e1.x, tri.e1.y, tri.e1.z};
    const f3 v02{tri.e2.x, tri.e2.y, tri.e2.z};
    const f3 p = hcross(r.d, v02);
    const float det = hdot(v01, p);
    if (std::fabs(det) < FLT_EPSILON) return false;
    const float inv_det = 1.0f / det;
    const f3 q = hsub(r.o, f3{tri.v0.x, tri.v0.y, tri.v0.z});
    u = inv_det * hdot(q, p);
    if (u < 0.0f || u > 1.0f) return false;
    const f3 rr = hcross(q, v01);
    v = inv_det * hdot(r.d, rr);
    if (v < 0.0f || u + v > 1.0f) return false;
    t = inv_det * hdot(v02, rr);
    return true;
}

}  // namespace

extern "C" {

int rt_hierarchy_boxes(const rt_ctx *ctx, float *boxes, int32_t *info, size_t capacity, size_t *count) {
    rgb::clear_error();
    if (!ctx || !count) {
        rgb::set_error("null argument");
        return RT_ERR_ARG;
    }
    HostHierarchy h;
    const int st = fetch(ctx, h, false);
    if (st != RT_OK) return st;
    Emit e{boxes, info, capacity};
    if (ctx->n_tris == 0) {
        *count = 0;
        return RT_OK;
    }
    e.push(ctx->root_box, 0, 0);
    // breadth first over inner nodes: (node, depth of its children)
    std::vector<std::pair<int, int>> level{{0, 1}}, next;
    while (!level.empty()) {
        next.clear();
        for (const auto &nd : level) {
            if (nd.first < 0 || (size_t)nd.first >= h.nodes.size()) {
                rgb::set_error("corrupt hierarchy");
                return RT_ERR_STATE;
            }
            const BvhNode &n = h.nodes[nd.first];
            const int *child = &n.child.x, *cnt = &n.count.x;
            for (int c = 0; c < 4; ++c) {
                if (cnt[c] < 0) continue;
                float b[6];
                child_box(n, c, b);
                e.push(b, nd.second, cnt[c]);
                if (cnt[c] == 0) next.push_back({child[c], nd.second + 1});
            }
        }
        level.swap(next);
    }
    *count = e.count;
    return RT_OK;
}

int rt_ray_levels(const rt_ctx *ctx, const rt_ray *ray, float *boxes, int32_t *info, size_t capacity, size_t *count,
                  rt_hit *hit) {
    rgb::clear_error();
    if (!ctx || !ray || !count || !hit) {
        rgb::set_error("null argument");
        return RT_ERR_ARG;
    }
    HostHierarchy h;
    const int st = fetch(ctx, h, true);
    if (st != RT_OK) return st;
    Emit e{boxes, info, capacity};
    *hit = rt_hit{FLT_MAX, 0.0f, 0.0f, RT_NO_HIT};
    const HostRay r = host_ray(*ray);
    if (!r.valid || ctx->n_tris == 0) {
        *count = 0;
        return RT_OK;
    }
    if (host_slab(r, ctx->root_box, r.tmin, r.tmax) != INFINITY) e.push(ctx->root_box, 0, 0);
    struct Entry {
        int node, depth;
        float near;
    };
    std::vector<Entry> stack;
    float cur_max = r.tmax;
    bool found = false;
    int node = 0, depth = 1;
    for (;;) {
        if (node < 0 || (size_t)node >= h.nodes.size()) {
            rgb::set_error("corrupt hierarchy");
            return RT_ERR_STATE;
        }
        const BvhNode &n = h.nodes[node];
        const int *child = &n.child.x, *cnt = &n.count.x;
        float k[4];
        int id[4];
        for (int c = 0; c < 4; ++c) {
            float b[6];
            child_box(n, c, b);
            k[c] = cnt[c] >= 0 ? host_slab(r, b, r.tmin, cur_max) : INFINITY;
            id[c] = child[c];
            if (k[c] != INFINITY) e.push(b, depth, cnt[c]);
        }
        for (int c = 0; c < 4; ++c) {  // leaves first, as on the device
            if (cnt[c] <= 0 || k[c] == INFINITY) continue;
            for (int q = 0; q < cnt[c]; ++q) {
                const size_t ti = (size_t)id[c] + q;
                if (ti >= h.tris.size()) {
                    rgb::set_error("corrupt hierarchy");
                    return RT_ERR_STATE;
                }
                const BvhTri &tri = h.tris[ti];
                float tt, u, v;
                if (!host_mt(r, tri, tt, u, v) || !(tt > r.tmin)) continue;
                uint32_t prim;
                std::memcpy(&prim, &tri.v0.w, 4);
                if (tt < cur_max || (found && tt == cur_max && prim < hit->prim)) {
                    found = true;
                    *hit = rt_hit{tt, u, v, prim};
                    cur_max = tt;
                }
            }
            k[c] = INFINITY;
        }
        for (int c = 0; c < 4; ++c)
            if (cnt[c] != 0 || !(k[c] <= cur_max)) k[c] = INFINITY;
        int order[4] = {0, 1, 2, 3};
        for (int a = 1; a < 4; ++a)  // nearest first (stable for equal distances)
            for (int b = a; b > 0 && k[order[b]] < k[order[b - 1]]; --b) std::swap(order[b], order[b - 1]);
        if (k[order[0]] != INFINITY) {
            for (int j = 3; j >= 1; --j)
                if (k[order[j]] != INFINITY) stack.push_back({id[order[j]], depth + 1, k[order[j]]});
            node = id[order[0]];
            depth = depth + 1;
            continue;
        }
        bool more = false;
        while (!stack.empty()) {
            const Entry top = stack.back();
            stack.pop_back();
            if (top.near <= cur_max) {
                node = top.node;
                depth = top.depth;
                more = true;
                break;
            }
        }
        if (!more) break;
    }
    if (!found) *hit = rt_hit{FLT_MAX, 0.0f, 0.0f, RT_NO_HIT};
    *count = e.count;
    return RT_OK;
}

}  // extern "C"
