// Device-side BVH traversal shared by the raycaster entry points (rt_trace.cu) and the
// path tracer's queue kernels (pt_kernels.cu). Replaces the per-ray body of
// Raycaster::intersects / intersectsAny (Raycaster.cpp:144-224 of kosua20/Rendu).
//
//  * Ray set-up exactly as Ray::Ray (Intersection.cpp:3-5): d = normalize(dir),
//    invdir = 1 / d, with the reference's rounding.
//  * Box tests use a fused slab test (one FFMA per slab) with finite reciprocals. Boxes
//    were grown at build time so that this test is conservative; it decides only which
//    triangles are visited, never the answer.
//  * The per-triangle test is Moller-Trumbore with the reference's exact operation order,
//    rejection threshold |det| < FLT_EPSILON and inclusive/exclusive bounds
//    (Raycaster.cpp:232-262), so every (ray, triangle) pair is accepted or rejected with
//    the same t, u, v as on the CPU.
//  * Closest hit keeps the smallest t; at exactly equal t the smaller global triangle id.
//    Any hit stops at the first accepted triangle.
//  * The stack (node index + entry distance) is per thread; its capacity is a template
//    parameter chosen from the tree height measured at build time. Overflow is reported
//    through the status word, never by trapping.
#pragma once

#include "rt_common.cuh"

namespace rgb {

struct RayState {
    f3 o, d, inv, oinv;
    float tmin, tmax;
    bool valid;
};

__device__ __forceinline__ RayState make_ray_state(float4 r0, float4 r1) {
    RayState s;
    s.o = mk(r0.x, r0.y, r0.z);
    s.tmin = r0.w;
    s.tmax = r1.w;
    s.d = xnormalize(mk(r1.x, r1.y, r1.z));
    // The box test uses a reciprocal of the direction with components below 1e-20 in
    // magnitude replaced by +-1e-20: an infinite reciprocal would turn the fused slab test
    // into inf - inf = NaN for origins inside a slab. The exact direction still drives the
    // per-triangle test, so only the (conservative) culling sees the difference.
    const float ex = fabsf(s.d.x) < 1e-20f ? copysignf(1e-20f, s.d.x) : s.d.x;
    const float ey = fabsf(s.d.y) < 1e-20f ? copysignf(1e-20f, s.d.y) : s.d.y;
    const float ez = fabsf(s.d.z) < 1e-20f ? copysignf(1e-20f, s.d.z) : s.d.z;
    s.inv = mk(1.0f / ex, 1.0f / ey, 1.0f / ez);
    s.oinv = mk(s.o.x * s.inv.x, s.o.y * s.inv.y, s.o.z * s.inv.z);
    // A zero-length or non-finite direction never hits (the reference's comparisons with
    // NaN all fail); neither does an empty window.
    s.valid = (s.d.x == s.d.x) && (s.d.y == s.d.y) && (s.d.z == s.d.z) && (s.tmin < s.tmax);
    return s;
}

// Moller-Trumbore in the reference's operation order (Raycaster.cpp:232-262).
__device__ __forceinline__ bool mt_exact(const RayState &r, const float4 v0, const float4 e1, const float4 e2, float &t,
                                         float &u, float &v) {
    const f3 v01 = mk(e1.x, e1.y, e1.z);
    const f3 v02 = mk(e2.x, e2.y, e2.z);
    const f3 p = xcross(r.d, v02);
    const float det = xdot(v01, p);
    if (fabsf(det) < FLT_EPSILON) return false;
    const float invDet = __fdiv_rn(1.0f, det);
    const f3 q = xsub(r.o, mk(v0.x, v0.y, v0.z));
    u = __fmul_rn(invDet, xdot(q, p));
    if (u < 0.0f || u > 1.0f) return false;
    const f3 rr = xcross(q, v01);
    v = __fmul_rn(invDet, xdot(r.d, rr));
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
    t = __fmul_rn(invDet, xdot(v02, rr));
    return true;
}

// Slab test of one child box against the window [lo_t, hi_t]; the entry distance, or
// +inf when the box is missed.
__device__ __forceinline__ float slab(const RayState &r, float x0, float x1, float y0, float y1, float z0, float z1,
                                      float lo_t, float hi_t) {
    const float tx0 = fmaf(x0, r.inv.x, -r.oinv.x), tx1 = fmaf(x1, r.inv.x, -r.oinv.x);
    const float ty0 = fmaf(y0, r.inv.y, -r.oinv.y), ty1 = fmaf(y1, r.inv.y, -r.oinv.y);
    const float tz0 = fmaf(z0, r.inv.z, -r.oinv.z), tz1 = fmaf(z1, r.inv.z, -r.oinv.z);
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), lo_t));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), hi_t));
    return tn <= tf ? tn : INFINITY;
}

struct TraceResult {
    float t, u, v;
    uint32_t prim;
    bool found;
};

// Traverse the hierarchy (root = node 0). ANY: stop at the first accepted triangle.
template <bool ANY, bool COUNT, int STACK>
__device__ __forceinline__ TraceResult traverse(const BvhNode *__restrict__ nodes, const BvhTri *__restrict__ tris,
                                                const RayState &r, unsigned *__restrict__ status, uint32_t &nvis,
                                                uint32_t &ntri) {
    TraceResult res;
    res.t = FLT_MAX;
    res.u = 0.0f;
    res.v = 0.0f;
    res.prim = RT_NO_HIT;
    res.found = false;
    float cur_max = r.tmax;  // shrinks to the best distance (Raycaster.cpp:170)
    int stack_node[STACK];
    float stack_near[STACK];
    int sp = 0;
    int node = 0;
    while (true) {
        const float4 *np = reinterpret_cast<const float4 *>(nodes + node);
        const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
        const int4 d = __ldg(reinterpret_cast<const int4 *>(np + 3));
        if (COUNT) ++nvis;
        float t0 = slab(r, a.x, a.y, a.z, a.w, c.x, c.y, r.tmin, cur_max);
        float t1 = d.y >= 0 ? slab(r, b.x, b.y, b.z, b.w, c.z, c.w, r.tmin, cur_max) : INFINITY;
        // Leaves are tested as soon as their box is entered.
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const float ts = s ? t1 : t0;
            const int cnt = s ? d.w : d.z;
            if (cnt == 0 || ts == INFINITY) continue;
            const int first = s ? d.y : d.x;
            for (int k = 0; k < cnt; ++k) {
                const float4 *tp = reinterpret_cast<const float4 *>(tris + first + k);
                const float4 v0 = __ldg(tp), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
                if (COUNT) ++ntri;
                float t, u, v;
                if (!mt_exact(r, v0, e1, e2, t, u, v)) continue;
                if (!(t > r.tmin)) continue;
                const uint32_t prim = __float_as_uint(v0.w);
                if (ANY) {
                    if (t < cur_max) {
                        res.found = true;
                        res.t = t;
                        res.u = u;
                        res.v = v;
                        res.prim = prim;
                        break;
                    }
                    continue;
                }
                if (t < cur_max || (res.found && t == cur_max && prim < res.prim)) {
                    res.found = true;
                    res.t = t;
                    res.u = u;
                    res.v = v;
                    res.prim = prim;
                    cur_max = t;
                }
            }
            if (ANY && res.found) break;
            if (s) t1 = INFINITY;
            else t0 = INFINITY;
        }
        if (ANY && res.found) break;
        const bool h0 = t0 <= cur_max, h1 = t1 <= cur_max;
        if (h0 && h1) {
            const bool first0 = t0 <= t1;
            if (sp >= STACK) {
                atomicOr(status, RT_DEV_STACK_OVERFLOW);
                break;
            }
            stack_node[sp] = first0 ? d.y : d.x;
            stack_near[sp] = first0 ? t1 : t0;
            ++sp;
            node = first0 ? d.x : d.y;
            continue;
        }
        if (h0) {
            node = d.x;
            continue;
        }
        if (h1) {
            node = d.y;
            continue;
        }
        // Pop the next entry still within the (possibly shrunk) window.
        bool popped = false;
        while (sp > 0) {
            --sp;
            if (stack_near[sp] <= cur_max) {
                node = stack_node[sp];
                popped = true;
                break;
            }
        }
        if (!popped) break;
    }
    return res;
}

// ---- persistent traversal with per-lane ray refill ---------------------------------------
// One iteration = one node visit (two child box tests, leaf triangles of entered children,
// push/pop). A lane whose ray has finished takes the next unclaimed ray at the start of
// the following iteration (one atomic per warp per refill), so rays that stop at the root
// and rays that descend deep share warps without idling lanes.
struct TravState {
    int node, sp;
    float cur_max;
    TraceResult res;
};

__device__ __forceinline__ void trav_init(TravState &t, const RayState &r) {
    t.node = 0;
    t.sp = 0;
    t.cur_max = r.tmax;
    t.res.t = FLT_MAX;
    t.res.u = 0.0f;
    t.res.v = 0.0f;
    t.res.prim = RT_NO_HIT;
    t.res.found = false;
}

// Returns true when the ray is finished.
template <bool ANY, int STACK>
__device__ __forceinline__ bool trav_step(const BvhNode *__restrict__ nodes, const BvhTri *__restrict__ tris,
                                          const RayState &r, TravState &t, int *stack_node, float *stack_near,
                                          unsigned *__restrict__ status) {
    const float4 *np = reinterpret_cast<const float4 *>(nodes + t.node);
    const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
    const int4 d = __ldg(reinterpret_cast<const int4 *>(np + 3));
    float t0 = slab(r, a.x, a.y, a.z, a.w, c.x, c.y, r.tmin, t.cur_max);
    float t1 = d.y >= 0 ? slab(r, b.x, b.y, b.z, b.w, c.z, c.w, r.tmin, t.cur_max) : INFINITY;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const float ts = s ? t1 : t0;
        const int cnt = s ? d.w : d.z;
        if (cnt == 0 || ts == INFINITY) continue;
        const int first = s ? d.y : d.x;
        for (int k = 0; k < cnt; ++k) {
            const float4 *tp = reinterpret_cast<const float4 *>(tris + first + k);
            const float4 v0 = __ldg(tp), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
            float tt, u, v;
            if (!mt_exact(r, v0, e1, e2, tt, u, v)) continue;
            if (!(tt > r.tmin)) continue;
            const uint32_t prim = __float_as_uint(v0.w);
            if (ANY) {
                if (tt < t.cur_max) {
                    t.res.found = true;
                    t.res.t = tt;
                    t.res.u = u;
                    t.res.v = v;
                    t.res.prim = prim;
                    return true;
                }
                continue;
            }
            if (tt < t.cur_max || (t.res.found && tt == t.cur_max && prim < t.res.prim)) {
                t.res.found = true;
                t.res.t = tt;
                t.res.u = u;
                t.res.v = v;
                t.res.prim = prim;
                t.cur_max = tt;
            }
        }
        if (s) t1 = INFINITY;
        else t0 = INFINITY;
    }
    const bool h0 = t0 <= t.cur_max, h1 = t1 <= t.cur_max;
    if (h0 && h1) {
        const bool first0 = t0 <= t1;
        if (t.sp >= STACK) {
            atomicOr(status, RT_DEV_STACK_OVERFLOW);
            return true;
        }
        stack_node[t.sp] = first0 ? d.y : d.x;
        stack_near[t.sp] = first0 ? t1 : t0;
        ++t.sp;
        t.node = first0 ? d.x : d.y;
        return false;
    }
    if (h0) {
        t.node = d.x;
        return false;
    }
    if (h1) {
        t.node = d.y;
        return false;
    }
    while (t.sp > 0) {
        --t.sp;
        if (stack_near[t.sp] <= t.cur_max) {
            t.node = stack_node[t.sp];
            return false;
        }
    }
    return true;
}

}  // namespace rgb
