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

// ---- traversal state and one node visit -----------------------------------------------------
struct TravState {
    int node, sp;
    float cur_max;  // shrinks to the best distance (Raycaster.cpp:170)
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

__device__ __forceinline__ void cswap(float &ka, int &ia, float &kb, int &ib) {
    if (kb < ka) {
        const float k = ka;
        ka = kb;
        kb = k;
        const int i = ia;
        ia = ib;
        ib = i;
    }
}

// Visit node t.node of the 4-wide hierarchy: slab-test its children, test the triangles of
// entered leaves (updating the window), then continue with the nearest entered inner child
// and push the others far-to-near; pop when none was entered. Returns true when the ray is
// finished (stack empty, or ANY and a hit was found).
template <bool ANY, bool COUNT, int STACK>
__device__ __forceinline__ bool trav_step(const BvhNode *__restrict__ nodes, const BvhTri *__restrict__ tris,
                                          const RayState &r, TravState &t, int *stack_node, float *stack_near,
                                          unsigned *__restrict__ status, uint32_t &nvis, uint32_t &ntri) {
    const float4 *np = reinterpret_cast<const float4 *>(nodes + t.node);
    const float4 lox = __ldg(np), hix = __ldg(np + 1), loy = __ldg(np + 2), hiy = __ldg(np + 3);
    const float4 loz = __ldg(np + 4), hiz = __ldg(np + 5);
    const int4 ch = __ldg(reinterpret_cast<const int4 *>(np + 6));
    const int4 cn = __ldg(reinterpret_cast<const int4 *>(np + 7));
    if (COUNT) ++nvis;
    float k[4];
    int id[4];
    const int cc[4] = {cn.x, cn.y, cn.z, cn.w};
    id[0] = ch.x; id[1] = ch.y; id[2] = ch.z; id[3] = ch.w;
    k[0] = cc[0] >= 0 ? slab(r, lox.x, hix.x, loy.x, hiy.x, loz.x, hiz.x, r.tmin, t.cur_max) : INFINITY;
    k[1] = cc[1] >= 0 ? slab(r, lox.y, hix.y, loy.y, hiy.y, loz.y, hiz.y, r.tmin, t.cur_max) : INFINITY;
    k[2] = cc[2] >= 0 ? slab(r, lox.z, hix.z, loy.z, hiy.z, loz.z, hiz.z, r.tmin, t.cur_max) : INFINITY;
    k[3] = cc[3] >= 0 ? slab(r, lox.w, hix.w, loy.w, hiy.w, loz.w, hiz.w, r.tmin, t.cur_max) : INFINITY;
    // Leaves first: they can only shrink the window for the inner children.
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (cc[c] <= 0 || k[c] == INFINITY) continue;
        const int first = id[c];
        for (int q = 0; q < cc[c]; ++q) {
            const float4 *tp = reinterpret_cast<const float4 *>(tris + first + q);
            const float4 v0 = __ldg(tp), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
            if (COUNT) ++ntri;
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
        k[c] = INFINITY;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
        if (cc[c] != 0 || !(k[c] <= t.cur_max)) k[c] = INFINITY;
    // Sort the four (distance, child) pairs.
    cswap(k[0], id[0], k[1], id[1]);
    cswap(k[2], id[2], k[3], id[3]);
    cswap(k[0], id[0], k[2], id[2]);
    cswap(k[1], id[1], k[3], id[3]);
    cswap(k[1], id[1], k[2], id[2]);
    if (k[0] != INFINITY) {
#pragma unroll
        for (int j = 3; j >= 1; --j) {
            if (k[j] == INFINITY) continue;
            if (t.sp >= STACK) {
                atomicOr(status, RT_DEV_STACK_OVERFLOW);
                return true;
            }
            stack_node[t.sp] = id[j];
            stack_near[t.sp] = k[j];
            ++t.sp;
        }
        t.node = id[0];
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

// Whole traversal for one ray (root = node 0).
template <bool ANY, bool COUNT, int STACK>
__device__ __forceinline__ TraceResult traverse(const BvhNode *__restrict__ nodes, const BvhTri *__restrict__ tris,
                                                const RayState &r, unsigned *__restrict__ status, uint32_t &nvis,
                                                uint32_t &ntri) {
    int stack_node[STACK];
    float stack_near[STACK];
    TravState t;
    trav_init(t, r);
    while (!trav_step<ANY, COUNT, STACK>(nodes, tris, r, t, stack_node, stack_near, status, nvis, ntri)) {
    }
    return t.res;
}

}  // namespace rgb
