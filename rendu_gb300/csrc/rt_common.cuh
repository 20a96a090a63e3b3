// Shared device helpers for the sm_103a raycaster and path tracer.
//
// Exactness contract: the ray set-up and the ray/triangle test reproduce the reference's
// float arithmetic operation by operation (kosua20/Rendu, glm 0.9.9.7 operator order):
//   glm::dot(vec3)      = (a.x*b.x + a.y*b.y) + a.z*b.z     glm/detail/func_geometric.inl:48-55
//   glm::cross          = (x.y*y.z - y.y*x.z, ...)          glm/detail/func_geometric.inl:68-79
//   glm::normalize(v)   = v * (1 / sqrt(dot(v, v)))         func_geometric.inl:88, func_exponential.inl:136-139
//   mat4 * vec4         = (m0*x + m1*y) + (m2*z + m3*w)     glm/detail/type_mat4x4.inl:561-572
// Every such operation uses the round-to-nearest intrinsics (__fmul_rn, __fadd_rn,
// __fsub_rn, __fdiv_rn, __fsqrt_rn), which the compiler never contracts into FMAs, so
// these paths are exact regardless of -fmad. Everything else is free to use FMAs.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "rendu_gb300.h"

namespace rgb {

struct f3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }

// ---- exact (reference-order) vector arithmetic ------------------------------------------
__device__ __forceinline__ f3 xsub(f3 a, f3 b) { return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 xadd(f3 a, f3 b) { return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 xscale(f3 a, float s) { return f3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)}; }
__device__ __forceinline__ float xdot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 xcross(f3 x, f3 y) {
    return f3{__fsub_rn(__fmul_rn(x.y, y.z), __fmul_rn(y.y, x.z)), __fsub_rn(__fmul_rn(x.z, y.x), __fmul_rn(y.z, x.x)),
              __fsub_rn(__fmul_rn(x.x, y.y), __fmul_rn(y.x, x.y))};
}
__device__ __forceinline__ f3 xnormalize(f3 v) {
    const float s = __fdiv_rn(1.0f, __fsqrt_rn(xdot(v, v)));
    return xscale(v, s);
}
// glm::min / glm::max on scalars (func_common.inl:17-29): (y < x) ? y : x, (x < y) ? y : x.
__host__ __device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__host__ __device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }

// ---- ordinary (fast) vector arithmetic --------------------------------------------------
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator*(float s, f3 a) { return f3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator/(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ f3 &operator+=(f3 &a, f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__host__ __device__ __forceinline__ f3 &operator*=(f3 &a, f3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; return a; }
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross(f3 x, f3 y) {
    return f3{x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
__device__ __forceinline__ f3 normalize(f3 v) { return v * rsqrtf(dot(v, v)); }
__host__ __device__ __forceinline__ f3 fmin3(f3 a, f3 b) { return f3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
__host__ __device__ __forceinline__ f3 fmax3(f3 a, f3 b) { return f3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }

// ---- device data layout ------------------------------------------------------------------
// 4-wide node, 128 bytes (one L2 line): child boxes in structure-of-arrays form,
//   lox = (c0.lo.x, c1.lo.x, c2.lo.x, c3.lo.x), hix, loy, hiy, loz, hiz likewise;
//   child = inner node index, or the first triangle of a leaf (leaf order);
//   count = 0: inner node; > 0: leaf of `count` triangles; -1: empty slot (box at +inf).
struct __align__(16) BvhNode {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 child;
    int4 count;
};

// Triangle in leaf order, 48 bytes: v0 and the two edges v1 - v0, v2 - v0 (computed with
// the same single rounding the reference applies at query time, Raycaster.cpp:235-236),
// the global triangle id in v0.w's bits.
struct __align__(16) BvhTri {
    float4 v0;  // xyz, w = __uint_as_float(prim)
    float4 e1;  // xyz, w unused
    float4 e2;  // xyz, w unused
};

// Hierarchy of one job of a batch (the traversal picks it per ray).
struct JobBvh {
    const BvhNode *nodes;
    const BvhTri *tris;
    int empty;  // no triangles: every ray misses
    int pad;
};

// Device status word bits (set with atomicOr by kernels, read by the host).
enum : unsigned {
    RT_DEV_STACK_OVERFLOW = 1u,
    RT_DEV_QUEUE_OVERFLOW = 2u,
    RT_DEV_TIMEOUT = 4u,
};

constexpr int RT_LEAF_MAX = 8;  // maximum triangles in one leaf

}  // namespace rgb
