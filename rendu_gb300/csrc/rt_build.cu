// GPU hierarchy build: replaces Raycaster::updateHierarchy (Raycaster.cpp:54-142 of
// kosua20/Rendu) and the vertex/triangle set-up of Raycaster::addMesh (Raycaster.cpp:14-52).
//
// The reference builds a top-down binary tree on one CPU thread (mean-of-centroids split,
// leaves of 1-2 triangles, one root per mesh). Here the hierarchy is a linear BVH built in
// parallel over all meshes at once:
//   1. vertices transformed by their mesh's model matrix (exact glm operator order);
//   2. per-triangle boxes, edges and 63-bit Morton codes of the box centroids;
//   3. radix sort of (code, triangle) pairs;
//   4. a binary tree over the sorted leaves: Karras' radix tree (one thread per inner node)
//      for a single mesh, locally-ordered clustering (PLOC, below) for several meshes;
//   5. a bottom-up pass (one thread per leaf, atomics decide who climbs) that merges child
//      boxes, collapses every subtree of <= RT_LEAF_MAX triangles into one leaf where the
//      surface-area cost says a leaf is cheaper, and decides how each subtree splits into
//      the (at most four) slots of a 4-wide node;
//   6. emission of 64-byte nodes holding both children's boxes and of 48-byte triangles in
//      leaf order.
// Query answers do not depend on the tree shape (closest hit = smallest distance, exact
// per-triangle test), so the tree only decides speed.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "rt_context.hpp"

namespace rgb {
namespace {

struct MeshXform {
    uint64_t first_vertex;
    float m[16];
    int identity;
};

// Raycaster::addMesh vertex transform (Raycaster.cpp:22-26): glm::vec3(model * vec4(v, 1)).
__global__ void k_transform(const float *__restrict__ pin, uint64_t nv, const MeshXform *__restrict__ xf, int nm,
                            float *__restrict__ pout) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= nv) return;
    int lo = 0, hi = nm - 1;
    while (lo < hi) {  // last mesh whose first vertex <= i
        const int mid = (lo + hi + 1) >> 1;
        if (xf[mid].first_vertex <= i) lo = mid;
        else hi = mid - 1;
    }
    const float x = pin[3 * i], y = pin[3 * i + 1], z = pin[3 * i + 2];
    const MeshXform &t = xf[lo];
    if (t.identity) {
        pout[3 * i] = x;
        pout[3 * i + 1] = y;
        pout[3 * i + 2] = z;
        return;
    }
    const float *m = t.m;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a0 = __fadd_rn(__fmul_rn(m[0 + k], x), __fmul_rn(m[4 + k], y));
        const float a1 = __fadd_rn(__fmul_rn(m[8 + k], z), __fmul_rn(m[12 + k], 1.0f));
        pout[3 * i + k] = __fadd_rn(a0, a1);
    }
}

__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Triangle boxes (BoundingBox(v0,v1,v2), Bounds.cpp:12-15), centroid and coordinate bounds.
__global__ void k_tri_setup(const float *__restrict__ verts, const uint32_t *__restrict__ idx, uint64_t nt,
                            float4 *__restrict__ tlo, float4 *__restrict__ thi, unsigned *__restrict__ cb /*6 ord*/,
                            unsigned *__restrict__ absmax /*ord*/) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    float c[3] = {0, 0, 0}, am = 0.0f;
    bool valid = t < nt;
    if (valid) {
        const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        float lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = verts[3 * i0 + k], b = verts[3 * i1 + k], d = verts[3 * i2 + k];
            lo[k] = gmin(gmin(a, b), d);
            hi[k] = gmax(gmax(a, b), d);
            c[k] = 0.5f * (lo[k] + hi[k]);
            am = fmaxf(am, fmaxf(fabsf(lo[k]), fabsf(hi[k])));
        }
        tlo[t] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        thi[t] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    }
    // Block-reduce centroid bounds and the largest coordinate magnitude.
    __shared__ float s[7][32];
    float v[7];
    for (int k = 0; k < 3; ++k) {
        v[k] = valid ? c[k] : INFINITY;
        v[3 + k] = valid ? c[k] : -INFINITY;
    }
    v[6] = valid ? am : 0.0f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 3; ++k) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
        for (int k = 3; k < 7; ++k) v[k] = fmaxf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    }
    if (lane == 0)
        for (int k = 0; k < 7; ++k) s[k][warp] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < 7; ++k) v[k] = lane < nw ? s[k][lane] : (k < 3 ? INFINITY : (k < 6 ? -INFINITY : 0.0f));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            for (int k = 0; k < 3; ++k) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
            for (int k = 3; k < 7; ++k) v[k] = fmaxf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
        }
        if (lane == 0) {
            for (int k = 0; k < 3; ++k) atomicMin(&cb[k], f2ord(v[k]));
            for (int k = 3; k < 6; ++k) atomicMax(&cb[k], f2ord(v[k]));
            atomicMax(absmax, f2ord(v[6]));
        }
    }
}

__device__ __forceinline__ uint64_t spread21(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

// Morton code of the triangle box centroid, 21 bits an axis. The centroid bounds are scaled
// by their largest extent on every axis (a cube), not axis by axis: on a flat scene the
// per-axis scaling spends as many top-level splits on the thin axis as on the wide ones.
// Measured on the 2M-triangle instanced scene (a 200-object layer on a ground plane): the
// 1080p extended render 224.8 -> 214.1 ms; no change on the displaced sphere (a cube
// already). Adding 6 bits of triangle size to the key measured no further gain.
__global__ void k_morton(const float4 *__restrict__ tlo, const float4 *__restrict__ thi, uint64_t nt,
                         const unsigned *__restrict__ cb, uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const float4 lo = tlo[t], hi = thi[t];
    const float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    float ext = 0.0f;
    for (int k = 0; k < 3; ++k) ext = fmaxf(ext, ord2f(cb[3 + k]) - ord2f(cb[k]));
    uint64_t code = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float u = ext > 0.0f ? (c[k] - ord2f(cb[k])) / ext : 0.5f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        const uint64_t q = (uint64_t)fminf(u * 2097152.0f, 2097151.0f);
        code |= spread21(q) << (2 - k);
    }
    keys[t] = code;
    vals[t] = (uint32_t)t;
}

// Common-prefix length of sorted keys i and j; equal keys compare their indices.
__device__ __forceinline__ int delta(const uint64_t *__restrict__ k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    if (a != b) return __clzll(a ^ b);
    return 64 + __clz((unsigned)(i ^ j));
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d trees".
// Inner node i (0..n-2): children encoded as (index << 1) | is_leaf.
__global__ void k_karras(const uint64_t *__restrict__ keys, int64_t n, uint32_t *__restrict__ child,
                         uint32_t *__restrict__ parent_inner, uint32_t *__restrict__ parent_leaf,
                         uint32_t *__restrict__ range_first, uint32_t *__restrict__ range_last) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int64_t lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int64_t l = 0;
    for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t gamma = i + s * d + (d < 0 ? d : 0);
    const int64_t first = i < j ? i : j, last = i < j ? j : i;
    range_first[i] = (uint32_t)first;
    range_last[i] = (uint32_t)last;
    const bool left_leaf = first == gamma, right_leaf = last == gamma + 1;
    child[2 * i] = (uint32_t)(gamma << 1) | (left_leaf ? 1u : 0u);
    child[2 * i + 1] = (uint32_t)((gamma + 1) << 1) | (right_leaf ? 1u : 0u);
    if (left_leaf) parent_leaf[gamma] = (uint32_t)i;
    else parent_inner[gamma] = (uint32_t)i;
    if (right_leaf) parent_leaf[gamma + 1] = (uint32_t)i;
    else parent_inner[gamma + 1] = (uint32_t)i;
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float x = fmaxf(hi.x - lo.x, 0.0f), y = fmaxf(hi.y - lo.y, 0.0f), z = fmaxf(hi.z - lo.z, 0.0f);
    return x * y + y * z + z * x;
}

// RT_COLLAPSE_DP 1 (default): binary -> 4-wide by the surface-area-optimal slot assignment of
// the bottom-up pass; 0: open the largest-area inner child until four slots. Measured: 535k
// instead of 649k nodes on the 1.3M-triangle sphere, closest hit 1.359 -> 1.344 ms, any hit
// 1.172 -> 1.143 ms; the instanced 1080p render 190.2 -> 188.8 ms.
#ifndef RT_COLLAPSE_DP
#define RT_COLLAPSE_DP 1
#endif
constexpr float kCostInner = 1.2f;  // relative cost of one node visit (two box tests)
// Relative cost of one triangle test. A leaf's triangles are tested in a loop whose length
// varies from lane to lane, so on the GPU a triangle costs more than a node visit: with
// this weight nearly every leaf holds one triangle, which measured fastest (closest hit on
// 16M random rays into 1.3M triangles -6 %, the 2M-triangle path-traced scene -3 %,
// against a weight of 1).
// With the optimal 4-wide collapse, weights 2, 4 and 6 measured no better than 3.
#ifndef RT_COST_TRI
#define RT_COST_TRI 3.0f
#endif
constexpr float kCostTri = RT_COST_TRI;

// Gather sorted triangle boxes (inflated by eps, making the traversal's box tests
// conservative) and write leaf-order triangles.
__global__ void k_leaves(const uint32_t *__restrict__ order, uint64_t nt, const float4 *__restrict__ tlo,
                         const float4 *__restrict__ thi, const float *__restrict__ verts,
                         const uint32_t *__restrict__ idx, float eps, float4 *__restrict__ slo,
                         float4 *__restrict__ shi, BvhTri *__restrict__ tris) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const uint32_t t = order[k];
    float4 lo = tlo[t], hi = thi[t];
    lo.x -= eps; lo.y -= eps; lo.z -= eps;
    hi.x += eps; hi.y += eps; hi.z += eps;
    slo[k] = lo;
    shi[k] = hi;
    const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
    const float ax = verts[3 * i0], ay = verts[3 * i0 + 1], az = verts[3 * i0 + 2];
    BvhTri tr;
    tr.v0 = make_float4(ax, ay, az, __uint_as_float(t));
    tr.e1 = make_float4(__fsub_rn(verts[3 * i1], ax), __fsub_rn(verts[3 * i1 + 1], ay), __fsub_rn(verts[3 * i1 + 2], az), 0.0f);
    tr.e2 = make_float4(__fsub_rn(verts[3 * i2], ax), __fsub_rn(verts[3 * i2 + 1], ay), __fsub_rn(verts[3 * i2 + 2], az), 0.0f);
    tris[k] = tr;
}

// Bottom-up: one thread per leaf climbs while it is the second child to arrive.
__global__ void k_bottom_up(uint64_t nt, const uint32_t *__restrict__ child, const uint32_t *__restrict__ parent_inner,
                            const uint32_t *__restrict__ parent_leaf, const uint32_t *__restrict__ range_first,
                            const uint32_t *__restrict__ range_last, const float4 *__restrict__ slo,
                            const float4 *__restrict__ shi, float4 *__restrict__ ilo, float4 *__restrict__ ihi,
                            float *__restrict__ cost, uint8_t *__restrict__ collapse, int *__restrict__ height,
                            unsigned *__restrict__ arrivals, float4 *__restrict__ cset, uchar4 *__restrict__ dec) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= nt) return;
    uint32_t node = parent_leaf[k];
    // A Karras tree over 64-bit keys with 32-bit index tie-breaks is at most 96 levels deep;
    // a clustered tree has no such bound, so the climb allows far more.
    for (int level = 0; level < 4096; ++level) {
        if (node >= nt - 1) return;
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0u) return;  // first arrival stops
        __threadfence();
        float4 lo[2], hi[2];
        float c[2];
        int h[2];
        float cs[2][4];  // cost of the child as at most k slots of the enclosing 4-wide node
        for (int s = 0; s < 2; ++s) {
            const uint32_t ch = child[2 * node + s];
            const uint32_t id = ch >> 1;
            if (ch & 1u) {
                lo[s] = slo[id];
                hi[s] = shi[id];
                c[s] = kCostTri * half_area(lo[s], hi[s]);
                h[s] = 0;
                for (int k = 0; k < 4; ++k) cs[s][k] = c[s];
            } else {
                lo[s] = __ldcg(&ilo[id]);
                hi[s] = __ldcg(&ihi[id]);
                c[s] = __ldcg(&cost[id]);
                h[s] = __ldcg(&height[id]);
                const float4 v = __ldcg(&cset[id]);
                cs[s][0] = v.x;
                cs[s][1] = v.y;
                cs[s][2] = v.z;
                cs[s][3] = v.w;
            }
        }
        const float4 blo = make_float4(fminf(lo[0].x, lo[1].x), fminf(lo[0].y, lo[1].y), fminf(lo[0].z, lo[1].z), 0.0f);
        const float4 bhi = make_float4(fmaxf(hi[0].x, hi[1].x), fmaxf(hi[0].y, hi[1].y), fmaxf(hi[0].z, hi[1].z), 0.0f);
        const float a = half_area(blo, bhi);
        const uint32_t count = range_last[node] - range_first[node] + 1;
        const float c_inner = kCostInner * a + c[0] + c[1];
        const float c_leaf = kCostTri * a * (float)count;
        const bool col = count <= (uint32_t)RT_LEAF_MAX && c_leaf <= c_inner;
        ilo[node] = blo;
        ihi[node] = bhi;
        cost[node] = col ? c_leaf : c_inner;
        collapse[node] = col ? 1 : 0;
        // Surface-area-optimal conversion to 4-wide nodes (dynamic programming over the number
        // of slots a subtree may take in its parent): comb[k] = the children as k slots in all,
        // best split k1 + (k - k1); the node as one slot is a 4-wide node over comb[4] (or its
        // leaf); as k > 1 slots it is the better of k - 1 slots and its children as k slots.
        float comb[5];
        uint8_t split[5] = {0, 0, 0, 0, 0};
        for (int k = 2; k <= 4; ++k) {
            comb[k] = INFINITY;
            for (int k1 = 1; k1 < k; ++k1) {
                const float v = cs[0][k1 - 1] + cs[1][k - k1 - 1];
                if (v < comb[k]) {
                    comb[k] = v;
                    split[k] = (uint8_t)k1;
                }
            }
        }
        float w[4];
        uint8_t d[4] = {0, 0, 0, 0};
        w[0] = col ? c_leaf : kCostInner * a + comb[4];
        for (int k = 2; k <= 4; ++k) {
            if (!col && comb[k] < w[k - 2]) {
                w[k - 1] = comb[k];
                d[k - 1] = split[k];
            } else {
                w[k - 1] = w[k - 2];
                d[k - 1] = 0;  // as k - 1 slots
            }
        }
        cset[node] = make_float4(w[0], w[1], w[2], w[3]);
        dec[node] = make_uchar4(split[4], d[1], d[2], d[3]);
        height[node] = col ? 0 : 1 + max(h[0], h[1]);
        if (node == 0) return;
        node = parent_inner[node];
    }
}

// ---- PLOC: parallel locally-ordered clustering (Meister & Bittner 2018) ----------------------
// The alternative to Karras' radix tree for step 4. Clusters start as the leaves in Morton
// order. Each round, every cluster finds its nearest neighbour within kPlocRadius positions
// (smallest half area of the union box); mutual pairs merge into a new inner node at the
// lower position, and the array is compacted. Ties are broken by the smaller index, which for
// a fixed cluster orders its pairs exactly like the pair key (area, min index, max index):
// the globally closest pair is always mutual, so every round merges at least one pair. Inner
// nodes are numbered in creation order (the root last); children always precede their
// parent. The leaves are then renumbered in depth-first order, so that every subtree's
// leaves are contiguous as the collapse into 4-wide nodes needs.
// RT_PLOC: 1 = always cluster, 0 = always the radix tree, 2 (default) = cluster when the
// context holds more than one mesh. Measured (1080p extended render of the 205-object
// instanced scene; 16M random rays into the 1.3M-triangle displaced sphere): clustering with
// radius 4 renders 214 -> 190 ms (SAH cost 77.4 -> 72.7), while on the single surface the
// radix tree's spatial-median splits stay 2 % faster for closest hits (1.38 vs 1.41 ms).
// Radii 6-64 measured no better than 4.
#ifndef RT_PLOC
#define RT_PLOC 2
#endif
#ifndef RT_PLOC_RADIUS
#define RT_PLOC_RADIUS 4
#endif
constexpr int kPlocRadius = RT_PLOC_RADIUS;
constexpr int kPlocBlock = 256;
constexpr size_t kPlocMaxRounds = 512;  // typical builds take about 50 rounds

__global__ void k_ploc_nn(const float4 *__restrict__ lo, const float4 *__restrict__ hi, uint32_t n,
                          uint32_t *__restrict__ nn) {
    __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
    const long b0 = (long)blockIdx.x * kPlocBlock;
    for (int t = threadIdx.x; t < kPlocBlock + 2 * kPlocRadius; t += kPlocBlock) {
        const long g = b0 - kPlocRadius + t;
        if (g >= 0 && g < (long)n) {
            slo[t] = lo[g];
            shi[t] = hi[g];
        }
    }
    __syncthreads();
    const long i = b0 + threadIdx.x;
    if (i >= (long)n) return;
    const float4 a = slo[threadIdx.x + kPlocRadius], b = shi[threadIdx.x + kPlocRadius];
    float best = INFINITY;
    uint32_t bj = (uint32_t)i;
    for (int o = -kPlocRadius; o <= kPlocRadius; ++o) {
        const long j = i + o;
        if (o == 0 || j < 0 || j >= (long)n) continue;
        const float4 c = slo[threadIdx.x + kPlocRadius + o], d = shi[threadIdx.x + kPlocRadius + o];
        const float area = half_area(make_float4(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z), 0.0f),
                                     make_float4(fmaxf(b.x, d.x), fmaxf(b.y, d.y), fmaxf(b.z, d.z), 0.0f));
        if (area < best) {
            best = area;
            bj = (uint32_t)j;
        }
    }
    nn[i] = bj;
}

__global__ void k_ploc_flags(const uint32_t *__restrict__ nn, uint32_t n, uint32_t *__restrict__ merge,
                             uint32_t *__restrict__ alive) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = nn[i];
    const bool mutual = j != i && j < n && nn[j] == i;
    merge[i] = mutual && i < j ? 1u : 0u;
    alive[i] = mutual && i > j ? 0u : 1u;
}

__global__ void k_ploc_compact(const uint32_t *__restrict__ node, const float4 *__restrict__ lo,
                               const float4 *__restrict__ hi, const uint32_t *__restrict__ cnt,
                               const uint32_t *__restrict__ nn, const uint32_t *__restrict__ merge,
                               const uint32_t *__restrict__ alive, const uint32_t *__restrict__ moff,
                               const uint32_t *__restrict__ apos, uint32_t n, uint32_t inner_base, uint32_t ni,
                               uint32_t *__restrict__ child, uint32_t *__restrict__ icount,
                               uint32_t *__restrict__ node2, float4 *__restrict__ lo2, float4 *__restrict__ hi2,
                               uint32_t *__restrict__ cnt2, unsigned *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !alive[i]) return;
    const uint32_t p = apos[i];
    if (p >= n) {
        atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
        return;
    }
    if (merge[i]) {
        const uint32_t j = nn[i];
        const uint32_t id = inner_base + moff[i];
        if (id >= ni || j >= n) {
            atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
            return;
        }
        child[2 * id] = node[i];
        child[2 * id + 1] = node[j];
        const uint32_t c = cnt[i] + cnt[j];
        icount[id] = c;
        const float4 a = lo[i], b = hi[i], e = lo[j], f = hi[j];
        node2[p] = id << 1;
        lo2[p] = make_float4(fminf(a.x, e.x), fminf(a.y, e.y), fminf(a.z, e.z), 0.0f);
        hi2[p] = make_float4(fmaxf(b.x, f.x), fmaxf(b.y, f.y), fmaxf(b.z, f.z), 0.0f);
        cnt2[p] = c;
    } else {
        node2[p] = node[i];
        lo2[p] = lo[i];
        hi2[p] = hi[i];
        cnt2[p] = cnt[i];
    }
}

__global__ void k_ploc_init(uint64_t nt, const float4 *__restrict__ slo, const float4 *__restrict__ shi,
                            uint32_t *__restrict__ node, float4 *__restrict__ lo, float4 *__restrict__ hi,
                            uint32_t *__restrict__ cnt) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= nt) return;
    node[k] = ((uint32_t)k << 1) | 1u;
    lo[k] = slo[k];
    hi[k] = shi[k];
    cnt[k] = 1u;
}

// First leaf position of each subtree, top-down one creation round at a time (latest round
// first: a node's parent is always of a later round). Leaves get their position in the
// depth-first leaf order, in which every subtree's leaves are contiguous.
__global__ void k_ploc_topdown(uint32_t id0, uint32_t count, uint32_t ni, uint64_t nt, const uint32_t *__restrict__ child,
                               const uint32_t *__restrict__ icount, uint32_t *__restrict__ ifirst,
                               uint32_t *__restrict__ lpos, unsigned *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t id = id0 + i;
    if (id >= ni) return;
    uint32_t f = ifirst[id];
    for (int s = 0; s < 2; ++s) {
        const uint32_t c = child[2 * id + s];
        const uint32_t x = c >> 1;
        if (c & 1u) {
            if (x >= nt || f >= nt) {
                atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
                return;
            }
            lpos[x] = f;
            f += 1;
        } else {
            if (x >= ni) {
                atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
                return;
            }
            ifirst[x] = f;
            f += icount[x];
        }
    }
}

// The tree in the layout the bottom-up pass and the collapse read: inner node ids reversed
// (root = 0), leaves renumbered to their depth-first positions, parents and leaf ranges.
__global__ void k_ploc_final(uint32_t ni, uint64_t nt, const uint32_t *__restrict__ child,
                             const uint32_t *__restrict__ icount, const uint32_t *__restrict__ ifirst,
                             const uint32_t *__restrict__ lpos, uint32_t *__restrict__ child_out,
                             uint32_t *__restrict__ pin, uint32_t *__restrict__ pleaf, uint32_t *__restrict__ rf,
                             uint32_t *__restrict__ rl, unsigned *__restrict__ status) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ni) return;
    const uint32_t id2 = ni - 1 - id;
    for (int s = 0; s < 2; ++s) {
        const uint32_t c = child[2 * id + s];
        const uint32_t x = c >> 1;
        if (c & 1u) {
            const uint32_t k2 = x < nt ? lpos[x] : 0xFFFFFFFFu;
            if (k2 >= nt) {
                atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
                return;
            }
            child_out[2 * id2 + s] = (k2 << 1) | 1u;
            pleaf[k2] = id2;
        } else {
            if (x >= ni) {
                atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
                return;
            }
            const uint32_t c2 = ni - 1 - x;
            child_out[2 * id2 + s] = c2 << 1;
            pin[c2] = id2;
        }
    }
    rf[id2] = ifirst[id];
    rl[id2] = ifirst[id] + icount[id] - 1;
}

__global__ void k_scatter_order(const uint32_t *__restrict__ order, const uint32_t *__restrict__ lpos, uint64_t nt,
                                uint32_t *__restrict__ order2) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const uint32_t p = lpos[k];
    if (p < nt) order2[p] = order[k];
}

__device__ __forceinline__ void set_slot(BvhNode &nd, int c, float4 lo, float4 hi, int child, int count) {
    float *lx = &nd.lox.x, *hx = &nd.hix.x, *ly = &nd.loy.x, *hy = &nd.hiy.x, *lz = &nd.loz.x, *hz = &nd.hiz.x;
    lx[c] = lo.x; hx[c] = hi.x; ly[c] = lo.y; hy[c] = hi.y; lz[c] = lo.z; hz[c] = hi.z;
    (&nd.child.x)[c] = child;
    (&nd.count.x)[c] = count;
}

__device__ __forceinline__ void set_empty(BvhNode &nd, int c) {
    const float4 inf = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
    set_slot(nd, c, inf, inf, -1, -1);
}

struct CollapseItem {
    uint32_t bin;   // inner node of the binary tree
    uint32_t slot;  // node of the 4-wide hierarchy it becomes
};

// One level of the binary -> 4-wide collapse: each queued binary inner node becomes a 4-wide
// node whose children are found by repeatedly opening the largest-area inner child (the
// surface-area-greedy rule); leaves and collapsed subtrees become leaf slots, remaining
// inner children get new slots and are queued for the next level.
__global__ void k_collapse(const CollapseItem *__restrict__ in, uint32_t n_in, CollapseItem *__restrict__ out,
                           uint32_t *__restrict__ n_out, uint32_t *__restrict__ node_count, uint32_t node_cap,
                           const uint32_t *__restrict__ child, const uint32_t *__restrict__ range_first,
                           const uint32_t *__restrict__ range_last, const float4 *__restrict__ slo,
                           const float4 *__restrict__ shi, const float4 *__restrict__ ilo,
                           const float4 *__restrict__ ihi, const uint8_t *__restrict__ collapse,
                           BvhNode *__restrict__ nodes, uint32_t *__restrict__ leaf_count,
                           unsigned *__restrict__ status, const uchar4 *__restrict__ dec) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_in) return;
    const CollapseItem item = in[i];
    uint32_t e[4];
    int ne = 0;
#if RT_COLLAPSE_DP
    // Slots of the 4-wide node: the binary children split k1 + (4 - k1) as the bottom-up
    // pass decided, each part expanded by its own decisions (a small explicit stack).
    {
        const uint8_t k1 = dec[item.bin].x;
        uint32_t st_ref[8];
        int st_k[8], sp = 0;
        st_ref[sp] = child[2 * item.bin + 1];
        st_k[sp++] = 4 - (k1 ? k1 : 2);
        st_ref[sp] = child[2 * item.bin];
        st_k[sp++] = k1 ? k1 : 2;
        while (sp > 0 && ne < 4) {
            const uint32_t ref = st_ref[--sp];
            int k = st_k[sp];
            if ((ref & 1u) || k <= 1 || collapse[ref >> 1]) {
                e[ne++] = ref;
                continue;
            }
            const uchar4 dd = dec[ref >> 1];
            const uint8_t dk[4] = {0, dd.y, dd.z, dd.w};
            while (k > 1 && dk[k - 1] == 0) --k;  // fewer slots are as good
            if (k <= 1 || sp + 2 > 8) {
                e[ne++] = ref;
                continue;
            }
            const int a = dk[k - 1];
            st_ref[sp] = child[2 * (ref >> 1) + 1];
            st_k[sp++] = k - a;
            st_ref[sp] = child[2 * (ref >> 1)];
            st_k[sp++] = a;
        }
        while (sp > 0 && ne < 4) e[ne++] = st_ref[--sp];  // cannot happen: slots never exceed 4
    }
#else
    ne = 2;
    e[0] = child[2 * item.bin];
    e[1] = child[2 * item.bin + 1];
    while (ne < 4) {
        int best = -1;
        float besta = -1.0f;
        for (int k = 0; k < ne; ++k) {
            if (e[k] & 1u) continue;
            const uint32_t id = e[k] >> 1;
            if (collapse[id]) continue;
            const float a = half_area(ilo[id], ihi[id]);
            if (a > besta) {
                besta = a;
                best = k;
            }
        }
        if (best < 0) break;
        const uint32_t b = e[best] >> 1;
        e[best] = child[2 * b];
        e[ne++] = child[2 * b + 1];
    }
#endif
    BvhNode nd;
    uint32_t leaves = 0;
    for (int c = 0; c < 4; ++c) {
        if (c >= ne) {
            set_empty(nd, c);
            continue;
        }
        const uint32_t id = e[c] >> 1;
        if (e[c] & 1u) {
            set_slot(nd, c, slo[id], shi[id], (int)id, 1);
            ++leaves;
        } else if (collapse[id]) {
            set_slot(nd, c, ilo[id], ihi[id], (int)range_first[id], (int)(range_last[id] - range_first[id] + 1));
            ++leaves;
        } else {
            const uint32_t slot = atomicAdd(node_count, 1u);
            if (slot >= node_cap) {  // cannot happen for a well-formed tree; never write out of bounds
                atomicOr(status, RT_DEV_QUEUE_OVERFLOW);
                set_empty(nd, c);
                continue;
            }
            set_slot(nd, c, ilo[id], ihi[id], (int)slot, 0);
            out[atomicAdd(n_out, 1u)] = CollapseItem{id, slot};
        }
    }
    nodes[item.slot] = nd;
    atomicAdd(leaf_count, leaves);
}

// Stack bound of the traversal, bottom-up one collapse level at a time (deepest first): a
// visit pushes at most (inner children - 1) entries and continues into one inner child, so
// need(node) = max(0, inner children - 1) + the largest need of its inner children bounds
// the stack depth of any walk below the node.
__global__ void k_stack_need(const BvhNode *__restrict__ nodes, uint32_t s0, uint32_t s1, uint32_t cap,
                             uint32_t *__restrict__ need) {
    const uint32_t slot = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s1 || slot >= cap) return;
    const BvhNode nd = nodes[slot];
    const int ch[4] = {nd.child.x, nd.child.y, nd.child.z, nd.child.w};
    const int cn[4] = {nd.count.x, nd.count.y, nd.count.z, nd.count.w};
    uint32_t inner = 0, deepest = 0;
    for (int c = 0; c < 4; ++c)
        if (cn[c] == 0 && ch[c] >= 0 && (uint32_t)ch[c] < cap) {
            ++inner;
            deepest = max(deepest, need[ch[c]]);
        }
    need[slot] = (inner > 0 ? inner - 1 : 0) + deepest;
}

// A root whose whole tree is one leaf (or a single triangle): slot 0 = the leaf.
__global__ void k_root_leaf(uint64_t nt, const float4 *__restrict__ slo, const float4 *__restrict__ shi,
                            BvhNode *__restrict__ nodes) {
    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0);
    for (uint64_t k = 0; k < nt; ++k) {
        const float4 a = slo[k], b = shi[k];
        lo = make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0);
        hi = make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0);
    }
    BvhNode nd;
    set_slot(nd, 0, lo, hi, 0, (int)nt);
    for (int c = 1; c < 4; ++c) set_empty(nd, c);
    nodes[0] = nd;
}

template <class T>
struct Scratch {
    T *p = nullptr;
    ~Scratch() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

}  // namespace

int build_hierarchy(rt_ctx *ctx) {
    cudaStream_t st = ctx->stream;
    const uint64_t nv = ctx->h_positions.size() / 3;
    const uint64_t nt = ctx->h_indices.size() / 3;
    ctx->n_tris = nt;
    RT_CUDA_TRY(cudaEventRecord(ctx->ev_a, st));

    // Vertices: upload and transform.
    Scratch<float> d_raw;
    Scratch<uint32_t> d_idx;
    Scratch<MeshXform> d_xf;
    RT_CUDA_TRY(d_raw.alloc(3 * nv));
    RT_CUDA_TRY(d_idx.alloc(3 * nt));
    std::vector<MeshXform> xf(ctx->meshes.size());
    for (size_t m = 0; m < ctx->meshes.size(); ++m) {
        xf[m].first_vertex = ctx->meshes[m].first_vertex;
        std::memcpy(xf[m].m, ctx->meshes[m].model, sizeof(xf[m].m));
        xf[m].identity = ctx->meshes[m].identity ? 1 : 0;
    }
    RT_CUDA_TRY(d_xf.alloc(xf.size()));
    if (ctx->d_verts.reserve(3 * nv * sizeof(float)) != RT_OK) return RT_ERR_OOM;
    if (nv) {
        RT_CUDA_TRY(cudaMemcpyAsync(d_raw.p, ctx->h_positions.data(), 3 * nv * sizeof(float), cudaMemcpyHostToDevice, st));
        RT_CUDA_TRY(cudaMemcpyAsync(d_xf.p, xf.data(), xf.size() * sizeof(MeshXform), cudaMemcpyHostToDevice, st));
        k_transform<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(d_raw.p, nv, d_xf.p, (int)xf.size(), ctx->d_verts.as<float>());
    }
    if (nt) RT_CUDA_TRY(cudaMemcpyAsync(d_idx.p, ctx->h_indices.data(), 3 * nt * sizeof(uint32_t), cudaMemcpyHostToDevice, st));

    if (ctx->d_nodes.reserve(sizeof(BvhNode) * (nt > 1 ? nt - 1 : 1)) != RT_OK) return RT_ERR_OOM;
    if (ctx->d_tris.reserve(sizeof(BvhTri) * (nt ? nt : 1)) != RT_OK) return RT_ERR_OOM;
    if (nt == 0) {
        ctx->n_inner = 0;
        ctx->n_leaves = 0;
        ctx->depth = 0;
        ctx->sah_cost = 0.0f;
        RT_CUDA_TRY(cudaEventRecord(ctx->ev_b, st));
        RT_CUDA_TRY(cudaEventSynchronize(ctx->ev_b));
        RT_CUDA_TRY(cudaEventElapsedTime(&ctx->build_ms, ctx->ev_a, ctx->ev_b));
        return RT_OK;
    }

    Scratch<float4> d_tlo, d_thi, d_slo, d_shi, d_ilo, d_ihi;
    Scratch<unsigned> d_cb;
    Scratch<uint64_t> d_keys, d_keys2;
    Scratch<uint32_t> d_vals, d_vals2;
    RT_CUDA_TRY(d_tlo.alloc(nt));
    RT_CUDA_TRY(d_thi.alloc(nt));
    RT_CUDA_TRY(d_cb.alloc(8));
    const unsigned cb_init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
    RT_CUDA_TRY(cudaMemcpyAsync(d_cb.p, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, st));
    const unsigned tb = (unsigned)((nt + 255) / 256);
    k_tri_setup<<<tb, 256, 0, st>>>(ctx->d_verts.as<float>(), d_idx.p, nt, d_tlo.p, d_thi.p, d_cb.p, d_cb.p + 6);
    RT_CUDA_TRY(d_keys.alloc(nt));
    RT_CUDA_TRY(d_keys2.alloc(nt));
    RT_CUDA_TRY(d_vals.alloc(nt));
    RT_CUDA_TRY(d_vals2.alloc(nt));
    k_morton<<<tb, 256, 0, st>>>(d_tlo.p, d_thi.p, nt, d_cb.p, d_keys.p, d_vals.p);
    size_t temp_bytes = 0;
    RT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, d_keys.p, d_keys2.p, d_vals.p, d_vals2.p, (int)nt, 0, 63, st));
    Scratch<unsigned char> d_temp;
    RT_CUDA_TRY(d_temp.alloc(temp_bytes));
    RT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(d_temp.p, temp_bytes, d_keys.p, d_keys2.p, d_vals.p, d_vals2.p, (int)nt, 0, 63, st));

    // Largest coordinate magnitude -> box inflation.
    unsigned cb_host[8];
    RT_CUDA_TRY(cudaMemcpyAsync(cb_host, d_cb.p, sizeof(cb_host), cudaMemcpyDeviceToHost, st));
    RT_CUDA_TRY(cudaStreamSynchronize(st));
    auto ord2f_h = [](unsigned u) {
        const unsigned b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
        float f;
        std::memcpy(&f, &b, 4);
        return f;
    };
    const float absmax = ord2f_h(cb_host[6]);
    // Boxes grow by 2^-16 of the largest coordinate: the traversal's fused slab test then
    // never rejects a box around a triangle the exact per-triangle test accepts, for ray
    // origins within 2^6 times the scene's coordinate range.
    const float eps = std::ldexp(std::fmax(absmax, 1e-30f), -16);

    RT_CUDA_TRY(d_slo.alloc(nt));
    RT_CUDA_TRY(d_shi.alloc(nt));
    k_leaves<<<tb, 256, 0, st>>>(d_vals2.p, nt, d_tlo.p, d_thi.p, ctx->d_verts.as<float>(), d_idx.p, eps, d_slo.p,
                                 d_shi.p, ctx->d_tris.as<BvhTri>());

    if (nt == 1) {
        k_root_leaf<<<1, 1, 0, st>>>(nt, d_slo.p, d_shi.p, ctx->d_nodes.as<BvhNode>());
        ctx->n_inner = 1;
        ctx->n_leaves = 1;
        ctx->depth = 3;
        ctx->sah_cost = 1.0f;
        float4 lo1, hi1;  // the whole hierarchy is the one (grown) leaf box
        RT_CUDA_TRY(cudaMemcpyAsync(&lo1, d_slo.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaMemcpyAsync(&hi1, d_shi.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaStreamSynchronize(st));
        ctx->root_box[0] = lo1.x; ctx->root_box[1] = lo1.y; ctx->root_box[2] = lo1.z;
        ctx->root_box[3] = hi1.x; ctx->root_box[4] = hi1.y; ctx->root_box[5] = hi1.z;
    } else {
        const uint64_t ni = nt - 1;
        Scratch<uint32_t> d_child, d_pin, d_pleaf, d_rf, d_rl;
        Scratch<float> d_cost;
        Scratch<float4> d_cset;
        Scratch<uchar4> d_dec;
        Scratch<uint8_t> d_col;
        Scratch<int> d_height;
        Scratch<unsigned> d_arr;
        RT_CUDA_TRY(d_child.alloc(2 * ni));
        RT_CUDA_TRY(d_pin.alloc(ni));
        RT_CUDA_TRY(d_pleaf.alloc(nt));
        RT_CUDA_TRY(d_rf.alloc(ni));
        RT_CUDA_TRY(d_rl.alloc(ni));
        RT_CUDA_TRY(d_ilo.alloc(ni));
        RT_CUDA_TRY(d_ihi.alloc(ni));
        RT_CUDA_TRY(d_cost.alloc(ni));
        RT_CUDA_TRY(d_cset.alloc(ni));
        RT_CUDA_TRY(d_dec.alloc(ni));
        RT_CUDA_TRY(d_col.alloc(ni));
        RT_CUDA_TRY(d_height.alloc(ni));
        RT_CUDA_TRY(d_arr.alloc(ni));
        RT_CUDA_TRY(cudaMemsetAsync(d_arr.p, 0, ni * sizeof(unsigned), st));
        const unsigned ib = (unsigned)((ni + 255) / 256);
        const bool cluster = RT_PLOC == 1 || (RT_PLOC == 2 && ctx->meshes.size() > 1);
        bool clustered = false;
        if (cluster) {
            // PLOC rounds over the Morton-ordered leaf boxes.
            Scratch<uint32_t> d_node[2], d_cnt[2], d_nn, d_merge, d_alive, d_moff, d_apos, d_pchild, d_icount, d_ifirst,
                d_lpos, d_order2;
            Scratch<float4> d_clo[2], d_chi[2];
            for (int b = 0; b < 2; ++b) {
                RT_CUDA_TRY(d_node[b].alloc(nt));
                RT_CUDA_TRY(d_cnt[b].alloc(nt));
                RT_CUDA_TRY(d_clo[b].alloc(nt));
                RT_CUDA_TRY(d_chi[b].alloc(nt));
            }
            RT_CUDA_TRY(d_nn.alloc(nt));
            RT_CUDA_TRY(d_merge.alloc(nt));
            RT_CUDA_TRY(d_alive.alloc(nt));
            RT_CUDA_TRY(d_moff.alloc(nt));
            RT_CUDA_TRY(d_apos.alloc(nt));
            RT_CUDA_TRY(d_pchild.alloc(2 * ni));
            RT_CUDA_TRY(d_icount.alloc(ni));
            RT_CUDA_TRY(d_ifirst.alloc(ni));
            RT_CUDA_TRY(d_lpos.alloc(nt));
            RT_CUDA_TRY(d_order2.alloc(nt));
            size_t scan_bytes = 0;
            RT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, d_merge.p, d_moff.p, (int)nt, st));
            Scratch<unsigned char> d_scan;
            RT_CUDA_TRY(d_scan.alloc(scan_bytes));
            unsigned *status = ctx->d_status.as<unsigned>();
            k_ploc_init<<<tb, 256, 0, st>>>(nt, d_slo.p, d_shi.p, d_node[0].p, d_clo[0].p, d_chi[0].p, d_cnt[0].p);
            std::vector<uint32_t> round_base, round_count;
            uint32_t n = (uint32_t)nt, inner = 0;
            int cur = 0;
            bool give_up = false;
            while (n > 1) {
                // Many coincident boxes merge one pair per round (every tie picks the lowest
                // index): past kPlocMaxRounds the build falls back to the radix tree.
                if (round_base.size() >= kPlocMaxRounds) {
                    give_up = true;
                    break;
                }
                const unsigned nb = (n + kPlocBlock - 1) / kPlocBlock;
                k_ploc_nn<<<nb, kPlocBlock, 0, st>>>(d_clo[cur].p, d_chi[cur].p, n, d_nn.p);
                k_ploc_flags<<<nb, kPlocBlock, 0, st>>>(d_nn.p, n, d_merge.p, d_alive.p);
                RT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(d_scan.p, scan_bytes, d_merge.p, d_moff.p, (int)n, st));
                RT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(d_scan.p, scan_bytes, d_alive.p, d_apos.p, (int)n, st));
                k_ploc_compact<<<nb, kPlocBlock, 0, st>>>(
                    d_node[cur].p, d_clo[cur].p, d_chi[cur].p, d_cnt[cur].p, d_nn.p, d_merge.p, d_alive.p, d_moff.p,
                    d_apos.p, n, inner, (uint32_t)ni, d_pchild.p, d_icount.p, d_node[cur ^ 1].p, d_clo[cur ^ 1].p,
                    d_chi[cur ^ 1].p, d_cnt[cur ^ 1].p, status);
                uint32_t tail[4];
                RT_CUDA_TRY(cudaMemcpyAsync(&tail[0], d_moff.p + (n - 1), 4, cudaMemcpyDeviceToHost, st));
                RT_CUDA_TRY(cudaMemcpyAsync(&tail[1], d_merge.p + (n - 1), 4, cudaMemcpyDeviceToHost, st));
                RT_CUDA_TRY(cudaMemcpyAsync(&tail[2], d_apos.p + (n - 1), 4, cudaMemcpyDeviceToHost, st));
                RT_CUDA_TRY(cudaMemcpyAsync(&tail[3], d_alive.p + (n - 1), 4, cudaMemcpyDeviceToHost, st));
                RT_CUDA_TRY(cudaStreamSynchronize(st));
                const uint32_t merges = tail[0] + tail[1], n_new = tail[2] + tail[3];
                if (merges == 0 || n_new + merges != n || inner + merges > ni) {
                    set_error("hierarchy clustering made no progress");
                    return RT_ERR_STATE;
                }
                round_base.push_back(inner);
                round_count.push_back(merges);
                inner += merges;
                n = n_new;
                cur ^= 1;
            }
            if (!give_up && inner != ni) {
                set_error("hierarchy clustering left several roots");
                return RT_ERR_STATE;
            }
            if (!give_up) {
                const uint32_t zero = 0;
                RT_CUDA_TRY(cudaMemcpyAsync(d_ifirst.p + (ni - 1), &zero, 4, cudaMemcpyHostToDevice, st));
                for (size_t r = round_base.size(); r-- > 0;)
                    k_ploc_topdown<<<(round_count[r] + 255) / 256, 256, 0, st>>>(
                        round_base[r], round_count[r], (uint32_t)ni, nt, d_pchild.p, d_icount.p, d_ifirst.p, d_lpos.p,
                        status);
                k_ploc_final<<<ib, 256, 0, st>>>((uint32_t)ni, nt, d_pchild.p, d_icount.p, d_ifirst.p, d_lpos.p,
                                                 d_child.p, d_pin.p, d_pleaf.p, d_rf.p, d_rl.p, status);
                // Leaves, their boxes and the triangles again, in the depth-first leaf order (zeroed
                // first: a malformed permutation would leave valid triangle ids, never stray ones).
                RT_CUDA_TRY(cudaMemsetAsync(d_order2.p, 0, nt * sizeof(uint32_t), st));
                k_scatter_order<<<tb, 256, 0, st>>>(d_vals2.p, d_lpos.p, nt, d_order2.p);
                k_leaves<<<tb, 256, 0, st>>>(d_order2.p, nt, d_tlo.p, d_thi.p, ctx->d_verts.as<float>(), d_idx.p, eps,
                                             d_slo.p, d_shi.p, ctx->d_tris.as<BvhTri>());
                clustered = true;
            }
        }
        if (!clustered)
            k_karras<<<ib, 256, 0, st>>>(d_keys2.p, (int64_t)nt, d_child.p, d_pin.p, d_pleaf.p, d_rf.p, d_rl.p);
        k_bottom_up<<<tb, 256, 0, st>>>(nt, d_child.p, d_pin.p, d_pleaf.p, d_rf.p, d_rl.p, d_slo.p, d_shi.p, d_ilo.p,
                                        d_ihi.p, d_cost.p, d_col.p, d_height.p, d_arr.p, d_cset.p, d_dec.p);
        uint8_t root_col = 0;
        int root_h = 0;
        float root_cost = 0.0f;
        float4 rlo, rhi;
        RT_CUDA_TRY(cudaMemcpyAsync(&root_col, d_col.p, 1, cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaMemcpyAsync(&root_h, d_height.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaMemcpyAsync(&root_cost, d_cost.p, sizeof(float), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaMemcpyAsync(&rlo, d_ilo.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaMemcpyAsync(&rhi, d_ihi.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
        RT_CUDA_TRY(cudaStreamSynchronize(st));
        const float ra = std::fmax((rhi.x - rlo.x) * (rhi.y - rlo.y) + (rhi.y - rlo.y) * (rhi.z - rlo.z) +
                                       (rhi.z - rlo.z) * (rhi.x - rlo.x), 1e-30f);
        ctx->sah_cost = root_cost / ra;
        ctx->root_box[0] = rlo.x; ctx->root_box[1] = rlo.y; ctx->root_box[2] = rlo.z;
        ctx->root_box[3] = rhi.x; ctx->root_box[4] = rhi.y; ctx->root_box[5] = rhi.z;
        if (root_col) {
            k_root_leaf<<<1, 1, 0, st>>>(nt, d_slo.p, d_shi.p, ctx->d_nodes.as<BvhNode>());
            ctx->n_inner = 1;
            ctx->n_leaves = 1;
            ctx->depth = 3;
        } else {
            // Binary -> 4-wide collapse, one level per launch (breadth-first slot order).
            Scratch<CollapseItem> d_q0, d_q1;
            Scratch<uint32_t> d_cnt;  // [0] n_out, [1] node count, [2] leaf count
            RT_CUDA_TRY(d_q0.alloc(ni));
            RT_CUDA_TRY(d_q1.alloc(ni));
            RT_CUDA_TRY(d_cnt.alloc(4));
            const CollapseItem root{0u, 0u};
            const uint32_t cnt_init[4] = {0u, 1u, 0u, 0u};
            RT_CUDA_TRY(cudaMemcpyAsync(d_q0.p, &root, sizeof(root), cudaMemcpyHostToDevice, st));
            RT_CUDA_TRY(cudaMemcpyAsync(d_cnt.p, cnt_init, sizeof(cnt_init), cudaMemcpyHostToDevice, st));
            uint32_t n_in = 1, levels = 0;
            std::vector<uint32_t> level_end(1, 1u);  // slots [level_end[l-1], level_end[l]) = level l
            CollapseItem *qin = d_q0.p, *qout = d_q1.p;
            while (n_in > 0) {
                RT_CUDA_TRY(cudaMemsetAsync(d_cnt.p, 0, sizeof(uint32_t), st));
                k_collapse<<<(n_in + 127) / 128, 128, 0, st>>>(qin, n_in, qout, d_cnt.p, d_cnt.p + 1, (uint32_t)ni,
                                                               d_child.p, d_rf.p, d_rl.p, d_slo.p, d_shi.p, d_ilo.p,
                                                               d_ihi.p, d_col.p, ctx->d_nodes.as<BvhNode>(),
                                                               d_cnt.p + 2, ctx->d_status.as<unsigned>(), d_dec.p);
                uint32_t cn2[2];
                RT_CUDA_TRY(cudaMemcpyAsync(cn2, d_cnt.p, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                RT_CUDA_TRY(cudaStreamSynchronize(st));
                n_in = cn2[0];
                if (n_in > 0) level_end.push_back(cn2[1]);
                std::swap(qin, qout);
                ++levels;
                if (levels > 200) {
                    set_error("hierarchy collapse did not terminate");
                    return RT_ERR_STATE;
                }
            }
            uint32_t cnt[4];
            RT_CUDA_TRY(cudaMemcpyAsync(cnt, d_cnt.p, sizeof(cnt), cudaMemcpyDeviceToHost, st));
            RT_CUDA_TRY(cudaStreamSynchronize(st));
            ctx->n_inner = cnt[1];
            ctx->n_leaves = cnt[2];
            // Stack bound from the collapsed tree (at most 3 entries per level, usually far fewer).
            Scratch<uint32_t> d_need;
            RT_CUDA_TRY(d_need.alloc(cnt[1]));
            for (size_t l = level_end.size(); l-- > 0;) {
                const uint32_t s0 = l ? level_end[l - 1] : 0u, s1 = std::min(level_end[l], cnt[1]);
                if (s1 > s0)
                    k_stack_need<<<(s1 - s0 + 127) / 128, 128, 0, st>>>(ctx->d_nodes.as<BvhNode>(), s0, s1, cnt[1],
                                                                      d_need.p);
            }
            uint32_t need0 = 0;
            RT_CUDA_TRY(cudaMemcpyAsync(&need0, d_need.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            RT_CUDA_TRY(cudaStreamSynchronize(st));
            ctx->depth = std::min(3 * (int)levels, (int)need0 + 1);
            (void)root_h;
        }
    }
    RT_CUDA_TRY(cudaEventRecord(ctx->ev_b, st));
    RT_CUDA_TRY(cudaEventSynchronize(ctx->ev_b));
    RT_CUDA_TRY(cudaGetLastError());
    RT_CUDA_TRY(cudaEventElapsedTime(&ctx->build_ms, ctx->ev_a, ctx->ev_b));
    return RT_OK;
}

}  // namespace rgb
