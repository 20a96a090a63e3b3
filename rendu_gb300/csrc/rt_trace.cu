// Raycaster query kernels: replace Raycaster::intersects / intersectsAny / visible
// (Raycaster.cpp:144-230 of kosua20/Rendu) with one thread per ray over the device
// hierarchy built in rt_build.cu; the per-ray traversal is rt_traverse.cuh.
// Ray records are read and hit records written with streaming (evict-first) accesses so
// that the L2 keeps the hierarchy, which every ray re-reads.
#include "rt_context.hpp"
#include "rt_traverse.cuh"

namespace rgb {
namespace {

template <bool ANY, bool COUNT, int STACK>
__global__ void __launch_bounds__(128) k_trace(const BvhNode *__restrict__ nodes, const BvhTri *__restrict__ tris,
                                               const rt_ray *__restrict__ rays, size_t n, rt_hit *__restrict__ hits,
                                               uint8_t *__restrict__ occ, uint32_t *__restrict__ node_cnt,
                                               uint32_t *__restrict__ tri_cnt, unsigned *__restrict__ status,
                                               int empty) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
    const RayState r = make_ray_state(__ldcs(rp), __ldcs(rp + 1));
    TraceResult res;
    res.found = false;
    res.t = FLT_MAX;
    res.u = res.v = 0.0f;
    res.prim = RT_NO_HIT;
    uint32_t nvis = 0, ntri = 0;
    if (r.valid && !empty) res = traverse<ANY, COUNT, STACK>(nodes, tris, r, status, nvis, ntri);
    if (ANY) {
        occ[i] = res.found ? 1 : 0;
    } else {
        __stcs(reinterpret_cast<float4 *>(hits + i),
               make_float4(res.found ? res.t : FLT_MAX, res.u, res.v, __uint_as_float(res.found ? res.prim : RT_NO_HIT)));
    }
    if (COUNT) {
        node_cnt[i] = nvis;
        tri_cnt[i] = ntri;
    }
}

// Raycaster::visible (Raycaster.cpp:226-230): window (1e-4, |p1 - p0|) along p1 - p0.
__global__ void k_segments_to_rays(const float *__restrict__ segs, size_t n, rt_ray *__restrict__ rays) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *s = segs + 6 * i;
    const f3 p0 = mk(s[0], s[1], s[2]);
    const f3 dir = xsub(mk(s[3], s[4], s[5]), p0);
    const float len = __fsqrt_rn(xdot(dir, dir));  // glm::length = sqrt(dot(v, v))
    rays[i] = rt_ray{p0.x, p0.y, p0.z, 0.0001f, dir.x, dir.y, dir.z, len};
}

__global__ void k_invert(uint8_t *__restrict__ v, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = v[i] ? 0 : 1;
}

template <bool ANY, bool COUNT>
int launch(rt_ctx *ctx, const rt_ray *rays, size_t n, rt_hit *hits, uint8_t *occ, uint32_t *nc, uint32_t *tc,
           cudaStream_t st) {
    if (n == 0) return RT_OK;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    const BvhNode *nodes = ctx->d_nodes.as<BvhNode>();
    const BvhTri *tris = ctx->d_tris.as<BvhTri>();
    unsigned *status = ctx->d_status.as<unsigned>();
    const int empty = ctx->n_tris == 0 ? 1 : 0;
    if (ctx->depth <= 64)
        k_trace<ANY, COUNT, 64><<<blocks, 128, 0, st>>>(nodes, tris, rays, n, hits, occ, nc, tc, status, empty);
    else
        k_trace<ANY, COUNT, 256><<<blocks, 128, 0, st>>>(nodes, tris, rays, n, hits, occ, nc, tc, status, empty);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

}  // namespace

int trace_closest(rt_ctx *ctx, const rt_ray *d_rays, size_t n, rt_hit *d_hits, cudaStream_t st) {
    return launch<false, false>(ctx, d_rays, n, d_hits, nullptr, nullptr, nullptr, st);
}

int trace_any(rt_ctx *ctx, const rt_ray *d_rays, size_t n, uint8_t *d_occ, cudaStream_t st) {
    return launch<true, false>(ctx, d_rays, n, nullptr, d_occ, nullptr, nullptr, st);
}

int trace_count(rt_ctx *ctx, const rt_ray *d_rays, size_t n, uint32_t *nc, uint32_t *tc, rt_hit *scratch,
                cudaStream_t st) {
    return launch<false, true>(ctx, d_rays, n, scratch, nullptr, nc, tc, st);
}

int segments_to_rays(const float *d_segs, size_t n, rt_ray *d_rays, cudaStream_t st) {
    if (n == 0) return RT_OK;
    k_segments_to_rays<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_segs, n, d_rays);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int invert_bytes(uint8_t *d, size_t n, cudaStream_t st) {
    if (n == 0) return RT_OK;
    k_invert<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, n);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

}  // namespace rgb
