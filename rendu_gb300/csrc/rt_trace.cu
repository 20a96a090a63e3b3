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

// Persistent variant: a grid sized to fill the GPU once; idle lanes take new rays from
// their block's interleaved share through a shared-memory counter (RT_FETCH_BLOCK 1) or from
// the global `counter` zeroed before the launch (0). n is read from n_dev when given
// (device-side queue length). The box of the whole hierarchy (the union of the grown leaf
// boxes): a ray that misses it misses every child box of the root, so it is answered
// without a node fetch.
// Refill heuristics (see k_trace_batch): on the raycaster workload, where 88 % of the rays
// miss the root box and are answered at intake, thresholds 8-16 measured equal to 1 and
// back-to-back rounds slower (2-4 rounds: 1.39 -> 1.55-2.02 ms per 16M rays).
// RT_FETCH_BLOCK 1 (default): interleaved chunks per block and a shared-memory counter;
// 0: one global counter for all warps. Measured on the raycaster workload: closest hit
// 1.380 -> 1.363 ms, any hit 1.186 -> 1.159 ms per 16M rays.
#ifndef RT_FETCH_BLOCK
#define RT_FETCH_BLOCK 1
#endif
#ifndef RT_REFILL_MIN
#define RT_REFILL_MIN 1
#endif
#ifndef RT_REFILL_ROUNDS
#define RT_REFILL_ROUNDS 1
#endif
// RT_INTAKE_QUEUE 1: a warp takes rays 32 at a time (one per lane), answers the ones that miss
// the hierarchy's box at once and queues the indices of the others in shared memory; idle
// lanes are refilled only from that queue, so every lane that traverses holds a ray that
// enters the hierarchy (on the raycaster workload 88 % of the rays do not).
#ifndef RT_INTAKE_QUEUE
#define RT_INTAKE_QUEUE 1
#endif
constexpr int kIntakeQueue = 64;  // queued ray indices per warp (at most 31 + 32 at a time)
struct RootBox {
    float lo[3], hi[3];
};

template <bool ANY, int STACK>
__global__ void __launch_bounds__(128) k_trace_persistent(const BvhNode *__restrict__ nodes,
                                                          const BvhTri *__restrict__ tris,
                                                          const rt_ray *__restrict__ rays, size_t n_host,
                                                          const uint32_t *__restrict__ n_dev, rt_hit *__restrict__ hits,
                                                          uint8_t *__restrict__ occ, unsigned *__restrict__ status,
                                                          unsigned long long *__restrict__ counter, const RootBox root) {
    const size_t n = n_dev ? (size_t)*n_dev : n_host;
    const unsigned lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
#if RT_FETCH_BLOCK
    // Rays are dealt to the blocks in interleaved chunks of 256 (chunk k to block k mod grid),
    // and a block's warps take them through a shared-memory counter: no global atomic per
    // refill round, while a cost that varies smoothly with the ray index still spreads over
    // all blocks.
    __shared__ unsigned s_next;
    if (threadIdx.x == 0) s_next = 0u;
    __syncthreads();
#endif
    int stack_node[STACK];
    float stack_near[STACK];
    RayState r;
    TravState t;
    size_t idx = 0;
    bool active = false, exhausted = false;
    uint32_t nv_ = 0, nt_ = 0;
#if RT_INTAKE_QUEUE && RT_FETCH_BLOCK
    // Queued rays keep their record in shared memory, so that each ray is read from its
    // buffer once (the buffer may be mapped host memory).
    __shared__ unsigned s_queue[4][kIntakeQueue];  // 128 threads = 4 warps
    __shared__ float4 s_qray[4][kIntakeQueue][2];
    unsigned *queue = s_queue[threadIdx.x >> 5];
    float4 (*qray)[2] = s_qray[threadIdx.x >> 5];
    int qn = 0;  // queued entries (warp-uniform)
    auto ray_of = [&](unsigned u) { return ((size_t)(u >> 8) * gridDim.x + blockIdx.x) * 256u + (u & 255u); };
    auto write_miss = [&](size_t i) {
        if (ANY) occ[i] = 0;
        else __stcs(reinterpret_cast<float4 *>(hits + i), make_float4(FLT_MAX, 0.0f, 0.0f, __uint_as_float(RT_NO_HIT)));
    };
    while (true) {
        unsigned need = __ballot_sync(0xffffffffu, !active);
        while (need) {
            if (qn < __popc(need) && !exhausted) {
                // Intake round: 32 rays, one per lane; misses answered, the others queued.
                unsigned v = 0;
                if (lane == 0) v = atomicAdd(&s_next, 32u);
                v = __shfl_sync(0xffffffffu, v, 0);
                if (ray_of(v + 31) >= n) exhausted = true;
                const size_t i = ray_of(v + lane);
                bool enters = false;
                float4 ra = make_float4(0.0f, 0.0f, 0.0f, 0.0f), rb = ra;
                if (i < n) {
                    const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
                    ra = __ldcs(rp);
                    rb = __ldcs(rp + 1);
                    const RayState q = make_ray_state(ra, rb);
                    enters = q.valid && slab(q, root.lo[0], root.hi[0], root.lo[1], root.hi[1], root.lo[2],
                                             root.hi[2], q.tmin, q.tmax) != INFINITY;
                    if (!enters) write_miss(i);
                }
                const unsigned em = __ballot_sync(0xffffffffu, enters);
                if (enters) {
                    const int slot = qn + __popc(em & lt_mask);
                    queue[slot] = (unsigned)i;
                    qray[slot][0] = ra;
                    qray[slot][1] = rb;
                }
                qn += __popc(em);
                __syncwarp();
            }
            if (qn == 0) {
                if (exhausted) break;
                continue;
            }
            // Idle lanes take queued rays, newest first.
            const unsigned take = min((unsigned)qn, (unsigned)__popc(need));
            const unsigned rank = __popc(need & lt_mask);
            if (!active && rank < take) {
                const int slot = qn - 1 - (int)rank;
                idx = queue[slot];
                r = make_ray_state(qray[slot][0], qray[slot][1]);
                trav_init(t, r);
                active = true;
            }
            qn -= (int)take;
            __syncwarp();
            need = __ballot_sync(0xffffffffu, !active);
            if (need && qn == 0 && exhausted) break;
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted && qn == 0) break;
            continue;
        }
        if (active && trav_step<ANY, false, STACK>(nodes, tris, r, t, stack_node, stack_near, status, nv_, nt_)) {
            active = false;
            if (ANY) {
                occ[idx] = t.res.found ? 1 : 0;
            } else {
                __stcs(reinterpret_cast<float4 *>(hits + idx),
                       make_float4(t.res.found ? t.res.t : FLT_MAX, t.res.u, t.res.v,
                                   __uint_as_float(t.res.found ? t.res.prim : RT_NO_HIT)));
            }
        }
    }
#else
    while (true) {
        // Refill idle lanes: up to RT_REFILL_ROUNDS rounds back to back while at least
        // RT_REFILL_MIN lanes are idle (a warp with no active lane always refills).
        for (int round = 0; round < RT_REFILL_ROUNDS && !exhausted; ++round) {
            const unsigned need = __ballot_sync(0xffffffffu, !active);
            if (!need || (__popc(need) < RT_REFILL_MIN && need != 0xffffffffu)) break;
            const int leader = __ffs(need) - 1;
            const unsigned take = (unsigned)__popc(need);
            const unsigned rank = __popc(need & lt_mask);
#if RT_FETCH_BLOCK
            unsigned v = 0;
            if ((int)lane == leader) v = atomicAdd(&s_next, take);
            v = __shfl_sync(0xffffffffu, v, leader);
            auto ray_of = [&](unsigned u) {
                return ((size_t)(u >> 8) * gridDim.x + blockIdx.x) * 256u + (u & 255u);
            };
            if (ray_of(v + take - 1) >= n) exhausted = true;
            if (!active) {
                idx = ray_of(v + rank);
                if (idx < n) {
#else
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)take);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + take >= n) exhausted = true;
            if (!active) {
                idx = (size_t)base + rank;
                if (idx < n) {
#endif
                    const float4 *rp = reinterpret_cast<const float4 *>(rays + idx);
                    r = make_ray_state(__ldcs(rp), __ldcs(rp + 1));
                    trav_init(t, r);
                    active = r.valid && slab(r, root.lo[0], root.hi[0], root.lo[1], root.hi[1], root.lo[2],
                                             root.hi[2], r.tmin, r.tmax) != INFINITY;
                    if (!active) {  // never hits: write the miss now
                        if (ANY) occ[idx] = 0;
                        else __stcs(reinterpret_cast<float4 *>(hits + idx),
                                    make_float4(FLT_MAX, 0.0f, 0.0f, __uint_as_float(RT_NO_HIT)));
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (active && trav_step<ANY, false, STACK>(nodes, tris, r, t, stack_node, stack_near, status, nv_, nt_)) {
            active = false;
            if (ANY) {
                occ[idx] = t.res.found ? 1 : 0;
            } else {
                __stcs(reinterpret_cast<float4 *>(hits + idx),
                       make_float4(t.res.found ? t.res.t : FLT_MAX, t.res.u, t.res.v,
                                   __uint_as_float(t.res.found ? t.res.prim : RT_NO_HIT)));
            }
        }
    }
#endif
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

template <bool ANY, int STACK>
int launch_persistent(rt_ctx *ctx, const rt_ray *rays, size_t n, const uint32_t *n_dev, rt_hit *hits, uint8_t *occ,
                      cudaStream_t st) {
    static int grid[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int &g = grid[ANY ? 1 : 0][STACK == 64 ? 0 : (STACK == 256 ? 1 : 2)];
    if (g == 0) {
        int per_sm = 0, sms = 0, dev = 0;
        RT_CUDA_TRY(cudaGetDevice(&dev));
        RT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_persistent<ANY, STACK>, 128, 0));
        g = sms * (per_sm > 0 ? per_sm : 1);
    }
    unsigned long long *counter =
        reinterpret_cast<unsigned long long *>(ctx->d_status.as<char>() + fetch_counter_offset(ctx, st));
    RT_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
    const RootBox root{{ctx->root_box[0], ctx->root_box[1], ctx->root_box[2]},
                       {ctx->root_box[3], ctx->root_box[4], ctx->root_box[5]}};
    k_trace_persistent<ANY, STACK><<<g, 128, 0, st>>>(ctx->d_nodes.as<BvhNode>(), ctx->d_tris.as<BvhTri>(), rays, n,
                                                      n_dev, hits, occ, status_word(ctx, st), counter, root);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

template <bool ANY, bool COUNT>
int launch(rt_ctx *ctx, const rt_ray *rays, size_t n, rt_hit *hits, uint8_t *occ, uint32_t *nc, uint32_t *tc,
           cudaStream_t st) {
    if (n == 0) return RT_OK;
    const int stack = traversal_stack(ctx);
    if (!COUNT && ctx->n_tris > 0) {
        if (stack == 64) return launch_persistent<ANY, 64>(ctx, rays, n, nullptr, hits, occ, st);
        if (stack == 256) return launch_persistent<ANY, 256>(ctx, rays, n, nullptr, hits, occ, st);
        return launch_persistent<ANY, 2>(ctx, rays, n, nullptr, hits, occ, st);
    }
    const unsigned blocks = (unsigned)((n + 127) / 128);
    const BvhNode *nodes = ctx->d_nodes.as<BvhNode>();
    const BvhTri *tris = ctx->d_tris.as<BvhTri>();
    unsigned *status = status_word(ctx, st);
    const int empty = ctx->n_tris == 0 ? 1 : 0;
    if (stack == 64)
        k_trace<ANY, COUNT, 64><<<blocks, 128, 0, st>>>(nodes, tris, rays, n, hits, occ, nc, tc, status, empty);
    else if (stack == 256)
        k_trace<ANY, COUNT, 256><<<blocks, 128, 0, st>>>(nodes, tris, rays, n, hits, occ, nc, tc, status, empty);
    else
        k_trace<ANY, COUNT, 2><<<blocks, 128, 0, st>>>(nodes, tris, rays, n, hits, occ, nc, tc, status, empty);
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

namespace {
__global__ void k_fill_miss(const uint32_t *__restrict__ count, rt_hit *__restrict__ hits, uint32_t cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < cap && i < *count) hits[i] = rt_hit{FLT_MAX, 0.0f, 0.0f, RT_NO_HIT};
}
}  // namespace

int trace_closest_queue(rt_ctx *ctx, const rt_ray *d_rays, const uint32_t *d_count, uint32_t cap, rt_hit *d_hits,
                        cudaStream_t st) {
    if (cap == 0) return RT_OK;
    if (ctx->n_tris == 0) {
        k_fill_miss<<<(cap + 255) / 256, 256, 0, st>>>(d_count, d_hits, cap);
        RT_CUDA_TRY(cudaGetLastError());
        return RT_OK;
    }
    const int stack = traversal_stack(ctx);
    if (stack == 64) return launch_persistent<false, 64>(ctx, d_rays, cap, d_count, d_hits, nullptr, st);
    if (stack == 256) return launch_persistent<false, 256>(ctx, d_rays, cap, d_count, d_hits, nullptr, st);
    return launch_persistent<false, 2>(ctx, d_rays, cap, d_count, d_hits, nullptr, st);
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
