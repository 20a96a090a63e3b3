// rt_visible_noalloc: the segment-visibility query (rt_visible) for callers that cannot
// allocate device memory, e.g. code that runs where cudaMalloc is forbidden or must not
// block (a frame loop or audio/robotics callback with a fixed memory budget, a plugin host
// that owns every allocation, code that must not trigger the implicit synchronisation of
// cudaMalloc/cudaFree). The caller passes device buffers for the segments and the answers;
// the library's own scratch -- the converted rays and the traversal's ray-fetch counter --
// lives in one file-scope device array instead of cudaMalloc'd memory. A traversal stack
// overflow is recorded in the context's status word for asynchronous calls (allocated once
// by rt_create), which rt_get_status reads and clears.
//
// Limits and rules (also stated in include/rendu_gb300.h):
//  * at most RT_NOALLOC_MAX_SEGMENTS segments per call (the array is 256 B + 32 B per
//    segment, 8 MiB in total, held by every GPU that loads the library until exit);
//  * every call shares the array: calls that overlap on the GPU (on different streams,
//    or from several threads) race and must be serialised by the caller;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device); make that first call before any stream
//    capture.
#include <cstring>
#include <mutex>
#include <string>

#include "rt_context.hpp"
#include "rt_traverse.cuh"

namespace rgb {
namespace {

constexpr size_t kHeaderBytes = 256;  // ray-fetch counter at 8 (bytes 0..15 cleared per call)
constexpr size_t kScratchBytes = kHeaderBytes + sizeof(rt_ray) * (size_t)RT_NOALLOC_MAX_SEGMENTS;

// The scratch. In host code this name is only a stand-in for the symbol: its device address
// comes from cudaGetSymbolAddress below and is what the kernels receive.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Raycaster::visible (Raycaster.cpp:226-230): window (1e-4, |p1 - p0|) along p1 - p0.
__global__ void k_noalloc_segments(const float *__restrict__ segs, uint32_t n, rt_ray *__restrict__ rays) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *s = segs + 6 * (size_t)i;
    const f3 p0 = mk(s[0], s[1], s[2]);
    const f3 dir = xsub(mk(s[3], s[4], s[5]), p0);
    rays[i] = rt_ray{p0.x, p0.y, p0.z, 0.0001f, dir.x, dir.y, dir.z, __fsqrt_rn(xdot(dir, dir))};
}

// Any-hit traversal with per-lane ray refill over the scratch rays; writes visibility.
template <int STACK>
__global__ void __launch_bounds__(128) k_noalloc_visible(const BvhNode *__restrict__ nodes,
                                                         const BvhTri *__restrict__ tris,
                                                         const rt_ray *__restrict__ rays, uint32_t n,
                                                         uint8_t *__restrict__ visible, unsigned *__restrict__ status,
                                                         unsigned long long *__restrict__ counter, int empty) {
    const unsigned lane = threadIdx.x & 31;
    int stack_node[STACK];
    float stack_near[STACK];
    RayState r;
    TravState t;
    uint32_t idx = 0;
    bool active = false, exhausted = false;
    uint32_t nv_ = 0, nt_ = 0;
    while (true) {
        const unsigned need = __ballot_sync(0xffffffffu, !active);
        if (need && !exhausted) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(need) >= n) exhausted = true;
            if (!active) {
                const unsigned long long k = base + __popc(need & ((1u << lane) - 1u));
                if (k < n) {
                    idx = (uint32_t)k;
                    const float4 *rp = reinterpret_cast<const float4 *>(rays + idx);
                    r = make_ray_state(rp[0], rp[1]);
                    trav_init(t, r);
                    active = r.valid && !empty;
                    if (!active) visible[idx] = 1;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (active && trav_step<true, false, STACK>(nodes, tris, r, t, stack_node, stack_near, status, nv_, nt_)) {
            active = false;
            visible[idx] = t.res.found ? 0 : 1;
        }
    }
}

struct DeviceScratch {
    void *ptr = nullptr;
    bool ready = false;
};

std::mutex g_lock;
DeviceScratch g_dev[64];
int g_grid[64][3];

}  // namespace
}  // namespace rgb

using namespace rgb;

extern "C" int rt_visible_noalloc(rt_ctx *ctx, const float *segs, size_t n, uint8_t *visible, void *stream) {
    clear_error();
    cudaGetLastError();  // a launch error reported below then belongs to this call
    if (!ctx || (n && (!segs || !visible))) {
        set_error("null argument");
        return RT_ERR_ARG;
    }
    if (!ctx->built || ctx->dirty) {
        set_error("rt_update_hierarchy must be called after the last rt_add_mesh");
        return RT_ERR_STATE;
    }
    if (n > (size_t)RT_NOALLOC_MAX_SEGMENTS) {
        set_error("rt_visible_noalloc takes at most " + std::to_string(RT_NOALLOC_MAX_SEGMENTS) +
                  " segments per call; got " + std::to_string(n));
        return RT_ERR_ARG;
    }
    if (ctx->device < 0 || ctx->device >= 64) {
        set_error("device index out of range");
        return RT_ERR_ARG;
    }
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != ctx->device) RT_CUDA_TRY(cudaSetDevice(ctx->device));
    int rc = RT_OK;
    unsigned char *base = nullptr;
    {
        // Once per device, with that device current: the device address of the scratch.
        std::lock_guard<std::mutex> g(g_lock);
        DeviceScratch &d = g_dev[ctx->device];
        if (!d.ready) {
            const cudaError_t e = cudaGetSymbolAddress(&d.ptr, g_noalloc_scratch);
            if (e != cudaSuccess) {
                set_error(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
                rc = RT_ERR_CUDA;
            } else {
                int sms = 0, per_sm = 0;
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_visible<64>, 128, 0);
                g_grid[ctx->device][0] = sms * (per_sm > 0 ? per_sm : 1);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_visible<256>, 128, 0);
                g_grid[ctx->device][1] = sms * (per_sm > 0 ? per_sm : 1);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_visible<2>, 128, 0);
                g_grid[ctx->device][2] = sms * (per_sm > 0 ? per_sm : 1);
                d.ready = true;
            }
        }
        base = static_cast<unsigned char *>(d.ptr);
    }
    if (rc == RT_OK && n > 0) {
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // Overflows go to the context's word for asynchronous calls (rt_get_status).
        unsigned *status = status_word(ctx, st);
        unsigned long long *counter = reinterpret_cast<unsigned long long *>(base + 8);
        rt_ray *rays = reinterpret_cast<rt_ray *>(base + kHeaderBytes);
        // The header (fetch counter included) must start at zero; the previous call's rays
        // are overwritten.
        const cudaError_t me = cudaMemsetAsync(base, 0, 16, st);
        if (me != cudaSuccess) {
            set_error(std::string("cudaMemsetAsync failed: ") + cudaGetErrorString(me));
            rc = RT_ERR_CUDA;
        }
        if (rc == RT_OK) {
            k_noalloc_segments<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(segs, (uint32_t)n, rays);
            const BvhNode *nodes = ctx->d_nodes.as<BvhNode>();
            const BvhTri *tris = ctx->d_tris.as<BvhTri>();
            const int empty = ctx->n_tris == 0 ? 1 : 0;
            const int stack = traversal_stack(ctx);
            if (stack == 64)
                k_noalloc_visible<64><<<g_grid[ctx->device][0], 128, 0, st>>>(nodes, tris, rays, (uint32_t)n, visible,
                                                                              status, counter, empty);
            else if (stack == 256)
                k_noalloc_visible<256><<<g_grid[ctx->device][1], 128, 0, st>>>(nodes, tris, rays, (uint32_t)n,
                                                                               visible, status, counter, empty);
            else
                k_noalloc_visible<2><<<g_grid[ctx->device][2], 128, 0, st>>>(nodes, tris, rays, (uint32_t)n, visible,
                                                                             status, counter, empty);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                set_error(std::string("launch failed: ") + cudaGetErrorString(e));
                rc = RT_ERR_CUDA;
            }
        }
    }
    if (prev >= 0 && prev != ctx->device) cudaSetDevice(prev);
    return rc;
}
