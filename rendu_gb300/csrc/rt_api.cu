// C-ABI of the raycaster (include/rendu_gb300.h): context life cycle, mesh intake,
// hierarchy build, batched queries with host or device buffers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "rt_chunks.hpp"
#include "rt_context.hpp"

namespace rgb {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

int DevBuf::reserve(size_t need) {
    if (need <= bytes && ptr) return RT_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    if (cudaMalloc(&ptr, need ? need : 16) != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation of " + std::to_string(need) + " bytes failed");
        return RT_ERR_OOM;
    }
    bytes = need;
    return RT_OK;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int build_hierarchy(rt_ctx *ctx);
int trace_count(rt_ctx *ctx, const rt_ray *d_rays, size_t n, uint32_t *nc, uint32_t *tc, rt_hit *scratch,
                cudaStream_t st);
int segments_to_rays(const float *d_segs, size_t n, rt_ray *d_rays, cudaStream_t st);
int invert_bytes(uint8_t *d, size_t n, cudaStream_t st);

// Reads the status word at `word` on stream `st` (waiting for the stream), clears it and
// maps its bits to a status code.
static int read_status(void *word, cudaStream_t st, unsigned *raw) {
    unsigned s = 0;
    RT_CUDA_TRY(cudaMemcpyAsync(&s, word, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    RT_CUDA_TRY(cudaStreamSynchronize(st));
    if (raw) *raw = s;
    if (s) {
        RT_CUDA_TRY(cudaMemsetAsync(word, 0, sizeof(unsigned), st));
        if (s & RT_DEV_TIMEOUT) {
            set_error("a bounded device loop gave up");
            return RT_ERR_TIMEOUT;
        }
        set_error("a traversal stack or queue overflowed");
        return RT_ERR_OVERFLOW;
    }
    return RT_OK;
}

int check_status(rt_ctx *ctx, cudaStream_t st) { return read_status(ctx->d_status.ptr, st, nullptr); }

// Hit -> (meshId, localId): the last mesh whose first triangle is <= prim (empty meshes share
// their successor's first triangle and are never the last such mesh for a valid prim).
__global__ void k_hit_info(const rt_hit *__restrict__ hits, size_t n, const uint32_t *__restrict__ first,
                           uint32_t meshes, uint32_t *__restrict__ mesh_id, uint32_t *__restrict__ local_id) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t prim = hits[i].prim;
    uint32_t m = RT_NO_HIT, l = RT_NO_HIT;
    if (prim != RT_NO_HIT && meshes > 0) {
        uint32_t lo = 0, hi = meshes;  // upper bound of prim in first[0..meshes)
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (first[mid] <= prim) lo = mid + 1;
            else hi = mid;
        }
        if (lo > 0) {
            m = lo - 1;
            l = 3u * (prim - first[m]);
        }
    }
    if (mesh_id) mesh_id[i] = m;
    if (local_id) local_id[i] = l;
}

}  // namespace rgb

using namespace rgb;

namespace {

// Records per chunk of the pipelined host-buffer path (rays, or segments for rt_visible,
// whose per-stream scratch is sized by it too).
constexpr size_t kHostChunk = size_t(1) << 21;

// The kernel streams of the pipelined host path, chunk c on s[c % n]: consecutive chunks'
// traversals overlap, so that one launch's tail (its last, longest rays, with most of the
// GPU idle) runs beside the next launch instead of before it.
struct KernelStreams {
    static constexpr int n = 1 + rt_ctx::kSide;
    cudaStream_t s[n];
    explicit KernelStreams(const rt_ctx *ctx) {
        s[0] = ctx->stream2;
        for (int i = 0; i < rt_ctx::kSide; ++i) s[1 + i] = ctx->kside[i];
    }
    cudaStream_t operator[](size_t c) const { return s[c % (size_t)n]; }
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int require_built(rt_ctx *ctx) {
    if (!ctx) {
        set_error("null context");
        return RT_ERR_ARG;
    }
    if (!ctx->built || ctx->dirty) {
        set_error("rt_update_hierarchy must be called after the last rt_add_mesh");
        return RT_ERR_STATE;
    }
    return RT_OK;
}

// The traversal kernels read rays and write hits as 16-byte vectors.
bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

bool is_pageable(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

// Pageable host buffers (a caller's std::vector or numpy array): cudaMemcpyAsync from or to
// pageable memory returns only once the copy is done, so one host thread cannot keep both
// copy directions and the kernels busy. Here the copy-out side runs on a second host thread:
// this thread copies chunk c in and launches its kernel, the other waits for that kernel (an
// event) and copies the chunk's results out; ring buffer b is reused once the second thread
// has finished chunk c - NB.
template <class Fn>
int host_chunked_pageable(rt_ctx *ctx, const void *h_in, size_t in_stride, size_t n, void *h_out, size_t out_stride,
                          size_t chunk, Fn fn) {
    constexpr int NB = rt_ctx::kRing;
    const size_t nchunks = (n + chunk - 1) / chunk;
    cudaStream_t sin = ctx->stream, sout = ctx->stream3;
    const KernelStreams ks(ctx);
    std::atomic<size_t> launched{0}, drained{0};
    std::atomic<int> fail{RT_OK};
    std::string out_msg;
    std::thread out([&]() {
        if (cudaSetDevice(ctx->device) != cudaSuccess) {
            out_msg = "cudaSetDevice failed on the copy-out thread";
            fail.store(RT_ERR_CUDA);
            return;
        }
        for (size_t c = 0; c < nchunks; ++c) {
            while (launched.load(std::memory_order_acquire) <= c) {
                if (fail.load() != RT_OK) return;
                std::this_thread::yield();
            }
            const int b = (int)(c % NB);
            const size_t s = c * chunk, m = (n - s) < chunk ? (n - s) : chunk;
            cudaError_t e = cudaStreamWaitEvent(sout, ctx->ev_k[b], 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(static_cast<char *>(h_out) + s * out_stride, ctx->ring_out[b].ptr, m * out_stride,
                                    cudaMemcpyDeviceToHost, sout);
            if (e == cudaSuccess) e = cudaStreamSynchronize(sout);
            if (e != cudaSuccess) {
                out_msg = std::string("copy-out failed: ") + cudaGetErrorString(e);
                fail.store(RT_ERR_CUDA);
                return;
            }
            drained.store(c + 1, std::memory_order_release);
        }
    });
    int r = RT_OK;
    for (size_t c = 0; c < nchunks && r == RT_OK; ++c) {
        const int b = (int)(c % NB);
        while (c >= (size_t)NB && drained.load(std::memory_order_acquire) < c - NB + 1) {
            if (fail.load() != RT_OK) break;
            std::this_thread::yield();
        }
        if (fail.load() != RT_OK) break;
        const size_t s = c * chunk, m = (n - s) < chunk ? (n - s) : chunk;
        const cudaStream_t sk = ks[c];
        cudaError_t e = cudaMemcpyAsync(ctx->ring_in[b].ptr, static_cast<const char *>(h_in) + s * in_stride,
                                        m * in_stride, cudaMemcpyHostToDevice, sin);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_in[b], sin);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sk, ctx->ev_in[b], 0);
        if (e != cudaSuccess) {
            set_error(std::string("copy-in failed: ") + cudaGetErrorString(e));
            r = RT_ERR_CUDA;
            break;
        }
        r = fn(ctx->ring_in[b].ptr, m, ctx->ring_out[b].ptr, sk);
        if (r == RT_OK && cudaEventRecord(ctx->ev_k[b], sk) != cudaSuccess) {
            set_error("cudaEventRecord failed");
            r = RT_ERR_CUDA;
        }
        if (r == RT_OK) launched.store(c + 1, std::memory_order_release);
    }
    if (r != RT_OK) fail.store(r);
    out.join();
    if (r == RT_OK && fail.load() != RT_OK) {
        set_error(out_msg);
        r = fail.load();
    }
    for (int i = 0; i < ks.n; ++i) RT_CUDA_TRY(cudaStreamSynchronize(ks.s[i]));
    RT_CUDA_TRY(cudaStreamSynchronize(sin));
    if (r != RT_OK) return r;
    return check_status(ctx, sin);
}

// Runs `fn(d_in, count, d_out, stream)` over host buffers in chunks of up to 2M records
// (chunk_plan) through a ring of eight staging buffers: copies in on `stream`, kernels in
// turn on `stream2` and `kside[0]`, copies out on `stream3`, ordered by events, so that both
// copy directions and the kernels stay busy at once (the host link, not the kernels, bounds
// this path). Pinned host buffers get asynchronous DMA; pageable ones go through
// host_chunked_pageable.
template <class Fn>
int host_chunked(rt_ctx *ctx, const void *h_in, size_t in_stride, size_t n, void *h_out, size_t out_stride, Fn fn) {
    constexpr int NB = rt_ctx::kRing;
    const size_t chunk = kHostChunk;
    const size_t cn = n < chunk ? n : chunk;
    if (!ctx->stream3) RT_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream3, cudaStreamNonBlocking));
    for (int i = 0; i < rt_ctx::kSide; ++i)
        if (!ctx->kside[i]) RT_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->kside[i], cudaStreamNonBlocking));
    for (int b = 0; b < NB; ++b) {
        if (ctx->ring_in[b].reserve(cn * in_stride) != RT_OK || ctx->ring_out[b].reserve(cn * out_stride) != RT_OK)
            return RT_ERR_OOM;
        for (cudaEvent_t *e : {&ctx->ev_in[b], &ctx->ev_k[b], &ctx->ev_out[b]})
            if (!*e) RT_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (n > chunk && (is_pageable(h_in) || is_pageable(h_out)))
        return host_chunked_pageable(ctx, h_in, in_stride, n, h_out, out_stride, chunk, fn);
    cudaStream_t sin = ctx->stream, sout = ctx->stream3;
    const KernelStreams ks(ctx);
    const std::vector<size_t> plan = chunk_plan(n, chunk);
    int r = RT_OK;
    size_t s = 0;
    for (size_t c = 0; c < plan.size() && r == RT_OK; s += plan[c], ++c) {
        const int b = (int)(c % NB);
        const size_t m = plan[c];
        const cudaStream_t sk = ks[c];
        // Buffer b is free once the copy-out of the chunk NB before has finished (which
        // itself followed that chunk's kernel).
        if (c >= (size_t)NB) RT_CUDA_TRY(cudaStreamWaitEvent(sin, ctx->ev_out[b], 0));
        RT_CUDA_TRY(cudaMemcpyAsync(ctx->ring_in[b].ptr, static_cast<const char *>(h_in) + s * in_stride, m * in_stride,
                                    cudaMemcpyHostToDevice, sin));
        RT_CUDA_TRY(cudaEventRecord(ctx->ev_in[b], sin));
        RT_CUDA_TRY(cudaStreamWaitEvent(sk, ctx->ev_in[b], 0));
        r = fn(ctx->ring_in[b].ptr, m, ctx->ring_out[b].ptr, sk);
        if (r != RT_OK) break;
        RT_CUDA_TRY(cudaEventRecord(ctx->ev_k[b], sk));
        RT_CUDA_TRY(cudaStreamWaitEvent(sout, ctx->ev_k[b], 0));
        RT_CUDA_TRY(cudaMemcpyAsync(static_cast<char *>(h_out) + s * out_stride, ctx->ring_out[b].ptr, m * out_stride,
                                    cudaMemcpyDeviceToHost, sout));
        RT_CUDA_TRY(cudaEventRecord(ctx->ev_out[b], sout));
    }
    RT_CUDA_TRY(cudaStreamSynchronize(sout));
    for (int i = 0; i < ks.n; ++i) RT_CUDA_TRY(cudaStreamSynchronize(ks.s[i]));
    RT_CUDA_TRY(cudaStreamSynchronize(sin));
    if (r != RT_OK) return r;
    return check_status(ctx, sin);
}

}  // namespace

extern "C" {

const char *rt_last_error(void) { return g_last_error.c_str(); }

int rt_create(rt_ctx **out, int device) {
    clear_error();
    if (!out) {
        set_error("null output pointer");
        return RT_ERR_ARG;
    }
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    DeviceGuard g(device);
    rt_ctx *ctx = new rt_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev_a) != cudaSuccess || cudaEventCreate(&ctx->ev_b) != cudaSuccess) {
        set_error(std::string("stream/event creation failed: ") + cudaGetErrorString(cudaGetLastError()));
        delete ctx;
        return RT_ERR_CUDA;
    }
    // Status word of the host-buffer calls at 0, three traversal fetch counters at 8, 16, 24,
    // status word of the asynchronous calls at 32.
    if (ctx->d_status.reserve(64) != RT_OK) {
        delete ctx;
        return RT_ERR_OOM;
    }
    cudaMemset(ctx->d_status.ptr, 0, 64);
    *out = ctx;
    return RT_OK;
}

int rt_destroy(rt_ctx *ctx) {
    if (!ctx) return RT_OK;
    DeviceGuard g(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->d_nodes.release();
    ctx->d_tris.release();
    ctx->d_verts.release();
    ctx->d_status.release();
    ctx->d_out2.release();
    ctx->d_mesh_first.release();
    ctx->d_info_stage.release();
    if (ctx->stream2) {
        cudaStreamSynchronize(ctx->stream2);
        cudaStreamDestroy(ctx->stream2);
    }
    if (ctx->ev_a) cudaEventDestroy(ctx->ev_a);
    if (ctx->ev_b) cudaEventDestroy(ctx->ev_b);
    if (ctx->stream3) {
        cudaStreamSynchronize(ctx->stream3);
        cudaStreamDestroy(ctx->stream3);
    }
    for (int i = 0; i < rt_ctx::kSide; ++i)
        if (ctx->kside[i]) {
            cudaStreamSynchronize(ctx->kside[i]);
            cudaStreamDestroy(ctx->kside[i]);
        }
    for (int b = 0; b < rt_ctx::kRing; ++b) {
        ctx->ring_in[b].release();
        ctx->ring_out[b].release();
        for (cudaEvent_t e : {ctx->ev_in[b], ctx->ev_k[b], ctx->ev_out[b]})
            if (e) cudaEventDestroy(e);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RT_OK;
}

int rt_add_mesh(rt_ctx *ctx, const float *positions, size_t vertex_count, const uint32_t *indices, size_t index_count,
                const float *model, uint32_t *mesh_id) {
    clear_error();
    if (!ctx || (vertex_count && !positions) || (index_count && !indices)) {
        set_error("null argument");
        return RT_ERR_ARG;
    }
    if (index_count % 3) {
        set_error("index_count must be a multiple of 3");
        return RT_ERR_ARG;
    }
    const uint64_t total_tris = ctx->h_indices.size() / 3 + index_count / 3;
    if (total_tris >= 0x7FFFFFFFull || ctx->h_positions.size() / 3 + vertex_count >= 0xFFFFFFFFull) {
        set_error("too many triangles or vertices for 32-bit ids");
        return RT_ERR_ARG;
    }
    for (size_t i = 0; i < index_count; ++i) {
        if (indices[i] >= vertex_count) {
            set_error("index " + std::to_string(i) + " out of range");
            return RT_ERR_ARG;
        }
    }
    MeshRecord rec;
    rec.first_vertex = ctx->h_positions.size() / 3;
    rec.vertex_count = vertex_count;
    rec.first_tri = ctx->h_indices.size() / 3;
    rec.tri_count = index_count / 3;
    rec.identity = true;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            const float v = model ? model[4 * c + r] : (c == r ? 1.0f : 0.0f);
            rec.model[4 * c + r] = v;
            // Raycaster.cpp:22: the transform is skipped only for the exact identity.
            if (v != (c == r ? 1.0f : 0.0f)) rec.identity = false;
        }
    ctx->h_positions.insert(ctx->h_positions.end(), positions, positions + 3 * vertex_count);
    const uint32_t off = (uint32_t)rec.first_vertex;
    const size_t base = ctx->h_indices.size();
    ctx->h_indices.resize(base + index_count);
    for (size_t i = 0; i < index_count; ++i) ctx->h_indices[base + i] = indices[i] + off;
    ctx->meshes.push_back(rec);
    ctx->dirty = true;
    if (mesh_id) *mesh_id = (uint32_t)(ctx->meshes.size() - 1);
    return RT_OK;
}

int rt_update_hierarchy(rt_ctx *ctx) {
    clear_error();
    if (!ctx) {
        set_error("null context");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    const int r = build_hierarchy(ctx);
    if (r != RT_OK) return r;
    if (ctx->depth > 256) {
        set_error("hierarchy deeper than the traversal stack (256)");
        return RT_ERR_OVERFLOW;
    }
    std::vector<uint32_t> first(ctx->meshes.size());
    for (size_t m = 0; m < first.size(); ++m) first[m] = (uint32_t)ctx->meshes[m].first_tri;
    if (ctx->d_mesh_first.reserve(first.size() * sizeof(uint32_t) + 16) != RT_OK) return RT_ERR_OOM;
    if (!first.empty())
        RT_CUDA_TRY(cudaMemcpy(ctx->d_mesh_first.ptr, first.data(), first.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice));
    ctx->built = true;
    ctx->dirty = false;
    return RT_OK;
}

int rt_intersect(rt_ctx *ctx, const rt_ray *rays, size_t n, rt_hit *hits, void *stream, uint32_t flags) {
    clear_error();
    int r = require_built(ctx);
    if (r != RT_OK) return r;
    if (n && (!rays || !hits)) {
        set_error("null rays or hits");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        if (!aligned16(rays) || !aligned16(hits)) {
            set_error("device ray and hit buffers must be 16-byte aligned");
            return RT_ERR_ARG;
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        return trace_closest(ctx, rays, n, hits, st);
    }
    return host_chunked(ctx, rays, sizeof(rt_ray), n, hits, sizeof(rt_hit),
                        [ctx](void *in, size_t m, void *out, cudaStream_t st) {
                            return trace_closest(ctx, static_cast<const rt_ray *>(in), m, static_cast<rt_hit *>(out), st);
                        });
}

int rt_intersect_any(rt_ctx *ctx, const rt_ray *rays, size_t n, uint8_t *occluded, void *stream, uint32_t flags) {
    clear_error();
    int r = require_built(ctx);
    if (r != RT_OK) return r;
    if (n && (!rays || !occluded)) {
        set_error("null rays or output");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        if (!aligned16(rays)) {
            set_error("device ray buffers must be 16-byte aligned");
            return RT_ERR_ARG;
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        return trace_any(ctx, rays, n, occluded, st);
    }
    return host_chunked(ctx, rays, sizeof(rt_ray), n, occluded, 1,
                        [ctx](void *in, size_t m, void *out, cudaStream_t st) {
                            return trace_any(ctx, static_cast<const rt_ray *>(in), m, static_cast<uint8_t *>(out), st);
                        });
}

int rt_visible(rt_ctx *ctx, const float *segs, size_t n, uint8_t *visible, void *stream, uint32_t flags) {
    clear_error();
    int r = require_built(ctx);
    if (r != RT_OK) return r;
    if (n && (!segs || !visible)) {
        set_error("null segments or output");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    // Scratch rays: one region per stream of the pipelined host path (reserved up front,
    // never reallocated while work is in flight).
    const size_t chunk = kHostChunk;
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    const size_t region = dev ? n : (n < chunk ? n : chunk);
    if (ctx->d_out2.reserve((dev ? 1 : 2 + rt_ctx::kSide) * region * sizeof(rt_ray) + 16) != RT_OK)
        return RT_ERR_OOM;
    auto run = [ctx, region](const float *d_segs, size_t m, uint8_t *d_vis, cudaStream_t st) -> int {
        // Region 0 for the caller's stream, 1 for stream2, 2.. for the side streams.
        const int side = side_index(ctx, st);
        const size_t k = st == ctx->stream2 ? 1 : (side >= 0 ? (size_t)(2 + side) : 0);
        rt_ray *d_r = ctx->d_out2.as<rt_ray>() + k * region;
        int rr = segments_to_rays(d_segs, m, d_r, st);
        if (rr != RT_OK) return rr;
        rr = trace_any(ctx, d_r, m, d_vis, st);
        if (rr != RT_OK) return rr;
        return invert_bytes(d_vis, m, st);
    };
    if (dev) return run(segs, n, visible, static_cast<cudaStream_t>(stream));
    return host_chunked(ctx, segs, 6 * sizeof(float), n, visible, 1,
                        [run](void *in, size_t m, void *out, cudaStream_t st) {
                            return run(static_cast<const float *>(in), m, static_cast<uint8_t *>(out), st);
                        });
}

int rt_count_visits(rt_ctx *ctx, const rt_ray *rays, size_t n, uint32_t *node_visits, uint32_t *tri_visits,
                    void *stream, uint32_t flags) {
    clear_error();
    int r = require_built(ctx);
    if (r != RT_OK) return r;
    if (n && (!rays || !node_visits || !tri_visits)) {
        set_error("null argument");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        if (!aligned16(rays)) {
            set_error("device ray buffers must be 16-byte aligned");
            return RT_ERR_ARG;
        }
        if (ctx->d_out2.reserve(n * sizeof(rt_hit)) != RT_OK) return RT_ERR_OOM;
        return trace_count(ctx, rays, n, node_visits, tri_visits, ctx->d_out2.as<rt_hit>(),
                           static_cast<cudaStream_t>(stream));
    }
    cudaStream_t st = ctx->stream;
    DevBuf dr, dn, dt, dh;
    if (dr.reserve(n * sizeof(rt_ray)) || dn.reserve(n * 4) || dt.reserve(n * 4) || dh.reserve(n * sizeof(rt_hit))) {
        dr.release(); dn.release(); dt.release(); dh.release();
        return RT_ERR_OOM;
    }
    int rc = RT_OK;
    if (cudaMemcpyAsync(dr.ptr, rays, n * sizeof(rt_ray), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = RT_ERR_CUDA;
    if (rc == RT_OK) rc = trace_count(ctx, dr.as<rt_ray>(), n, dn.as<uint32_t>(), dt.as<uint32_t>(), dh.as<rt_hit>(), st);
    if (rc == RT_OK && (cudaMemcpyAsync(node_visits, dn.ptr, n * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                        cudaMemcpyAsync(tri_visits, dt.ptr, n * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                        cudaStreamSynchronize(st) != cudaSuccess))
        rc = RT_ERR_CUDA;
    if (rc == RT_OK) rc = check_status(ctx, st);
    dr.release(); dn.release(); dt.release(); dh.release();
    return rc;
}

int rt_prim_info(const rt_ctx *ctx, uint32_t prim, uint32_t *mesh_id, uint32_t *local_id) {
    clear_error();
    if (!ctx || !mesh_id || !local_id) {
        set_error("null argument");
        return RT_ERR_ARG;
    }
    size_t lo = 0, hi = ctx->meshes.size();
    if (hi == 0 || prim >= ctx->h_indices.size() / 3) {
        set_error("triangle id out of range");
        return RT_ERR_ARG;
    }
    --hi;
    while (lo < hi) {  // last non-empty mesh whose first triangle <= prim
        const size_t mid = (lo + hi + 1) / 2;
        if (ctx->meshes[mid].first_tri <= prim) lo = mid;
        else hi = mid - 1;
    }
    while (ctx->meshes[lo].tri_count == 0 && lo > 0) --lo;
    *mesh_id = (uint32_t)lo;
    *local_id = (uint32_t)(3 * (prim - ctx->meshes[lo].first_tri));
    return RT_OK;
}

int rt_hit_info(rt_ctx *ctx, const rt_hit *hits, size_t n, uint32_t *mesh_ids, uint32_t *local_ids, void *stream,
                uint32_t flags) {
    clear_error();
    int r = require_built(ctx);
    if (r != RT_OK) return r;
    if (n && (!hits || (!mesh_ids && !local_ids))) {
        set_error("null hits or outputs");
        return RT_ERR_ARG;
    }
    if (n == 0) return RT_OK;
    DeviceGuard g(ctx->device);
    const uint32_t meshes = (uint32_t)ctx->meshes.size();
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (flags & RT_FLAG_DEVICE_PTRS) {
        k_hit_info<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            hits, n, ctx->d_mesh_first.as<uint32_t>(), meshes, mesh_ids, local_ids);
        RT_CUDA_TRY(cudaGetLastError());
        return RT_OK;
    }
    // Host buffers: hits in, the two id arrays out, through one staging buffer on the
    // context's stream.
    const size_t in_bytes = n * sizeof(rt_hit), out_bytes = n * sizeof(uint32_t);
    if (ctx->d_info_stage.reserve(in_bytes + 2 * out_bytes) != RT_OK) return RT_ERR_OOM;
    cudaStream_t st = ctx->stream;
    char *base = ctx->d_info_stage.as<char>();
    uint32_t *dm = reinterpret_cast<uint32_t *>(base + in_bytes), *dl = dm + n;
    RT_CUDA_TRY(cudaMemcpyAsync(base, hits, in_bytes, cudaMemcpyHostToDevice, st));
    k_hit_info<<<blocks, 256, 0, st>>>(reinterpret_cast<const rt_hit *>(base), n, ctx->d_mesh_first.as<uint32_t>(),
                                       meshes, mesh_ids ? dm : nullptr, local_ids ? dl : nullptr);
    RT_CUDA_TRY(cudaGetLastError());
    if (mesh_ids) RT_CUDA_TRY(cudaMemcpyAsync(mesh_ids, dm, out_bytes, cudaMemcpyDeviceToHost, st));
    if (local_ids) RT_CUDA_TRY(cudaMemcpyAsync(local_ids, dl, out_bytes, cudaMemcpyDeviceToHost, st));
    RT_CUDA_TRY(cudaStreamSynchronize(st));
    return RT_OK;
}

int rt_get_status(rt_ctx *ctx, void *stream, uint32_t *word) {
    clear_error();
    if (!ctx) {
        set_error("null context");
        return RT_ERR_ARG;
    }
    DeviceGuard g(ctx->device);
    unsigned raw = 0;
    const int r = read_status(ctx->d_status.as<char>() + 32, static_cast<cudaStream_t>(stream), &raw);
    if (word) *word = raw;
    return r;
}

int rt_set_traversal_stack(rt_ctx *ctx, uint32_t entries) {
    clear_error();
    if (!ctx) {
        set_error("null context");
        return RT_ERR_ARG;
    }
    if (entries > 256) {
        set_error("the traversal stack holds at most 256 entries");
        return RT_ERR_ARG;
    }
    ctx->stack_cap = entries;
    return RT_OK;
}

int rt_get_stats(const rt_ctx *ctx, rt_stats *out) {
    clear_error();
    if (!ctx || !out) {
        set_error("null argument");
        return RT_ERR_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    out->triangles = ctx->h_indices.size() / 3;
    out->vertices = ctx->h_positions.size() / 3;
    out->meshes = ctx->meshes.size();
    out->nodes = ctx->n_inner;
    out->leaves = ctx->n_leaves;
    out->device_bytes = ctx->n_inner * sizeof(BvhNode) + ctx->n_tris * sizeof(BvhTri);
    out->build_ms = ctx->build_ms;
    out->sah_cost = ctx->sah_cost;
    return RT_OK;
}

}  // extern "C"
