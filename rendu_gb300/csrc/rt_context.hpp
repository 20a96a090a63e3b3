// Host-side state of a raycaster context and small utilities shared by the C-ABI units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "rendu_gb300.h"
#include "rt_common.cuh"

namespace rgb {

// Thread-local message of the last failure (rt_last_error).
void set_error(const std::string &msg);
void clear_error();

// Device buffer that only grows; freed with the owner.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);  // RT_OK or RT_ERR_OOM
    void release();
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

struct MeshRecord {
    uint64_t first_vertex;
    uint64_t vertex_count;
    uint64_t first_tri;
    uint64_t tri_count;
    float model[16];  // column-major
    bool identity;
};

}  // namespace rgb

struct rt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;   // the context's own stream
    cudaStream_t stream2 = nullptr;  // kernels of the pipelined host-buffer path
    // Host copies appended by rt_add_mesh (raw positions; indices already offset).
    std::vector<float> h_positions;
    std::vector<uint32_t> h_indices;
    std::vector<rgb::MeshRecord> meshes;
    bool dirty = true;  // meshes added since the last build
    bool built = false;

    // Device hierarchy.
    rgb::DevBuf d_nodes;   // BvhNode[n_inner] (at least 1: a root, possibly wrapping a leaf)
    rgb::DevBuf d_tris;    // BvhTri[n_tris] in leaf order
    rgb::DevBuf d_verts;   // float3 transformed vertices (kept for the path tracer)
    // 64 bytes: status word of the host-buffer calls at 0, traversal fetch counters at 8
    // (the caller's streams), 16 (`stream`), 24 (`stream2`) and 40 (`kside[0]`),
    // status word of the asynchronous calls (device pointers on the caller's stream,
    // rt_visible_noalloc) at 32, read and cleared by rt_get_status.
    rgb::DevBuf d_status;
    uint32_t stack_cap = 0;  // rt_set_traversal_stack: 0 = the hierarchy's exact bound
    uint64_t n_tris = 0;
    uint64_t n_inner = 0;
    uint64_t n_leaves = 0;
    int depth = 0;
    float build_ms = 0.0f;
    float sah_cost = 0.0f;
    float root_box[6] = {0, 0, 0, 0, 0, 0};

    // Scratch of rt_visible (converted rays) and rt_count_visits (hits).
    rgb::DevBuf d_out2;
    // First triangle of every mesh (addMesh order), uploaded by rt_update_hierarchy for
    // rt_hit_info; and the staging of rt_hit_info's host-buffer path.
    rgb::DevBuf d_mesh_first;
    rgb::DevBuf d_info_stage;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    // Host-buffer pipeline: copy-in on `stream`, kernels in turn on `stream2` and `kside`,
    // copy-out on `stream3`, through a ring of staging buffers (created on first use).
    static constexpr int kRing = 8;
    static constexpr int kSide = 1;
    cudaStream_t stream3 = nullptr;
    cudaStream_t kside[kSide] = {};
    rgb::DevBuf ring_in[kRing], ring_out[kRing];
    cudaEvent_t ev_in[kRing] = {}, ev_k[kRing] = {}, ev_out[kRing] = {};
};

namespace rgb {
// Launchers used across units (all asynchronous on `stream`).
int trace_closest(rt_ctx *ctx, const rt_ray *d_rays, size_t n, rt_hit *d_hits, cudaStream_t stream);
int trace_any(rt_ctx *ctx, const rt_ray *d_rays, size_t n, uint8_t *d_occ, cudaStream_t stream);
// Closest hit for a device-side queue: the length is read from d_count (at most cap).
int trace_closest_queue(rt_ctx *ctx, const rt_ray *d_rays, const uint32_t *d_count, uint32_t cap, rt_hit *d_hits,
                        cudaStream_t stream);
int check_status(rt_ctx *ctx, cudaStream_t stream);  // reads and clears the device status word

// The status word a traversal on `st` reports into: the host-buffer path's own streams use
// the word check_status reads; every other stream (the caller's) the word rt_get_status reads.
// Which of the pipeline's extra kernel streams `st` is, or -1.
inline int side_index(const rt_ctx *ctx, cudaStream_t st) {
    for (int i = 0; st && i < rt_ctx::kSide; ++i)
        if (st == ctx->kside[i]) return i;
    return -1;
}

inline unsigned *status_word(rt_ctx *ctx, cudaStream_t st) {
    const bool own = st == ctx->stream || st == ctx->stream2 || side_index(ctx, st) >= 0;
    return reinterpret_cast<unsigned *>(ctx->d_status.as<char>() + (own ? 0 : 32));
}

// Entries of the traversal stack the kernels are instantiated with (2, 64 or 256): the
// smallest that holds the hierarchy's exact bound, or the cap set by rt_set_traversal_stack
// (the 2-entry kernels only exist for that diagnostic).
// Byte offset in d_status of the fetch counter of a persistent traversal on `st`: one per
// stream the context launches on, since the pipelined host path runs traversals on two
// streams at once, and the caller's stream may run one beside them.
inline size_t fetch_counter_offset(const rt_ctx *ctx, cudaStream_t st) {
    if (st == ctx->stream) return 16;
    if (st == ctx->stream2) return 24;
    const int i = side_index(ctx, st);
    return i >= 0 ? 40 + 8 * (size_t)i : 8;
}

inline int traversal_stack(const rt_ctx *ctx) {
    const int need = ctx->stack_cap ? (int)ctx->stack_cap : ctx->depth;
    return need <= 2 && ctx->stack_cap ? 2 : (need <= 64 ? 64 : 256);
}
}  // namespace rgb

#define RT_CUDA_TRY(expr)                                                                    \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess) {                                                             \
            rgb::set_error(std::string(#expr " failed: ") + cudaGetErrorString(_e));        \
            return RT_ERR_CUDA;                                                              \
        }                                                                                    \
    } while (0)
