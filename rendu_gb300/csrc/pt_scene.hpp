// Host-side state of a path-tracer scene and the per-render launch parameters.
#pragma once

#include <vector>

#include "pt_device.cuh"
#include "rt_context.hpp"

namespace rgb {

// Per-render constants (camera, sampling grid, wave window).
struct PtFrame {
    float corner[3], dx[3], dy[3], eye[3];
    uint32_t W, H, npix, spp, cx, cy, depth;
    float cell_x, cell_y;
    uint32_t s0, S;  // this wave covers sample indices [s0, s0 + S)
    uint32_t seed_lo, seed_hi;
    int mode;     // PT_MODE_REFERENCE / PT_MODE_EXTENDED
    float clamp;  // per-sample clamp (<= 0: none)
};

// Device buffers of one wave (capacity P = npix * S paths).
struct PtWave {
    float4 *atten, *color;
    float2 *ndc;
    rt_ray *qray[2];
    uint32_t *qpath[2];
    rt_hit *hits;
    rt_ray *sray;
    float4 *scontrib;
    uint32_t *counters;  // [0], [1]: ray queues, [2]: analytic-light shadow queue, [3]: emitter/env shadow queue
    uint32_t shadow_cap; // the second shadow queue starts at this entry
    unsigned long long *stats;  // [0] primary, [1] bounce, [2] shadow rays
    float *accum;       // npix x 3
};

struct HostTex {
    uint32_t w, h;
    std::vector<float> rgba;  // w * h * 4
};

struct HostMesh {
    std::vector<float> pos, nrm, tan, bit, uv;
    std::vector<uint32_t> idx;
};

struct HostObject {
    uint32_t mesh, material;
    float model[16];
};

int pt_launch_material(const float *cases, const float *uniforms, uint32_t n, float *out, cudaStream_t st);
int pt_launch_raygen(const PtFrame &f, const PtWave &w, cudaStream_t st);
int pt_launch_trace(rt_ctx *rc, const PtWave &w, int cur, uint32_t cap, cudaStream_t st);
int pt_launch_shade(const PtScene &s, const PtFrame &f, const PtWave &w, int cur, uint32_t did, uint32_t cap,
                    cudaStream_t st);
int pt_launch_shadow(const PtScene &s, const PtWave &w, uint32_t cap, int queue, cudaStream_t st);
int pt_launch_accumulate(const PtFrame &f, const PtWave &w, cudaStream_t st);
int pt_launch_load(const float *img, uint32_t comps, uint32_t npix, float *accum, cudaStream_t st);
int pt_launch_store(const float *accum, uint32_t npix, float spp, uint32_t comps, float *img, cudaStream_t st);

}  // namespace rgb

struct pt_scene {
    int device = 0;
    rt_ctx *rc = nullptr;
    std::vector<rgb::HostTex> textures;
    std::vector<rgb::HostMesh> meshes;
    std::vector<pt_material_desc> materials;
    std::vector<rgb::HostObject> objects;
    std::vector<pt_light_desc> lights;
    int bg_mode = PT_BG_COLOR;
    float bg_color[3] = {0, 0, 0};
    uint32_t bg_tex[6] = {0, 0, 0, 0, 0, 0};
    bool committed = false;

    // Scene pools on the device.
    rgb::DevBuf d_objects, d_meshes, d_materials, d_tex, d_texels, d_positions, d_normals, d_tangents, d_bitangents,
        d_uvs, d_indices, d_lights, d_emitters, d_emitter_cdf, d_env_marg, d_env_cond, d_env_func;
    int env_tex = -1;
    float env_intensity = 1.0f;
    rgb::PtScene dev{};

    // Wave buffers (grow-only).
    rgb::DevBuf w_atten, w_color, w_ndc, w_qray0, w_qray1, w_qpath0, w_qpath1, w_hits, w_sray, w_scontrib,
        w_counters, w_stats, w_accum, w_image;
    size_t wave_cap = 0;
    size_t accum_cap = 0;

    pt_render_stats last{};
};
