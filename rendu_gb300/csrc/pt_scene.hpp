// Host-side state of a path-tracer scene and the per-render launch parameters.
#pragma once

#include <memory>
#include <vector>

#include "pt_device.cuh"
#include "rt_context.hpp"

// Feature buffer: PT_AOV floats per pixel out (albedo rgb, normal xyz, distance, standard
// error of the mean luminance), PT_AOV_ACCUM accumulated (the first 7, then the sum and the
// sum of squares of the samples' luminance).
#define PT_AOV 8
#define PT_AOV_ACCUM 9

namespace rgb {

// One render of a call (a batch has many): its scene, camera frame, sampling grid, options.
struct PtJob {
    PtScene scene;
    float corner[3], dx[3], dy[3], eye[3];
    uint32_t W, H, npix, spp, cx, cy, depth, comps;
    float cell_x, cell_y;
    float clamp;  // per-sample clamp (<= 0: none)
    uint32_t seed_lo, seed_hi;
    uint32_t accum_offset;  // first pixel of this job in the accumulation buffer
    int fp64;               // accumulate in the double buffer
    int aov;                // collect first-hit features
};

// Pixels [pixel0, pixel0 + npix) of `job` x samples [s0, s0 + S), laid out sample-major
// from wave path `path0`.
struct PtTile {
    uint32_t job, pixel0, npix, s0, S, path0;
};

// Device buffers and tables of the wave engine (capacity `cap` paths per wave).
struct PtWave {
    float4 *atten, *color;  // atten.w: pdf of the BSDF sample that made the current ray
    float2 *ndc;
    uint32_t *pjob, *ppix, *psamp;  // per path: job, pixel, sample
    rt_ray *qray[2];
    uint32_t *qpath[2];
    rt_hit *hits;
    rt_ray *sray;
    float4 *scontrib;
    uint32_t shadow_cap;  // the second shadow queue starts at this entry
    uint32_t *counters;   // [0], [1] ray queues, [2] analytic-light shadows, [3] emitter/env shadows, [4] wave
    unsigned long long *fetch;  // ray-fetch counter of the persistent traversal
    unsigned long long *stats;  // [0] primary, [1] bounce, [2] shadow rays
    float *accum;               // 3 floats per pixel of every job
    double *accum64;            // 3 doubles per pixel of every job (jobs with fp64)
    float4 *aov0, *aov1;        // per path: albedo.rgb + distance, normal.xyz (jobs with aov)
    float *aov_accum;           // PT_AOV_ACCUM floats per pixel of every job (jobs with aov)
    const PtJob *jobs;
    const JobBvh *bvhs;
    const PtTile *tiles;
    const uint32_t *wave_tiles;  // tiles of wave k: [wave_tiles[k], wave_tiles[k + 1])
    const uint32_t *wave_paths;  // paths of wave k
    unsigned *status;
    uint32_t cap;
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
// The sky's scattering table (res x res, `samples` march steps, half-precision rounding
// optional) and MaterialSky::eval over n cases {origin, direction, sun}.
constexpr uint32_t kSkyTableRes = 512, kSkyTableSamples = 256;
int pt_launch_sky_table(uint32_t res, uint32_t samples, bool half_prec, float4 *out, cudaStream_t st);
int pt_launch_sky_eval(const float4 *table, uint32_t w, uint32_t h, const float *cases, uint32_t n, float *out,
                       cudaStream_t st);
// End of a wave: the wave index advances; with a conditional handle (the wave sequence is the
// body of a graph's while node) the loop goes on while waves remain (counters[5] waves).
int pt_launch_wave_end(const PtWave &w, cudaStream_t st, const cudaGraphConditionalHandle *loop = nullptr);
// counters[5] = the number of waves of this call (read by the graph's loop).
int pt_launch_set_waves(const PtWave &w, uint32_t nwaves, cudaStream_t st);
int pt_launch_raygen(const PtWave &w, cudaStream_t st);
int pt_launch_shade(const PtWave &w, int cur, uint32_t did, bool ext, cudaStream_t st);
int pt_launch_shadow(const PtWave &w, int queue, bool big_stack, cudaStream_t st);
int pt_launch_accumulate(const PtWave &w, cudaStream_t st);
int pt_launch_load(const float *img, uint32_t comps, uint32_t npix, float *accum, double *accum64, cudaStream_t st);
int pt_launch_store(const float *accum, const double *accum64, uint32_t npix, float spp, uint32_t comps, uint32_t ranks,
                    uint32_t rank, float *img, const float *aov_accum, float *aov, cudaStream_t st);
// Closest hit for the wave's ray queue `cur`, each ray against its job's hierarchy.
int trace_closest_batch(const PtWave &w, int cur, bool big_stack, cudaStream_t st);
int trace_closest_batch_prepare(bool big_stack);
// Camera::pose + Camera::pixelShifts (Camera.cpp:10-18, 42-49).
void pixel_shifts(const pt_camera_desc &c, float corner[3], float dx[3], float dy[3], float eye[3]);

// One render request of the engine.
struct JobSpec {
    pt_scene *scene;
    pt_camera_desc camera;
    uint32_t samples, depth;
    uint64_t seed;
    float *image;
    uint32_t width, height, components;
    float clamp;
    int fp64;
    float *aov;  // width x height x 7 output (host or device like the image), or null
    uint32_t ranks = 1, rank = 0;  // pixel split (pt_render_options.ranks / .rank)
};

// Wave-engine tuning (chosen by pt_batch_autotune or defaults).
struct Tuning {
    uint32_t wave_paths;   // capacity of a wave
    uint32_t tile_pixels;  // pixels per tile
    uint32_t max_samples;  // most samples of one pixel in one wave (power of two)
};

Tuning default_tuning();
bool load_tuning(const char *path, Tuning &t);

// Runs renders as waves of one captured CUDA graph: the wave sequence is the body of the
// graph's while node, which loops on the device until the call's last wave, so a whole
// render or batch is one graph launch. Owns every device buffer it uses (grow-only) and the
// instantiated graph, reused while the launch shape is unchanged.
class WaveEngine {
  public:
    explicit WaveEngine(int device) : device_(device) {}
    ~WaveEngine();
    // profile: launch the per-wave sequence directly (not the captured graph) with events
    // between the steps, and report the time of every kernel class in stats->kernel_ms.
    int run(const std::vector<JobSpec> &jobs, int mode, const Tuning &t, bool device_images, cudaStream_t st,
            pt_render_stats *stats, bool profile = false);
    uint64_t capacity() const { return cap_; }  // paths of the wave buffers held

  private:
    int ensure_capacity(uint64_t cap, uint64_t accum_pixels, uint64_t ntiles, uint64_t nwaves, size_t njobs,
                        uint64_t staging_floats, bool fp64, bool aov);
    int capture(const PtWave &w, uint32_t depth, bool ext, bool shadow_a, bool shadow_b, bool big_stack);
    // The per-wave launch sequence on `st`. With `marks`, an event is recorded after every
    // step and `kinds` receives the step's kernel class (PT_KERNEL_*), for per-kernel times.
    // With `loop`, the sequence ends by setting that while-node handle.
    int launch_wave(const PtWave &w, uint32_t depth, bool ext, bool shadow_a, bool shadow_b, bool big_stack,
                    cudaStream_t st, std::vector<cudaEvent_t> *marks, std::vector<int> *kinds,
                    const cudaGraphConditionalHandle *loop = nullptr);
    int device_;
    cudaStream_t capture_stream_ = nullptr;
    DevBuf atten_, color_, ndc_, pjob_, ppix_, psamp_, qray0_, qray1_, qpath0_, qpath1_, hits_, sray_, scontrib_;
    DevBuf counters_, accum_, accum64_, aov0_, aov1_, aov_accum_, aov_staging_, jobs_, bvhs_, tiles_, wave_tiles_,
        wave_paths_, staging_;
    uint64_t cap_ = 0;
    uint64_t generation_ = 0;  // bumped whenever a buffer the graph refers to moves
    cudaGraphExec_t exec_ = nullptr;
    struct Key {
        uint64_t generation, cap;
        uint32_t depth;
        bool ext, shadow_a, shadow_b, big_stack;
    } key_{};
};

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
    float sun[3] = {0.0f, 1.0f, 0.0f};  // ATMOSPHERE: normalised sun direction
    std::vector<float> sky_table;      // ATMOSPHERE: caller's table (RGBA), empty = computed
    uint32_t sky_w = 0, sky_h = 0;
    rgb::DevBuf d_sky;
    rgb::PtScene dev{};

    std::unique_ptr<rgb::WaveEngine> engine;  // runs pt_render

    pt_render_stats last{};
};

struct pt_batch {
    int device = 0;
    std::unique_ptr<rgb::WaveEngine> engine;
    pt_render_stats last{};
};
