// Wave engine: runs one render (pt_render) or a batch of renders (pt_batch_render) as a
// sequence of waves whose launch sequence is captured once as the body of a CUDA graph's
// while node, which loops over the call's waves on the device (one graph launch per call).
//
// Scheduling. Each job is cut into tiles of at most `tile_pixels` pixels x S samples
// (S = a power of two <= the job's sample count and <= `max_samples`). Tiles are issued
// pass by pass (all jobs' first S samples, then the next S, ...) and packed greedily into
// waves of at most `wave_paths` paths; a wave never holds two tiles of the same pixels, so
// the per-pixel accumulation is race-free and in sample order (PathTracer.cpp:288).
// A single render with the default tuning is one tile per wave: every pixel x S samples.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "pt_scene.hpp"

namespace rgb {

namespace {
struct V3 {
    float x, y, z;
};
V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 vadd(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 vscale(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
float vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 vcross(V3 x, V3 y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
V3 vnormalize(V3 v) {
    const float s = 1.0f / std::sqrt(vdot(v, v));
    return {v.x * s, v.y * s, v.z * s};
}
}  // namespace

// Camera::pose (Camera.cpp:10-18) followed by Camera::pixelShifts (Camera.cpp:42-49), in
// glm's operation order (this unit is compiled without floating-point contraction).
void pixel_shifts(const pt_camera_desc &c, float corner[3], float dx[3], float dy[3], float eye[3]) {
    const V3 e{c.eye[0], c.eye[1], c.eye[2]}, ce{c.center[0], c.center[1], c.center[2]};
    V3 up = vnormalize(V3{c.up[0], c.up[1], c.up[2]});
    const V3 view = vnormalize(vsub(ce, e));
    const V3 right = vcross(view, up);
    up = vcross(right, view);
    const float hs = std::tan(0.5f * c.fov);
    const float ws = c.ratio * hs;
    const V3 de = vsub(ce, e);
    const float dist = std::sqrt(vdot(de, de));
    const V3 k = vadd(vscale(-ws, right), vscale(hs, up));
    const V3 co = vadd(ce, vscale(dist, k));
    const V3 ddx = vscale(2.0f * ws * dist, right);
    const V3 ddy = vscale(-2.0f * hs * dist, up);
    corner[0] = co.x; corner[1] = co.y; corner[2] = co.z;
    dx[0] = ddx.x; dx[1] = ddx.y; dx[2] = ddx.z;
    dy[0] = ddy.x; dy[1] = ddy.y; dy[2] = ddy.z;
    eye[0] = e.x; eye[1] = e.y; eye[2] = e.z;
}

namespace {
uint32_t floor_pow2(uint64_t v) {
    uint32_t p = 1;
    while ((uint64_t)p * 2 <= v && p < (1u << 30)) p *= 2;
    return p;
}
}  // namespace

WaveEngine::~WaveEngine() {
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device_) cudaSetDevice(device_);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
    for (DevBuf *b : {&atten_, &color_, &ndc_, &pjob_, &ppix_, &psamp_, &qray0_, &qray1_, &qpath0_, &qpath1_, &hits_,
                      &sray_, &scontrib_, &counters_, &accum_, &accum64_, &aov0_, &aov1_, &aov_accum_, &aov_staging_,
                      &jobs_, &bvhs_, &tiles_, &wave_tiles_, &wave_paths_, &staging_})
        b->release();
    if (prev >= 0 && prev != device_) cudaSetDevice(prev);
}

int WaveEngine::ensure_capacity(uint64_t cap, uint64_t accum_pixels, uint64_t ntiles, uint64_t nwaves, size_t njobs,
                                uint64_t staging_floats, bool fp64, bool aov) {
    bool moved = false;
    int r = RT_OK;
    auto grow = [&](DevBuf &b, uint64_t bytes) {
        if (r != RT_OK || (b.ptr && bytes <= b.bytes)) return;
        moved = true;
        r = b.reserve(bytes);
    };
    if (cap > cap_) {
        grow(atten_, cap * 16); grow(color_, cap * 16); grow(ndc_, cap * 8);
        grow(pjob_, cap * 4); grow(ppix_, cap * 4); grow(psamp_, cap * 4);
        grow(qray0_, cap * 32); grow(qray1_, cap * 32); grow(qpath0_, cap * 4); grow(qpath1_, cap * 4);
        grow(hits_, cap * 16); grow(sray_, 2 * cap * 32); grow(scontrib_, 2 * cap * 16);
        if (r != RT_OK) return r;
        cap_ = cap;
    }
    grow(counters_, 128);
    grow(accum_, std::max<uint64_t>(accum_pixels, 1) * 12);
    grow(jobs_, std::max<size_t>(njobs, 1) * sizeof(PtJob));
    grow(bvhs_, std::max<size_t>(njobs, 1) * sizeof(JobBvh));
    grow(tiles_, std::max<uint64_t>(ntiles, 1) * sizeof(PtTile));
    grow(wave_tiles_, (nwaves + 1) * 4);
    grow(wave_paths_, std::max<uint64_t>(nwaves, 1) * 4);
    if (staging_floats) grow(staging_, staging_floats * 4);
    if (fp64) grow(accum64_, std::max<uint64_t>(accum_pixels, 1) * 24);
    if (aov) {
        grow(aov0_, cap_ * 16);
        grow(aov1_, cap_ * 16);
        grow(aov_accum_, std::max<uint64_t>(accum_pixels, 1) * 4 * PT_AOV_ACCUM);
        grow(aov_staging_, std::max<uint64_t>(accum_pixels, 1) * 4 * PT_AOV);
    }
    if (moved) ++generation_;
    return r;
}

int WaveEngine::launch_wave(const PtWave &w, uint32_t depth, bool ext, bool shadow_a, bool shadow_b, bool big_stack,
                            cudaStream_t cs, std::vector<cudaEvent_t> *marks, std::vector<int> *kinds,
                            const cudaGraphConditionalHandle *loop) {
    auto mark = [&](int kind) -> int {
        if (!marks) return RT_OK;
        cudaEvent_t e = nullptr;
        RT_CUDA_TRY(cudaEventCreate(&e));
        marks->push_back(e);
        kinds->push_back(kind);
        RT_CUDA_TRY(cudaEventRecord(e, cs));
        return RT_OK;
    };
    int r = mark(-1);
    if (r == RT_OK) r = pt_launch_raygen(w, cs);  // also starts the wave's queues
    if (r == RT_OK) r = mark(PT_KERNEL_RAYGEN);
    int cur = 0;
    for (uint32_t did = 0; r == RT_OK && did < depth; ++did) {
        // (the traversal also empties the queues the shading appends to)
        r = trace_closest_batch(w, cur, big_stack, cs);
        if (r == RT_OK) r = mark(PT_KERNEL_TRACE);
        if (r == RT_OK) r = pt_launch_shade(w, cur, did, ext, cs);
        if (r == RT_OK) r = mark(PT_KERNEL_SHADE);
        if (r == RT_OK && shadow_a) r = pt_launch_shadow(w, 0, big_stack, cs);
        if (r == RT_OK && shadow_b) r = pt_launch_shadow(w, 1, big_stack, cs);
        if (r == RT_OK && (shadow_a || shadow_b)) r = mark(PT_KERNEL_SHADOW);
        cur ^= 1;
    }
    if (r == RT_OK) r = pt_launch_accumulate(w, cs);
    if (r == RT_OK) r = pt_launch_wave_end(w, cs, loop);
    if (r == RT_OK) r = mark(PT_KERNEL_ACCUMULATE);
    return r;
}

int WaveEngine::capture(const PtWave &w, uint32_t depth, bool ext, bool shadow_a, bool shadow_b, bool big_stack) {
    if (!capture_stream_) RT_CUDA_TRY(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
    if (exec_) {
        RT_CUDA_TRY(cudaGraphExecDestroy(exec_));
        exec_ = nullptr;
    }
    cudaStream_t cs = capture_stream_;
    // graph = { while (waves remain) { wave } }: the handle starts at 1 on every launch (a
    // call has at least one wave) and the wave's last kernel sets it.
    cudaGraph_t graph = nullptr;
    RT_CUDA_TRY(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle loop = 0;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};  // the rest zero
    cudaGraphNode_t node = nullptr;
    cudaError_t e = cudaGraphConditionalHandleCreate(&loop, graph, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
        cp.conditional.handle = loop;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    }
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        cudaGetLastError();
        set_error(std::string("wave loop graph set-up failed: ") + cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    const int r = launch_wave(w, depth, ext, shadow_a, shadow_b, big_stack, cs, nullptr, nullptr, &loop);
    cudaGraph_t body = nullptr;
    e = cudaStreamEndCapture(cs, &body);
    if (r != RT_OK) {
        cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        set_error(std::string("graph capture failed: ") + cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    const cudaError_t e2 = cudaGraphInstantiate(&exec_, graph, 0);
    cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) {
        exec_ = nullptr;
        set_error(std::string("graph instantiation failed: ") + cudaGetErrorString(e2));
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

int WaveEngine::run(const std::vector<JobSpec> &jobs, int mode, const Tuning &tn, bool device_images, cudaStream_t st,
                    pt_render_stats *stats, bool profile) {
    if (jobs.empty()) return RT_OK;
    const bool ext = mode == PT_MODE_EXTENDED;
    // Wave capacity: the tuning's, but no more than the call's paths (the path state and the
    // queues are sized by it, so a small render does not hold a large wave's memory).
    uint64_t total_paths = 0;
    for (const JobSpec &js : jobs)
        total_paths += (uint64_t)js.width * js.height *
                       (uint64_t)std::pow(2.0, std::round(std::log2((float)std::max<uint32_t>(js.samples, 1u))));
    const uint64_t cap = std::max<uint64_t>(std::min<uint64_t>(tn.wave_paths, total_paths), 1u << 12);
    // ---- per-job set-up -------------------------------------------------------------------
    std::vector<PtJob> hj(jobs.size());
    std::vector<JobBvh> hb(jobs.size());
    std::vector<uint32_t> S(jobs.size()), chunk(jobs.size()), passes(jobs.size());
    uint64_t accum_pixels = 0, staging = 0;
    uint32_t depth = 0, max_passes = 0;
    bool shadow_a = false, shadow_b = false, big_stack = false, any_fp64 = false, any_aov = false;
    for (size_t j = 0; j < jobs.size(); ++j) {
        const JobSpec &js = jobs[j];
        PtJob &J = hj[j];
        std::memset(&J, 0, sizeof(J));
        J.scene = js.scene->dev;
        pixel_shifts(js.camera, J.corner, J.dx, J.dy, J.eye);
        J.W = js.width;
        J.H = js.height;
        J.npix = js.width * js.height;
        J.comps = js.components;
        // Power-of-two sample count and stratification grid (PathTracer.cpp:169-178, 57-69).
        J.spp = (uint32_t)std::pow(2.0, std::round(std::log2((float)js.samples)));
        const int k = (int)std::floor(std::log2((double)J.spp));
        J.cx = (uint32_t)std::pow(2, k / 2);
        J.cy = J.cx;
        if (k % 2 == 1) {
            J.cx = (uint32_t)std::pow(2, (k + 1) / 2);
            J.cy = (uint32_t)std::pow(2, (k - 1) / 2);
        }
        J.cell_x = 1.0f / (float)J.cx;
        J.cell_y = 1.0f / (float)J.cy;
        J.depth = js.depth;
        J.clamp = js.clamp;
        J.seed_lo = (uint32_t)js.seed;
        J.seed_hi = (uint32_t)(js.seed >> 32);
        J.accum_offset = (uint32_t)accum_pixels;
        J.fp64 = js.fp64 ? 1 : 0;
        J.aov = js.aov ? 1 : 0;
        any_fp64 |= js.fp64 != 0;
        any_aov |= js.aov != nullptr;
        accum_pixels += J.npix;
        staging += (uint64_t)J.npix * J.comps;
        hb[j] = JobBvh{J.scene.nodes, J.scene.tris, J.scene.empty, 0};
        depth = std::max(depth, J.depth);
        shadow_a |= J.scene.nlights > 0;
        shadow_b |= ext && (J.scene.nemitters > 0 || J.scene.env_tex >= 0);
        big_stack |= J.scene.big_stack != 0;
        chunk[j] = (uint32_t)std::min<uint64_t>(std::max<uint32_t>(tn.tile_pixels, 1u), J.npix);
        chunk[j] = (uint32_t)std::min<uint64_t>(chunk[j], cap);
        S[j] = std::min<uint32_t>(J.spp, std::max<uint32_t>(floor_pow2(tn.max_samples), 1u));
        S[j] = std::min<uint32_t>(S[j], floor_pow2(cap / chunk[j]));
        passes[j] = J.spp / S[j];
        max_passes = std::max(max_passes, passes[j]);
    }
    if (accum_pixels >= (1ull << 31)) {
        set_error("batch too large");
        return RT_ERR_ARG;
    }
    // ---- tiles and waves -----------------------------------------------------------------------
    // Pixel ranges of every job: chunks of `chunk` pixels, or under a rank split the chunks of
    // this rank's PT_RANK_TILE_PIXELS tiles only.
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> ranges(jobs.size());
    for (size_t j = 0; j < jobs.size(); ++j) {
        const uint32_t npix = hj[j].npix, ranks = std::max<uint32_t>(jobs[j].ranks, 1u);
        if (ranks == 1) {
            for (uint32_t p0 = 0; p0 < npix; p0 += chunk[j]) ranges[j].push_back({p0, std::min(chunk[j], npix - p0)});
            continue;
        }
        const uint32_t c = std::min<uint32_t>(chunk[j], PT_RANK_TILE_PIXELS);
        for (uint32_t t0 = jobs[j].rank * PT_RANK_TILE_PIXELS; t0 < npix; t0 += ranks * PT_RANK_TILE_PIXELS) {
            const uint32_t t1 = std::min<uint32_t>(t0 + PT_RANK_TILE_PIXELS, npix);
            for (uint32_t p0 = t0; p0 < t1; p0 += c) ranges[j].push_back({p0, std::min(c, t1 - p0)});
        }
    }
    std::vector<PtTile> tiles;
    std::vector<uint32_t> wave_tiles{0}, wave_paths;
    std::vector<std::vector<uint32_t>> last_wave(jobs.size());
    for (size_t j = 0; j < jobs.size(); ++j) last_wave[j].assign(ranges[j].size(), UINT32_MAX);
    uint64_t in_wave = 0;
    auto close_wave = [&]() {
        if (in_wave == 0) return;
        wave_paths.push_back((uint32_t)in_wave);
        wave_tiles.push_back((uint32_t)tiles.size());
        in_wave = 0;
    };
    for (uint32_t pass = 0; pass < max_passes; ++pass) {
        for (size_t j = 0; j < jobs.size(); ++j) {
            if (pass >= passes[j]) continue;
            for (uint32_t c = 0; c < last_wave[j].size(); ++c) {
                const uint32_t p0 = ranges[j][c].first;
                const uint32_t np = ranges[j][c].second;
                const uint64_t paths = (uint64_t)np * S[j];
                const uint32_t wave = (uint32_t)wave_paths.size();
                if (in_wave + paths > cap || last_wave[j][c] == wave) close_wave();
                last_wave[j][c] = (uint32_t)wave_paths.size();
                tiles.push_back(PtTile{(uint32_t)j, p0, np, pass * S[j], S[j], (uint32_t)in_wave});
                in_wave += paths;
            }
        }
    }
    close_wave();
    const uint64_t nwaves = wave_paths.size();
    int r = ensure_capacity(cap, accum_pixels, tiles.size(), nwaves, jobs.size(), device_images ? 0 : staging, any_fp64,
                            any_aov);
    if (r != RT_OK) return r;

    PtWave w{};
    w.atten = atten_.as<float4>();
    w.color = color_.as<float4>();
    w.ndc = ndc_.as<float2>();
    w.pjob = pjob_.as<uint32_t>();
    w.ppix = ppix_.as<uint32_t>();
    w.psamp = psamp_.as<uint32_t>();
    w.qray[0] = qray0_.as<rt_ray>();
    w.qray[1] = qray1_.as<rt_ray>();
    w.qpath[0] = qpath0_.as<uint32_t>();
    w.qpath[1] = qpath1_.as<uint32_t>();
    w.hits = hits_.as<rt_hit>();
    w.sray = sray_.as<rt_ray>();
    w.scontrib = scontrib_.as<float4>();
    w.shadow_cap = (uint32_t)cap_;
    w.counters = counters_.as<uint32_t>();
    w.fetch = reinterpret_cast<unsigned long long *>(counters_.as<char>() + 32);
    w.stats = reinterpret_cast<unsigned long long *>(counters_.as<char>() + 64);
    w.status = reinterpret_cast<unsigned *>(counters_.as<char>() + 96);
    w.accum = accum_.as<float>();
    // The optional buffers go into the captured graph whether or not this call uses them:
    // a graph replayed by a later call whose jobs do use them must hold their addresses.
    // They are null only until first allocated, and that allocation forces a new capture.
    w.accum64 = accum64_.as<double>();
    w.aov0 = aov0_.as<float4>();
    w.aov1 = aov1_.as<float4>();
    w.aov_accum = aov_accum_.as<float>();
    w.jobs = jobs_.as<PtJob>();
    w.bvhs = bvhs_.as<JobBvh>();
    w.tiles = tiles_.as<PtTile>();
    w.wave_tiles = wave_tiles_.as<uint32_t>();
    w.wave_paths = wave_paths_.as<uint32_t>();
    w.cap = (uint32_t)cap;

    RT_CUDA_TRY(cudaMemcpyAsync(jobs_.ptr, hj.data(), hj.size() * sizeof(PtJob), cudaMemcpyHostToDevice, st));
    RT_CUDA_TRY(cudaMemcpyAsync(bvhs_.ptr, hb.data(), hb.size() * sizeof(JobBvh), cudaMemcpyHostToDevice, st));
    RT_CUDA_TRY(cudaMemcpyAsync(tiles_.ptr, tiles.data(), tiles.size() * sizeof(PtTile), cudaMemcpyHostToDevice, st));
    RT_CUDA_TRY(cudaMemcpyAsync(wave_tiles_.ptr, wave_tiles.data(), wave_tiles.size() * 4, cudaMemcpyHostToDevice, st));
    RT_CUDA_TRY(cudaMemcpyAsync(wave_paths_.ptr, wave_paths.data(), wave_paths.size() * 4, cudaMemcpyHostToDevice, st));
    RT_CUDA_TRY(cudaMemsetAsync(counters_.ptr, 0, 128, st));
    if (any_aov) RT_CUDA_TRY(cudaMemsetAsync(aov_accum_.ptr, 0, accum_pixels * 4 * PT_AOV_ACCUM, st));
    // Images: accumulate into what the caller passed (PathTracer.cpp:288).
    std::vector<float *> dimg(jobs.size());
    uint64_t off = 0;
    for (size_t j = 0; j < jobs.size(); ++j) {
        const uint64_t n = (uint64_t)hj[j].npix * hj[j].comps;
        if (device_images) {
            dimg[j] = jobs[j].image;
        } else {
            dimg[j] = staging_.as<float>() + off;
            if (jobs[j].image)
                RT_CUDA_TRY(cudaMemcpyAsync(dimg[j], jobs[j].image, n * 4, cudaMemcpyHostToDevice, st));
            else
                RT_CUDA_TRY(cudaMemsetAsync(dimg[j], 0, n * 4, st));
            off += n;
        }
        r = pt_launch_load(dimg[j], hj[j].comps, hj[j].npix, w.accum + 3 * (size_t)hj[j].accum_offset,
                           hj[j].fp64 ? w.accum64 + 3 * (size_t)hj[j].accum_offset : nullptr, st);
        if (r != RT_OK) return r;
    }
    // ---- the graph ------------------------------------------------------------------------------
    Key key;
    std::memset(&key, 0, sizeof(key));
    key.generation = generation_;
    key.cap = cap;
    key.depth = depth;
    key.ext = ext;
    key.shadow_a = shadow_a;
    key.shadow_b = shadow_b;
    key.big_stack = big_stack;
    if (!exec_ || std::memcmp(&key, &key_, sizeof(Key)) != 0) {
        r = trace_closest_batch_prepare(big_stack);
        if (r != RT_OK) return r;
        std::memset(&key_, 0, sizeof(Key));
        r = capture(w, depth, ext, shadow_a, shadow_b, big_stack);
        if (r != RT_OK) return r;
        key_ = key;
    }
    cudaEvent_t e0, e1;
    RT_CUDA_TRY(cudaEventCreate(&e0));
    RT_CUDA_TRY(cudaEventCreate(&e1));
    RT_CUDA_TRY(cudaEventRecord(e0, st));
    float kernel_ms[PT_KERNEL_KINDS] = {0, 0, 0, 0};
    if (!profile) {
        // One launch: the graph loops over the waves on the device.
        if (nwaves > 0) r = pt_launch_set_waves(w, (uint32_t)nwaves, st);
        if (r == RT_OK && nwaves > 0 && cudaGraphLaunch(exec_, st) != cudaSuccess) {
            set_error(std::string("graph launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            r = RT_ERR_CUDA;
        }
    } else {
        // Per-kernel times: the same sequence launched directly on `st`, an event after every
        // step, read back wave by wave.
        for (uint64_t k = 0; k < nwaves && r == RT_OK; ++k) {
            std::vector<cudaEvent_t> marks;
            std::vector<int> kinds;
            r = launch_wave(w, depth, ext, shadow_a, shadow_b, big_stack, st, &marks, &kinds);
            if (r == RT_OK && !marks.empty() && cudaEventSynchronize(marks.back()) != cudaSuccess) r = RT_ERR_CUDA;
            for (size_t q = 1; r == RT_OK && q < marks.size(); ++q) {
                float ms = 0.0f;
                if (cudaEventElapsedTime(&ms, marks[q - 1], marks[q]) == cudaSuccess) kernel_ms[kinds[q]] += ms;
            }
            for (cudaEvent_t e : marks) cudaEventDestroy(e);
        }
    }
    if (r == RT_OK && cudaEventRecord(e1, st) != cudaSuccess) r = RT_ERR_CUDA;
    std::vector<float *> daov(jobs.size(), nullptr);
    for (size_t j = 0; j < jobs.size() && r == RT_OK; ++j) {
        const size_t off3 = 3 * (size_t)hj[j].accum_offset, off_a = PT_AOV_ACCUM * (size_t)hj[j].accum_offset;
        if (jobs[j].aov)
            daov[j] = device_images ? jobs[j].aov : aov_staging_.as<float>() + PT_AOV * (size_t)hj[j].accum_offset;
        r = pt_launch_store(w.accum + off3, hj[j].fp64 ? w.accum64 + off3 : nullptr, hj[j].npix, (float)hj[j].spp,
                            hj[j].comps, std::max<uint32_t>(jobs[j].ranks, 1u), jobs[j].rank, dimg[j],
                            jobs[j].aov ? w.aov_accum + off_a : nullptr, daov[j], st);
    }
    unsigned long long hs[3] = {0, 0, 0};
    unsigned hstatus = 0;
    if (r == RT_OK && (cudaMemcpyAsync(hs, w.stats, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                       cudaMemcpyAsync(&hstatus, w.status, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess))
        r = RT_ERR_CUDA;
    if (r == RT_OK && !device_images)
        for (size_t j = 0; j < jobs.size() && r == RT_OK; ++j)
            if (jobs[j].aov && cudaMemcpyAsync(jobs[j].aov, daov[j], (size_t)hj[j].npix * 4 * PT_AOV, cudaMemcpyDeviceToHost,
                                               st) != cudaSuccess)
                r = RT_ERR_CUDA;
    if (r == RT_OK && !device_images)
        for (size_t j = 0; j < jobs.size() && r == RT_OK; ++j)
            if (jobs[j].image &&
                cudaMemcpyAsync(jobs[j].image, dimg[j], (size_t)hj[j].npix * hj[j].comps * 4, cudaMemcpyDeviceToHost,
                                st) != cudaSuccess)
                r = RT_ERR_CUDA;
    if (r == RT_OK && cudaStreamSynchronize(st) != cudaSuccess) {
        set_error(std::string("render failed: ") + cudaGetErrorString(cudaGetLastError()));
        r = RT_ERR_CUDA;
    }
    if (r == RT_OK && stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->primary_rays = hs[0];
        stats->bounce_rays = hs[1];
        stats->shadow_rays = hs[2];
        stats->paths = 0;
        for (size_t j = 0; j < hj.size(); ++j)
            for (const auto &rg : ranges[j]) stats->paths += (uint64_t)rg.second * hj[j].spp;
        stats->device_ms = ms;
        for (int k = 0; k < PT_KERNEL_KINDS; ++k) stats->kernel_ms[k] = kernel_ms[k];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r == RT_OK && hstatus) {
        set_error(hstatus & RT_DEV_TIMEOUT ? "a bounded device loop gave up" : "a traversal stack overflowed");
        r = (hstatus & RT_DEV_TIMEOUT) ? RT_ERR_TIMEOUT : RT_ERR_OVERFLOW;
    }
    return r;
}

}  // namespace rgb
