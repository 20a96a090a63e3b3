// Wavefront kernels of the path tracer: replace the per-sample loop body of
// PathTracer::render (PathTracer.cpp:186-293 of kosua20/Rendu), for one render or for a
// batch of renders of different scenes, resolutions, sample counts and depths.
//
// A wave is a list of tiles (job, pixel range, run of S consecutive samples) packed from
// all jobs of the call; every path carries its job, pixel and sample. Per wave:
//   raygen     -- primary rays from each job's camera (PathTracer.cpp:186-198); also
//                 starts the wave's queue counters;
//   per bounce:
//     trace    -- closest hit of the compacted ray queue: the persistent traversal with
//                 per-lane refill (rt_trace.cu), each ray against its own job's hierarchy;
//                 also empties the queues the shading appends to;
//     shade    -- the reference's hit logic (background on miss, alpha cut-out, emission,
//                 local frame, NEE light pick + evaluation, BSDF sampling); continuing
//                 paths and shadow rays are appended to queues with one atomic per warp;
//     shadow   -- PathTracer::checkVisibility for each queued shadow ray (two queues,
//                 resolved in a fixed order);
//   accumulate -- min(L, clamp) of each sample added to its pixel in sample order;
//   wave_end   -- advance the wave index (and, inside the graph, set its loop condition).
// The whole per-wave sequence reads its wave from device memory, so it is captured once as
// the body of a CUDA graph's while node that runs it for every wave (pt_engine.cu).
#include <cuda_fp16.h>

#include <algorithm>

#include "pt_scene.hpp"
#include "rt_traverse.cuh"

namespace rgb {
namespace {

__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool pred) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, pred);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(act) - 1;
    uint32_t base = 0;
    if (lane == leader && m) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(act, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

// Tile of the current wave containing wave path p (tiles sorted by path0).
__device__ __forceinline__ uint32_t find_tile(const PtWave &w, uint32_t t0, uint32_t t1, uint32_t p) {
    uint32_t lo = t0, hi = t1 - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (w.tiles[mid].path0 <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_wave_end(PtWave w, cudaGraphConditionalHandle loop, int has_loop) {
    const uint32_t next = w.counters[4] + 1u;
    w.counters[4] = next;
    if (has_loop) cudaGraphSetConditional(loop, next < w.counters[5] ? 1u : 0u);
}

__global__ void k_set_waves(PtWave w, uint32_t n) { w.counters[5] = n; }

__device__ __forceinline__ void raygen_one(const PtWave &w, uint32_t p, uint32_t wave) {
    const PtTile tile = w.tiles[find_tile(w, w.wave_tiles[wave], w.wave_tiles[wave + 1], p)];
    const uint32_t local = p - tile.path0;
    const uint32_t pixel = tile.pixel0 + local % tile.npix;
    const uint32_t sid = tile.s0 + local / tile.npix;
    const PtJob &J = w.jobs[tile.job];
    const uint32_t x = pixel % J.W, y = pixel / J.W;
    const U4 r = philox(U4{pixel, sid, 0u, 0u}, J.seed_lo, J.seed_hi);
    const float jx = u01(r.x), jy = u01(r.y);
    // PathTracer::getSamplePosition (PathTracer.cpp:71-84) and the ray set-up (:191-198).
    const int sidy = (int)sid / (int)J.cx, sidx = (int)sid % (int)J.cx;
    const float sx = (float)x + ((float)sidx + jx) * J.cell_x;
    const float sy = (float)y + ((float)sidy + jy) * J.cell_y;
    const float nx = sx / (float)J.W, ny = sy / (float)J.H;
    const f3 world = mk(J.corner[0] + nx * J.dx[0] + ny * J.dy[0], J.corner[1] + nx * J.dx[1] + ny * J.dy[1],
                        J.corner[2] + nx * J.dx[2] + ny * J.dy[2]);
    const f3 dir = xnormalize(xsub(world, mk(J.eye[0], J.eye[1], J.eye[2])));
    w.qray[0][p] = rt_ray{J.eye[0], J.eye[1], J.eye[2], 1e-4f, dir.x, dir.y, dir.z, 1e8f};
    w.qpath[0][p] = p;
    w.pjob[p] = tile.job;
    w.ppix[p] = pixel;
    w.psamp[p] = sid;
    w.atten[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    w.color[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w.ndc[p] = make_float2(nx, ny);
    if (J.aov) {
        w.aov0[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.aov1[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// The wave's primary rays, grid-stride over its paths (the grid is fixed in the captured
// graph; the wave's size is read on the device). Block 0 also starts the wave's queues: the
// first ray queue holds every path, the traversal's fetch counter restarts.
__global__ void k_raygen(PtWave w) {
    const uint32_t wave = w.counters[4];
    const uint32_t n = w.wave_paths[wave];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counters[0] = n;
        *w.fetch = 0ull;
    }
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) raygen_one(w, p, wave);
}

struct SurfaceHit {
    int obj;
    uint32_t i0, i1, i2;  // global vertex indices into the attribute pools
    float u, v, w;
};

__device__ __forceinline__ SurfaceHit surface(const PtScene &s, uint32_t prim, float u, float v) {
    SurfaceHit h;
    h.obj = find_object(s, prim);
    const PtObject &o = s.objects[h.obj];
    const PtMesh m = s.meshes[o.mesh];
    const uint32_t local = prim - o.first_tri;
    const uint32_t *ix = s.indices + m.first_index + 3 * local;
    h.i0 = m.first_vertex + ix[0];
    h.i1 = m.first_vertex + ix[1];
    h.i2 = m.first_vertex + ix[2];
    h.u = u;
    h.v = v;
    h.w = 1.0f - u - v;  // Raycaster::Hit (Raycaster.cpp:10-12)
    return h;
}

// Raycaster::interpolateAttribute (Raycaster.hpp:90-97).
__device__ __forceinline__ f3 interp3(const float *a, const SurfaceHit &h) {
    const f3 a0 = ld3(a, h.i0), a1 = ld3(a, h.i1), a2 = ld3(a, h.i2);
    return mk(h.w * a0.x + h.u * a1.x + h.v * a2.x, h.w * a0.y + h.u * a1.y + h.v * a2.y,
              h.w * a0.z + h.u * a1.z + h.v * a2.z);
}

__device__ __forceinline__ float2 interp_uv(const float *a, const SurfaceHit &h) {
    return make_float2(h.w * a[2 * h.i0] + h.u * a[2 * h.i1] + h.v * a[2 * h.i2],
                       h.w * a[2 * h.i0 + 1] + h.u * a[2 * h.i1 + 1] + h.v * a[2 * h.i2 + 1]);
}

__device__ __forceinline__ void push_shadow(const PtWave &w, uint32_t slot, f3 o, f3 d, float tmax, f3 c, uint32_t path) {
    w.sray[slot] = rt_ray{o.x, o.y, o.z, 0.001f, d.x, d.y, d.z, tmax};
    w.scontrib[slot] = make_float4(c.x, c.y, c.z, __uint_as_float(path));
}

template <bool EXT>
// At least 7 resident blocks per SM (at most 72 registers): shading is gather-latency bound,
// and the occupancy gained outweighs the spilled registers (the 1080p extended render:
// 108 registers -> 6 blocks 3.4 % faster; 6 -> 7 blocks 189.4 -> 185.3 ms; 8 blocks 187.4 ms).
#ifndef PT_SHADE_MINB
#define PT_SHADE_MINB 7
#endif
__global__ void __launch_bounds__(128, PT_SHADE_MINB) k_shade(PtWave w, int cur, uint32_t did) {
    const uint32_t n = min(w.counters[cur], w.cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&w.stats[did == 0 ? 0 : 1], (unsigned long long)n);  // rays traced this bounce
        *w.fetch = 0ull;  // ray-fetch counter of the next bounce's traversal
    }
    // grid-stride over the queue, whose length is known only on the device
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        constexpr bool ext = EXT;
        const int nxt = cur ^ 1;
        const uint32_t path = w.qpath[cur][i];
        const PtJob &J = w.jobs[w.pjob[path]];
        const PtScene &s = J.scene;
        const rt_ray ray = w.qray[cur][i];
        const rt_hit hit = w.hits[i];
        const f3 pos = mk(ray.ox, ray.oy, ray.oz);
        const f3 dir = mk(ray.dx, ray.dy, ray.dz);
        float4 c4 = w.color[path], a4 = w.atten[path];
        f3 color = mk(c4.x, c4.y, c4.z), atten = mk(a4.x, a4.y, a4.z);
        float prev_pdf = a4.w;  // solid-angle pdf of the BSDF sample that produced this ray (0: none)
        bool cont = false;
        bool sh_a = false, sh_b = false;  // analytic-light and emitter/environment shadow rays
        f3 next_o = pos, next_d = dir;
        f3 sa_o = pos, sa_d = dir, sa_c = mk(0, 0, 0), sb_o = pos, sb_d = dir, sb_c = mk(0, 0, 0);
        float sa_max = 0.0f, sb_max = 0.0f;

        if (hit.prim == RT_NO_HIT) {
            if (ext && s.env_tex >= 0) {
                const f3 le = env_radiance(s, dir);
                float wgt = 1.0f;
                if (did > 0 && prev_pdf > 0.0f) wgt = mis_power(prev_pdf, s.p_env * env_pdf(s, dir));
                color += atten * (le * wgt);
            } else {
                // PathTracer.cpp:206-209.
                const float2 ndc = w.ndc[path];
                color += atten * eval_background(s, pos, dir, ndc.x, ndc.y, did == 0);
            }
        } else {
            const SurfaceHit sh = surface(s, hit.prim, hit.u, hit.v);
            const PtObject &obj = s.objects[sh.obj];
            const PtMaterial mat = s.materials[obj.material];
            const f3 p = mk(pos.x + hit.t * dir.x, pos.y + hit.t * dir.y, pos.z + hit.t * dir.z);
            const float2 uv = obj.use_uv ? interp_uv(s.uvs, sh) : make_float2(0.5f, 0.5f);
            const float4 bcol = tex_rgbal(s, mat.tex[0], uv.x, uv.y);
            if (mat.masked && bcol.w < 0.01f) {
                // Alpha cut-out: same direction from the hit point, one bounce consumed (:223-226).
                cont = did + 1 < J.depth;
                next_o = p;
            } else if (mat.type == PT_MAT_EMISSIVE) {
                f3 le = mk(bcol.x, bcol.y, bcol.z);  // :228-234
                if (did == 0 && J.aov) {  // feature buffer: emitted colour scaled into [0, 1]
                    const float m = fmaxf(fmaxf(fmaxf(le.x, le.y), le.z), 1.0f);
                    w.aov0[path] = make_float4(le.x / m, le.y / m, le.z / m, hit.t);
                }
                if (ext && did > 0 && prev_pdf > 0.0f && s.nemitters > 0) {
                    // Solid-angle pdf with which emitter sampling would have produced this point:
                    // (area * lum / power) * (1 / area) * t^2 / |cos| = lum * t^2 / (power * |cos|).
                    const f3 p0 = ld3(s.positions, sh.i0), p1 = ld3(s.positions, sh.i1), p2 = ld3(s.positions, sh.i2);
                    const f3 ng = normalize(mat3_mul(obj.invtp, cross(p1 - p0, p2 - p0)));
                    const float cosl = fabsf(dot(ng, dir));
                    const float pl = cosl > 0.0f ? (1.0f - s.p_env) * luminance(le) * hit.t * hit.t / (s.emit_power * cosl)
                                                 : 0.0f;
                    le = le * mis_power(prev_pdf, pl);
                }
                color += atten * le;
            } else {
                // PathTracer::buildLocalFrame (:86-122).
                const f3 nn = normalize(interp3(s.normals, sh));
                const f3 tt = normalize(interp3(s.tangents, sh));
                const f3 bb = normalize(interp3(s.bitangents, sh));
                f3 t0 = mat3_mul(obj.invtp, tt), t1 = mat3_mul(obj.invtp, bb), t2 = mat3_mul(obj.invtp, nn);
                if (!(dot(t2, dir) < 0.0f)) t2 = -t2;
                if (obj.use_uv) {
                    const float4 img = tex_rgbal(s, mat.tex[1], uv.x, uv.y);
                    const f3 ln = normalize(mk(2.0f * img.x - 1.0f, 2.0f * img.y - 1.0f, 2.0f * img.z - 1.0f));
                    t2 = mk(t0.x * ln.x + t1.x * ln.y + t2.x * ln.z, t0.y * ln.x + t1.y * ln.y + t2.y * ln.z,
                            t0.z * ln.x + t1.z * ln.y + t2.z * ln.z);
                }
                t2 = normalize(t2);
                t1 = normalize(cross(t2, normalize(t0)));
                t0 = normalize(cross(t1, t2));
                // World -> local is the transpose of the frame.
                const f3 mdir = -dir;
                const f3 wo = normalize(mk(dot(t0, mdir), dot(t1, mdir), dot(t2, mdir)));
                const f3 base = mk(powf(bcol.x, 2.2f), powf(bcol.y, 2.2f), powf(bcol.z, 2.2f));
                const float4 rmao = tex_rgbal(s, mat.tex[2], uv.x, uv.y);
                if (did == 0 && J.aov) {  // feature buffers: linear base colour, shading normal, distance
                    w.aov0[path] = make_float4(base.x, base.y, base.z, hit.t);
                    w.aov1[path] = make_float4(t2.x, t2.y, t2.z, 0.0f);
                }
                const uint32_t pix = w.ppix[path], sid = w.psamp[path];
                const U4 rnd = philox(U4{pix, sid, did + 1u, 0u}, J.seed_lo, J.seed_hi);
                const f3 ps = mk(p.x + 0.001f * t2.x, p.y + 0.001f * t2.y, p.z + 0.001f * t2.z);
                if (s.nlights > 0) {
                    // Next-event estimation on one uniformly picked analytic light (:248-272).
                    const PtLight &L = s.lights[uint_below(rnd.x, (uint32_t)s.nlights)];
                    float maxd, fall;
                    const f3 ld = light_sample(L, ps, maxd, fall);
                    if (fall > 0.0f) {
                        const f3 lwi = normalize(mk(dot(t0, ld), dot(t1, ld), dot(t2, ld)));
                        const f3 ev = ggx_eval(wo, base, rmao.x, rmao.y, lwi);
                        const float inv_pdf = (float)s.nlights;  // 1 / (1 / lights)
                        const f3 ill = mk(fall * ev.x * L.color[0] * inv_pdf, fall * ev.y * L.color[1] * inv_pdf,
                                          fall * ev.z * L.color[2] * inv_pdf);
                        const f3 contrib = atten * ill;
                        if (L.shadows) {
                            sh_a = true;
                            sa_o = ps;
                            sa_d = ld;
                            sa_max = maxd;
                            sa_c = contrib;
                        } else {
                            color += contrib;
                        }
                    }
                }
                if (ext && (s.nemitters > 0 || s.env_tex >= 0)) {
                    // Extended: one emitter-or-environment sample, MIS against BSDF sampling.
                    const U4 r2 = philox(U4{pix, sid, did + 1u, 1u}, J.seed_lo, J.seed_hi);
                    const float usel = u01(r2.x);
                    f3 ld, le;
                    float pl = 0.0f, dist = 1e8f;
                    bool ok = false;
                    if (s.env_tex >= 0 && (s.nemitters == 0 || usel < s.p_env)) {
                        ld = env_sample(s, u01(r2.y), u01(r2.z), pl);
                        pl *= s.p_env;
                        le = env_radiance(s, ld);
                        ok = pl > 0.0f;
                    } else if (s.nemitters > 0) {
                        const float ue = s.env_tex >= 0 ? (usel - s.p_env) / (1.0f - s.p_env) : usel;
                        const PtEmitter em = s.emitters[emitter_pick(s, fminf(fmaxf(ue, 0.0f), 0.99999994f))];
                        const float su = sqrtf(u01(r2.y)), b1 = 1.0f - su, b2 = u01(r2.z) * su;
                        const f3 e1 = mk(em.e1[0], em.e1[1], em.e1[2]), e2 = mk(em.e2[0], em.e2[1], em.e2[2]);
                        const f3 q = mk(em.v0[0] + b1 * e1.x + b2 * e2.x, em.v0[1] + b1 * e1.y + b2 * e2.y,
                                        em.v0[2] + b1 * e1.z + b2 * e2.z);
                        const f3 dq = q - ps;
                        const float d2 = dot(dq, dq);
                        dist = sqrtf(d2);
                        ld = dq / dist;
                        const f3 ng = normalize(cross(e1, e2));
                        const float cosl = fabsf(dot(ng, ld));
                        le = mk(em.emission[0], em.emission[1], em.emission[2]);
                        pl = cosl > 0.0f ? (1.0f - s.p_env) * em.lum * d2 / (s.emit_power * cosl) : 0.0f;
                        ok = pl > 0.0f && dist > 0.0f;
                    }
                    if (ok) {
                        const f3 lwi = normalize(mk(dot(t0, ld), dot(t1, ld), dot(t2, ld)));
                        const f3 ev = ggx_eval(wo, base, rmao.x, rmao.y, lwi);
                        const float pb = ggx_pdf(wo, base, rmao.x, rmao.y, lwi);
                        const float wgt = mis_power(pl, pb) / pl;
                        const f3 contrib = atten * (ev * le) * wgt;
                        if (contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f) {
                            sh_b = true;
                            sb_o = ps;
                            sb_d = ld;
                            sb_max = dist < 1e8f ? dist * (1.0f - 1e-3f) : 1e8f;
                            sb_c = contrib;
                        }
                    }
                }
                f3 wi;
                const f3 weight = ggx_sample_eval(wo, base, rmao.x, rmao.y, u01(rnd.y), u01(rnd.z), u01(rnd.w), wi);
                const f3 nd = normalize(mk(t0.x * wi.x + t1.x * wi.y + t2.x * wi.z, t0.y * wi.x + t1.y * wi.y + t2.y * wi.z,
                                           t0.z * wi.x + t1.z * wi.y + t2.z * wi.z));
                atten *= weight;
                if (ext) prev_pdf = (weight.x > 0.0f || weight.y > 0.0f || weight.z > 0.0f)
                                        ? ggx_pdf(wo, base, rmao.x, rmao.y, wi) : 0.0f;
                if (did + 1 < J.depth) {
                    cont = true;
                    next_o = p;
                    next_d = normalize(nd);
                }
            }
        }
        w.color[path] = make_float4(color.x, color.y, color.z, 0.0f);
        w.atten[path] = make_float4(atten.x, atten.y, atten.z, prev_pdf);
        uint32_t slot = warp_append(&w.counters[nxt], cont);
        if (cont && slot >= w.cap) {  // cannot happen (one append per path); never write past the queue
            atomicOr(w.status, RT_DEV_QUEUE_OVERFLOW);
            cont = false;
        }
        if (cont) {
            w.qray[nxt][slot] = rt_ray{next_o.x, next_o.y, next_o.z, 1e-4f, next_d.x, next_d.y, next_d.z, 1e8f};
            w.qpath[nxt][slot] = path;
        }
        // Two shadow queues (analytic lights; emitters/environment), resolved by two launches
        // in that order: a path never has two shadow rays in one queue, so the radiance update
        // in k_shadow is race-free and the summation order is fixed.
        const uint32_t sa = warp_append(&w.counters[2], sh_a);
        if (sh_a && sa < w.shadow_cap) push_shadow(w, sa, sa_o, sa_d, sa_max, sa_c, path);
        else if (sh_a) atomicOr(w.status, RT_DEV_QUEUE_OVERFLOW);
        const uint32_t sb = warp_append(&w.counters[3], sh_b);
        if (sh_b && sb < w.shadow_cap) push_shadow(w, w.shadow_cap + sb, sb_o, sb_d, sb_max, sb_c, path);
        else if (sh_b) atomicOr(w.status, RT_DEV_QUEUE_OVERFLOW);
    }
}

// Shadow ray through alpha-masked surfaces: closest-hit walks from surface to surface, passing
// texels whose alpha is below 0.01 (PathTracer::checkVisibility, PathTracer.cpp:124-157).
// Bounded to 256 steps (reported as RT_DEV_TIMEOUT and treated as occluded).
template <int STACK>
__device__ bool shadow_walk(const PtWave &w, const PtScene &s, const rt_ray &ray) {
    uint32_t a = 0, b = 0;
    f3 lpos = mk(ray.ox, ray.oy, ray.oz);
    const f3 d = mk(ray.dx, ray.dy, ray.dz);
    float maxd = ray.tmax;
    int steps = 0;
    while (maxd > 0.0f) {
        if (++steps > 256) {
            atomicOr(w.status, RT_DEV_TIMEOUT);
            return false;
        }
        if (steps > 1) atomicAdd(&w.stats[2], 1ull);
        const RayState r = make_ray_state(make_float4(lpos.x, lpos.y, lpos.z, 0.001f),
                                          make_float4(d.x, d.y, d.z, maxd));
        if (!r.valid) break;
        const TraceResult h = traverse<false, false, STACK>(s.nodes, s.tris, r, w.status, a, b);
        if (!h.found) break;
        const SurfaceHit sh = surface(s, h.prim, h.u, h.v);
        const PtObject &obj = s.objects[sh.obj];
        const PtMaterial mat = s.materials[obj.material];
        if (!mat.masked || !obj.use_uv) return false;
        const float2 uv = interp_uv(s.uvs, sh);
        if (tex_rgbal(s, mat.tex[0], uv.x, uv.y).w >= 0.01f) return false;
        maxd = maxd - h.t;
        lpos = mk(lpos.x + h.t * d.x, lpos.y + h.t * d.y, lpos.z + h.t * d.z);
    }
    return true;
}

// One thread per shadow ray (grid-stride over the queue, whose length is known only on the
// device); without masked materials the any-hit traversal decides.
template <int STACK>
// At least 8 resident blocks per SM (64 registers) for the same reason (with the shading
// bound, the 1080p extended render measured 5.5 % faster).
__global__ void __launch_bounds__(128, 8) k_shadow(PtWave w, int queue) {
    const uint32_t n = min(w.counters[2 + queue], w.shadow_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&w.stats[2], (unsigned long long)n);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t e = (queue ? w.shadow_cap : 0u) + i;
        const rt_ray ray = w.sray[e];
        const float4 c = w.scontrib[e];
        const uint32_t path = __float_as_uint(c.w);
        const PtScene &s = w.jobs[w.pjob[path]].scene;
        bool visible = true;
        uint32_t a = 0, b = 0;
        if (!s.empty) {
            if (!s.any_masked) {
                const float4 *rp = reinterpret_cast<const float4 *>(&ray);
                const RayState r = make_ray_state(rp[0], rp[1]);
                if (r.valid) visible = !traverse<true, false, STACK>(s.nodes, s.tris, r, w.status, a, b).found;
            } else {
                visible = shadow_walk<STACK>(w, s, ray);
            }
        }
        if (visible) {
            float4 col = w.color[path];
            col.x += c.x;
            col.y += c.y;
            col.z += c.z;
            w.color[path] = col;
        }
    }
}

// Idle lanes of a warp take new rays only once at least PT_REFILL_MIN of them are idle (a warp
// with no active lane always refills): a refill round (queue atomic, ray load, job lookup)
// stalls the warp's active lanes, so it pays to amortise it. Measured on the 2M-triangle
// instanced 1080p render: threshold 1 -> 64.7 ms, 8 -> 55.6, 16 -> 54.1, 20 -> 53.9,
// 24 -> 54.1 ms per 16 spp; back-to-back rounds gained nothing.
#ifndef PT_REFILL_MIN
#define PT_REFILL_MIN 16
#endif
#ifndef PT_REFILL_ROUNDS
#define PT_REFILL_ROUNDS 1
#endif

template <int STACK>
__global__ void __launch_bounds__(128) k_trace_batch(PtWave w, int cur) {
    const size_t n = min(w.counters[cur], w.cap);
    // The queues the following shading appends to start empty: the next ray queue and both
    // shadow queues (nothing reads them until the shading launch, which follows this one).
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counters[cur ^ 1] = 0u;
        w.counters[2] = 0u;
        w.counters[3] = 0u;
    }
    const rt_ray *__restrict__ rays = w.qray[cur];
    const uint32_t *__restrict__ qpath = w.qpath[cur];
    const unsigned lane = threadIdx.x & 31;
    int stack_node[STACK];
    float stack_near[STACK];
    RayState r;
    TravState t;
    JobBvh jb;
    size_t idx = 0;
    bool active = false, exhausted = false;
    uint32_t nv_ = 0, nt_ = 0;
    while (true) {
        for (int round = 0; round < PT_REFILL_ROUNDS && !exhausted; ++round) {
            const unsigned need = __ballot_sync(0xffffffffu, !active);
            if (!need || (__popc(need) < PT_REFILL_MIN && need != 0xffffffffu)) break;
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(w.fetch, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + __popc(need) >= n) exhausted = true;
            if (!active) {
                idx = (size_t)base + __popc(need & ((1u << lane) - 1u));
                if (idx < n) {
                    const float4 *rp = reinterpret_cast<const float4 *>(rays + idx);
                    r = make_ray_state(rp[0], rp[1]);
                    jb = w.bvhs[w.pjob[qpath[idx]]];
                    trav_init(t, r);
                    active = r.valid && !jb.empty;
                    if (!active) w.hits[idx] = rt_hit{FLT_MAX, 0.0f, 0.0f, RT_NO_HIT};
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (active &&
            trav_step<false, false, STACK>(jb.nodes, jb.tris, r, t, stack_node, stack_near, w.status, nv_, nt_)) {
            active = false;
            w.hits[idx] = rt_hit{t.res.found ? t.res.t : FLT_MAX, t.res.u, t.res.v,
                                 t.res.found ? t.res.prim : RT_NO_HIT};
        }
    }
}

// render.rgb(x, y) += min(sampleColor, 5) in sample order (PathTracer.cpp:288); the clamp
// value is an option of the extended estimator. One thread per (tile, pixel).
__device__ __forceinline__ void accumulate_one(const PtWave &w, uint32_t p, uint32_t wave) {
    const PtTile tile = w.tiles[find_tile(w, w.wave_tiles[wave], w.wave_tiles[wave + 1], p)];
    const uint32_t local = p - tile.path0;
    if (local >= tile.npix) return;
    const PtJob &J = w.jobs[tile.job];
    const size_t px = (size_t)J.accum_offset + tile.pixel0 + local;
    const float cl = J.clamp;
    const bool clamp = cl > 0.0f;
    if (J.fp64) {
        double *acc = w.accum64 + 3 * px;
        double r = acc[0], g = acc[1], b = acc[2];
        for (uint32_t s = 0; s < tile.S; ++s) {
            const float4 c = w.color[(size_t)tile.path0 + (size_t)s * tile.npix + local];
            r += (double)(clamp ? gmin(c.x, cl) : c.x);
            g += (double)(clamp ? gmin(c.y, cl) : c.y);
            b += (double)(clamp ? gmin(c.z, cl) : c.z);
        }
        acc[0] = r;
        acc[1] = g;
        acc[2] = b;
    } else {
        float *acc = w.accum + 3 * px;
        float r = acc[0], g = acc[1], b = acc[2];
        for (uint32_t s = 0; s < tile.S; ++s) {
            const float4 c = w.color[(size_t)tile.path0 + (size_t)s * tile.npix + local];
            r += clamp ? gmin(c.x, cl) : c.x;
            g += clamp ? gmin(c.y, cl) : c.y;
            b += clamp ? gmin(c.z, cl) : c.z;
        }
        acc[0] = r;
        acc[1] = g;
        acc[2] = b;
    }
    if (J.aov) {
        // First-hit features, and the sum and sum of squares of the samples' luminance
        // (as accumulated: clamped) for the standard error of the pixel's mean.
        float *a = w.aov_accum + PT_AOV_ACCUM * px;
        float f[PT_AOV_ACCUM];
#pragma unroll
        for (int k = 0; k < PT_AOV_ACCUM; ++k) f[k] = a[k];
        for (uint32_t s = 0; s < tile.S; ++s) {
            const size_t q = (size_t)tile.path0 + (size_t)s * tile.npix + local;
            const float4 a0 = w.aov0[q], a1 = w.aov1[q], c = w.color[q];
            f[0] += a0.x; f[1] += a0.y; f[2] += a0.z;
            f[3] += a1.x; f[4] += a1.y; f[5] += a1.z;
            f[6] += a0.w;
            const float lum = 0.2126f * (clamp ? gmin(c.x, cl) : c.x) + 0.7152f * (clamp ? gmin(c.y, cl) : c.y) +
                              0.0722f * (clamp ? gmin(c.z, cl) : c.z);
            f[7] += lum;
            f[8] += lum * lum;
        }
#pragma unroll
        for (int k = 0; k < PT_AOV_ACCUM; ++k) a[k] = f[k];
    }
}

__global__ void k_accumulate(PtWave w) {
    const uint32_t wave = w.counters[4];
    const uint32_t n = w.wave_paths[wave];
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        accumulate_one(w, p, wave);
}

__global__ void k_load(const float *__restrict__ img, uint32_t comps, uint32_t npix, float *__restrict__ accum,
                       double *__restrict__ accum64) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npix) return;
    for (int k = 0; k < 3; ++k) {
        const float v = img[(size_t)px * comps + k];
        if (accum64) accum64[3 * (size_t)px + k] = (double)v;
        else accum[3 * (size_t)px + k] = v;
    }
}

// render.rgb(x, y) /= samples (PathTracer.cpp:291-292); feature buffers averaged likewise.
__global__ void k_store(const float *__restrict__ accum, const double *__restrict__ accum64, uint32_t npix,
                        float spp, uint32_t comps, uint32_t ranks, uint32_t rank, float *__restrict__ img,
                        const float *__restrict__ aov_accum, float *__restrict__ aov) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= npix) return;
    if (ranks > 1 && (px / PT_RANK_TILE_PIXELS) % ranks != rank) {
        // Another rank's pixel: zero, so that the sum over ranks assembles the image.
        for (uint32_t k = 0; k < comps; ++k) img[(size_t)px * comps + k] = 0.0f;
        if (aov)
            for (int k = 0; k < PT_AOV; ++k) aov[PT_AOV * (size_t)px + k] = 0.0f;
        return;
    }
    for (int k = 0; k < 3; ++k)
        img[(size_t)px * comps + k] =
            accum64 ? (float)(accum64[3 * (size_t)px + k] / (double)spp) : accum[3 * (size_t)px + k] / spp;
    if (aov) {
        const float *a = aov_accum + PT_AOV_ACCUM * (size_t)px;
        float *o = aov + PT_AOV * (size_t)px;
        for (int k = 0; k < 7; ++k) o[k] = a[k] / spp;
        // Standard error of the mean luminance: sqrt((E[L^2] - E[L]^2) / spp).
        const float m = a[7] / spp, m2 = a[8] / spp;
        o[7] = sqrtf(fmaxf(m2 - m * m, 0.0f) / spp);
    }
}

__global__ void k_mat_eval(const float *__restrict__ c, uint32_t n, float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *q = c + 11 * (size_t)i;
    const f3 r = ggx_eval(mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), q[6], q[7], mk(q[8], q[9], q[10]));
    out[3 * (size_t)i] = r.x;
    out[3 * (size_t)i + 1] = r.y;
    out[3 * (size_t)i + 2] = r.z;
}

__global__ void k_mat_sample(const float *__restrict__ c, const float *__restrict__ u, uint32_t n,
                             float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *q = c + 8 * (size_t)i;
    const float *uu = u + 3 * (size_t)i;
    f3 wi = mk(0.0f, 0.0f, 0.0f);
    const f3 r = ggx_sample_eval(mk(q[0], q[1], q[2]), mk(q[3], q[4], q[5]), q[6], q[7], uu[0], uu[1], uu[2], wi);
    float *o = out + 6 * (size_t)i;
    o[0] = r.x; o[1] = r.y; o[2] = r.z;
    o[3] = wi.x; o[4] = wi.y; o[5] = wi.z;
}

}  // namespace

// AtmosphereApp::precomputeTable (AtmosphereApp.cpp:145-188): the sky's secondary
// attenuation towards the sun, x = relative height, y = cosine of the sun's vertical angle;
// optionally rounded to half precision like the reference's stored table.
__global__ void k_sky_table(uint32_t res, uint32_t samples, int half_prec, float4 *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= res * res) return;
    const uint32_t x = i % res, y = i / res;
    const float xf = (float)x / ((float)res - 1.0f), yf = (float)y / ((float)res - 1.0f);
    const f3 pos = mk(0.0f, (sky::kTop - sky::kGround) * xf + sky::kGround, 0.0f);
    const float cosA = 2.0f * yf - 1.0f;
    const float sinA = sqrtf(1.0f - cosA * cosA);
    const f3 sun = -xnormalize(mk(sinA, cosA, 0.0f));
    float r0 = 0.0f, r1 = 0.0f;
    const bool hit = sphere_roots(pos, sun, sky::kTop, r0, r1);
    const float step = hit ? r1 / (float)samples : 0.0f;
    float rd = 0.0f, md = 0.0f;
    for (uint32_t j = 0; j < samples; ++j) {
        const f3 p = pos + (((float)j + 0.5f) * step) * sun;
        const float hgt = sqrtf(dot(p, p)) - sky::kGround;
        rd += expf(-hgt / sky::kHRayleigh) * step;
        md += expf(-hgt / sky::kHMie) * step;
    }
    const f3 kr = sky::rayleigh_k();
    float a[3] = {expf(-(sky::kMie * md + kr.x * rd)), expf(-(sky::kMie * md + kr.y * rd)),
                  expf(-(sky::kMie * md + kr.z * rd))};
    if (half_prec)
        for (int c = 0; c < 3; ++c) a[c] = __half2float(__float2half_rn(a[c]));
    out[i] = make_float4(a[0], a[1], a[2], 1.0f);
}

// MaterialSky::eval for n cases {origin.xyz, direction.xyz, sun.xyz}.
__global__ void k_sky_eval(const float4 *__restrict__ table, uint32_t w, uint32_t h, const float *__restrict__ cases,
                           uint32_t n, float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *c = cases + 9 * (size_t)i;
    const f3 r = sky_eval(table, w, h, mk(c[0], c[1], c[2]), mk(c[3], c[4], c[5]), mk(c[6], c[7], c[8]));
    out[3 * (size_t)i] = r.x;
    out[3 * (size_t)i + 1] = r.y;
    out[3 * (size_t)i + 2] = r.z;
}

int pt_launch_sky_table(uint32_t res, uint32_t samples, bool half_prec, float4 *out, cudaStream_t st) {
    const uint32_t n = res * res;
    k_sky_table<<<(n + 255) / 256, 256, 0, st>>>(res, samples, half_prec ? 1 : 0, out);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_sky_eval(const float4 *table, uint32_t w, uint32_t h, const float *cases, uint32_t n, float *out,
                       cudaStream_t st) {
    if (n == 0) return RT_OK;
    k_sky_eval<<<(n + 127) / 128, 128, 0, st>>>(table, w, h, cases, n, out);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_material(const float *cases, const float *uniforms, uint32_t n, float *out, cudaStream_t st) {
    if (n == 0) return RT_OK;
    if (uniforms) k_mat_sample<<<(n + 127) / 128, 128, 0, st>>>(cases, uniforms, n, out);
    else k_mat_eval<<<(n + 127) / 128, 128, 0, st>>>(cases, n, out);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_wave_end(const PtWave &w, cudaStream_t st, const cudaGraphConditionalHandle *loop) {
    k_wave_end<<<1, 1, 0, st>>>(w, loop ? *loop : cudaGraphConditionalHandle(0), loop ? 1 : 0);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_set_waves(const PtWave &w, uint32_t nwaves, cudaStream_t st) {
    k_set_waves<<<1, 1, 0, st>>>(w, nwaves);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

// Grid of the wave-wide element-wise kernels (grid-stride loops): at most 16 blocks of 256
// per SM, fewer for a small capacity.
static unsigned wave_grid(const PtWave &w) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            sms = 152;
    }
    return (unsigned)std::min<uint64_t>((w.cap + 255) / 256, (uint64_t)sms * 16);
}

int pt_launch_raygen(const PtWave &w, cudaStream_t st) {
    k_raygen<<<wave_grid(w), 256, 0, st>>>(w);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

// Shading launches: SHADE_WAVES full residencies of the GPU, grid-stride over the ray queue
// (its length is known only on the device); 0 = one block per 128 slots of capacity.
// Against 0: Cornell 256^2 0.63 -> 0.51 ms (its later bounces hold few paths), the large
// 1080p render within 1 % (4 residencies: 2.5 % slower there; 64: no gain on Cornell).
#ifndef SHADE_WAVES
#define SHADE_WAVES 16
#endif
static int g_shade_grid[2] = {0, 0};

int pt_launch_shade(const PtWave &w, int cur, uint32_t did, bool ext, cudaStream_t st) {
    const int g = SHADE_WAVES ? g_shade_grid[ext ? 1 : 0] : (int)((w.cap + 127) / 128);
    if (g == 0) {
        set_error("shading grid not prepared");
        return RT_ERR_STATE;
    }
    if (ext) k_shade<true><<<g, 128, 0, st>>>(w, cur, did);
    else k_shade<false><<<g, 128, 0, st>>>(w, cur, did);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

// Shadow launches: SHADOW_WAVES full residencies of the GPU, grid-stride over the queue (its
// length is known only on the device); 0 = one block per 128 slots of capacity. Measured
// with shading at 16: Cornell 256^2 0.62 ms at 0, 0.51 ms at 16; the large 1080p render
// 224.8-226.5 ms for 0, 4, 16 and 64 alike.
#ifndef SHADOW_WAVES
#define SHADOW_WAVES 16
#endif
static int g_shadow_grid[2] = {0, 0};

int pt_launch_shadow(const PtWave &w, int queue, bool big_stack, cudaStream_t st) {
    const int g = SHADOW_WAVES ? g_shadow_grid[big_stack ? 1 : 0] : (int)((w.cap + 127) / 128);
    if (g == 0) {
        set_error("shadow traversal grid not prepared");
        return RT_ERR_STATE;
    }
    if (big_stack) k_shadow<256><<<g, 128, 0, st>>>(w, queue);
    else k_shadow<64><<<g, 128, 0, st>>>(w, queue);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

static int g_batch_grid[2] = {0, 0};

// Grid of the persistent batch traversal (one full residency of the GPU); computed outside
// any stream capture.
int trace_closest_batch_prepare(bool big_stack) {
    int &g = g_batch_grid[big_stack ? 1 : 0];
    if (g == 0) {
        int per_sm = 0, sms = 0, dev = 0;
        RT_CUDA_TRY(cudaGetDevice(&dev));
        RT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (big_stack) RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_batch<256>, 128, 0));
        else RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_batch<64>, 128, 0));
        g = sms * (per_sm > 0 ? per_sm : 1);
        int &gs = g_shadow_grid[big_stack ? 1 : 0];
        per_sm = 0;
        if (big_stack) RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shadow<256>, 128, 0));
        else RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shadow<64>, 128, 0));
        gs = sms * (per_sm > 0 ? per_sm : 1) * SHADOW_WAVES;
        for (int e = 0; e < 2; ++e) {
            per_sm = 0;
            if (e) RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade<true>, 128, 0));
            else RT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade<false>, 128, 0));
            g_shade_grid[e] = sms * (per_sm > 0 ? per_sm : 1) * SHADE_WAVES;
        }
    }
    return RT_OK;
}

int trace_closest_batch(const PtWave &w, int cur, bool big_stack, cudaStream_t st) {
    const int g = g_batch_grid[big_stack ? 1 : 0];
    if (g == 0) {
        set_error("batch traversal grid not prepared");
        return RT_ERR_STATE;
    }
    if (big_stack) k_trace_batch<256><<<g, 128, 0, st>>>(w, cur);
    else k_trace_batch<64><<<g, 128, 0, st>>>(w, cur);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_accumulate(const PtWave &w, cudaStream_t st) {
    k_accumulate<<<wave_grid(w), 256, 0, st>>>(w);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_load(const float *img, uint32_t comps, uint32_t npix, float *accum, double *accum64, cudaStream_t st) {
    k_load<<<(npix + 255) / 256, 256, 0, st>>>(img, comps, npix, accum, accum64);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

int pt_launch_store(const float *accum, const double *accum64, uint32_t npix, float spp, uint32_t comps, uint32_t ranks,
                    uint32_t rank, float *img, const float *aov_accum, float *aov, cudaStream_t st) {
    k_store<<<(npix + 255) / 256, 256, 0, st>>>(accum, accum64, npix, spp, comps, ranks, rank, img, aov_accum, aov);
    RT_CUDA_TRY(cudaGetLastError());
    return RT_OK;
}

}  // namespace rgb
