// Device-side scene model and shading functions of the path tracer.
//
// Restates, for sm_103a, the per-sample math of kosua20/Rendu's offline path tracer:
//   MaterialGGX::F/D/V/alphaFromRoughness/GGX/sampleAndEval/eval  MaterialGGX.cpp:5-101
//   Random::sampleDisk / sampleCosineHemisphere                   Random.cpp:41-70
//   Image::rgbl / rgbal (bilinear, wrapped)                        Image.cpp:64-106
//   Texture::sampleCubemap                                         Texture.cpp:141-191
//   PointLight/DirectionalLight/SpotLight::sample                  PointLight.cpp:68-87,
//                                                                  DirectionalLight.cpp:40-44,
//                                                                  SpotLight.cpp:52-78
//   PathTracer::buildLocalFrame / evalBackground                   PathTracer.cpp:23-55, 86-122
// The reference draws its random numbers from per-thread std::mt19937 streams; here every
// draw comes from a counter-based generator (Philox-4x32-10, Salmon et al., SC'11) keyed by
// the render seed and indexed by (pixel, sample, bounce), so a render is reproducible and
// independent of the launch shape. The draws are consumed in the reference's order.
#pragma once

#include "rt_common.cuh"

namespace rgb {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kOneOverPi = 0.318309886183790671538f;  // glm::one_over_pi<float>()
constexpr float kTwoPi = 6.28318530717958647692f;       // glm::two_pi<float>()

// ---- Philox-4x32-10 --------------------------------------------------------------------
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Uniform float in [0, 1) from the top 24 bits.
__host__ __device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Uniform integer in [0, n) (multiply-high).
__host__ __device__ __forceinline__ uint32_t uint_below(uint32_t x, uint32_t n) { return mulhi32(x, n); }

// ---- device scene -----------------------------------------------------------------------
struct PtTex {
    uint32_t w, h;
    uint64_t offset;  // into the float4 texel pool
    int constant;     // all texels equal: `value` is returned without filtering
    float4 value;
};

struct PtMesh {
    uint32_t first_vertex;  // into the attribute pools
    uint32_t first_index;   // into the index pool (mesh-local vertex indices)
    uint32_t has_uv;
    uint32_t pad;
};

struct PtObject {
    uint32_t mesh, material, first_tri, use_uv;
    float invtp[9];  // inverse(transpose(mat3(model))), row-major
};

struct PtMaterial {
    int type, masked;
    uint32_t tex[3];
};

struct PtLight {
    int type, shadows;
    float color[3], position[3], direction[3];  // direction normalised as the constructors do
    float radius, half_inner, half_outer;
};

// Emissive triangle in world space (extended estimator).
struct PtEmitter {
    float v0[3], e1[3], e2[3];
    float emission[3];
    float lum;  // luminance of the emission
};

struct PtScene {
    const BvhNode *nodes;
    const BvhTri *tris;
    unsigned *status;
    int big_stack, empty;
    const PtObject *objects;
    int nobjects;
    const PtMesh *meshes;
    const PtMaterial *materials;
    const PtTex *textures;
    const float4 *texels;
    const float *positions, *normals, *tangents, *bitangents, *uvs;  // model space, per mesh vertex
    const uint32_t *indices;
    const PtLight *lights;
    int nlights;
    int any_masked;
    int bg_mode;
    float bg_color[3];
    uint32_t bg_tex[6];
    // Extended estimator: emitter table + power CDF, environment map + 2-D distribution.
    const PtEmitter *emitters;
    const float *emitter_cdf;  // inclusive cumulative, last = 1
    int nemitters;
    float emit_power;          // sum of area x luminance
    int env_tex;               // -1: none
    float env_intensity;
    uint32_t env_w, env_h;
    const float *env_marg;     // env_h + 1 cumulative (first 0, last 1)
    const float *env_cond;     // env_h rows of env_w + 1 cumulative
    const float *env_func;     // env_h x env_w piecewise-constant weights
    float env_integral;        // mean of env_func over the unit square
    float p_env;               // probability of sampling the environment in NEE
    // ATMOSPHERE background: normalised sun direction and the scattering table.
    float sun[3];
    const float4 *sky;
    uint32_t sky_w, sky_h;
};

// ---- textures ----------------------------------------------------------------------------
__device__ __forceinline__ int mod_pos(int x, int w) { return ((x % w) + w) % w; }

__device__ __forceinline__ int f2i_sat(float f) {
    return (int)fminf(fmaxf(f, -2147483520.0f), 2147483520.0f);
}

// Image::rgbal (Image.cpp:86-106): bilinear with wrapping.
__device__ __forceinline__ float4 tex_rgbal(const PtScene &s, uint32_t id, float x, float y) {
    const PtTex t = s.textures[id];
    if (t.constant) return t.value;
    const float xi = x * (float)t.w, yi = y * (float)t.h;
    const float xb = floorf(xi), yb = floorf(yi);
    const float dx = xi - xb, dy = yi - yb;
    const int ixb = f2i_sat(xb), iyb = f2i_sat(yb);
    const int x0 = mod_pos(ixb, (int)t.w), y0 = mod_pos(iyb, (int)t.h);
    const int x1 = mod_pos(ixb + 1, (int)t.w), y1 = mod_pos(iyb + 1, (int)t.h);
    const float4 *px = s.texels + t.offset;
    const float4 p00 = px[(size_t)y0 * t.w + x0], p01 = px[(size_t)y1 * t.w + x0];
    const float4 p10 = px[(size_t)y0 * t.w + x1], p11 = px[(size_t)y1 * t.w + x1];
    const float a = 1.0f - dx, b = 1.0f - dy;
    return make_float4(a * (b * p00.x + dy * p01.x) + dx * (b * p10.x + dy * p11.x),
                       a * (b * p00.y + dy * p01.y) + dx * (b * p10.y + dy * p11.y),
                       a * (b * p00.z + dy * p01.z) + dx * (b * p10.z + dy * p11.z),
                       a * (b * p00.w + dy * p01.w) + dx * (b * p10.w + dy * p11.w));
}

// Texture::sampleCubemap (Texture.cpp:141-191); faces +x,-x,+y,-y,+z,-z.
__device__ __forceinline__ f3 cubemap(const PtScene &s, f3 dir) {
    const float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
    int face = 0;
    float x = 0.0f, y = 0.0f, denom = 1.0f;
    if (ax >= ay && ax >= az) {
        denom = ax;
        y = dir.y;
        face = dir.x >= 0.0f ? 0 : 1;
        x = dir.x >= 0.0f ? -dir.z : dir.z;
    } else if (ay >= ax && ay >= az) {
        denom = ay;
        x = dir.x;
        face = dir.y >= 0.0f ? 2 : 3;
        y = dir.y >= 0.0f ? -dir.z : dir.z;
    } else if (az >= ax && az >= ay) {
        denom = az;
        y = dir.y;
        face = dir.z >= 0.0f ? 4 : 5;
        x = dir.z >= 0.0f ? dir.x : -dir.x;
    }
    x = 0.5f * (x / denom) + 0.5f;
    y = 0.5f * (-y / denom) + 0.5f;
    const PtTex t = s.textures[s.bg_tex[face]];
    const float eps = 1.0f / (float)min(t.w, t.h);
    x = fminf(fmaxf(x, eps), 1.0f - eps);
    y = fminf(fmaxf(y, eps), 1.0f - eps);
    const float4 c = tex_rgbal(s, s.bg_tex[face], x, y);
    return mk(c.x, c.y, c.z);
}

// ---- atmosphere (MaterialSky.cpp:6-98; parameters Sky.hpp:53-65) ----------------------------
// Evaluated in the reference's operation order in a unit compiled without FMA contraction.
namespace sky {
constexpr float kGround = 6371e3f, kTop = 6471e3f, kSunIntensity = 20.0f, kMie = 21e-6f;
constexpr float kHRayleigh = 8000.0f, kHMie = 1200.0f, kGMie = 0.758f, kSunRadius = 0.04675f;
constexpr float kSunRadiusCos = 0.998f, kPi = 3.14159265358979323846f;
constexpr int kSteps = 16;  // MaterialSky::samplesCount
__device__ __forceinline__ f3 rayleigh_k() { return mk(5.5e-6f, 13.0e-6f, 22.4e-6f); }
__device__ __forceinline__ f3 sun_color() { return mk(1.474f, 1.8504f, 1.91198f); }
}  // namespace sky

// Intersection::sphere (Intersection.cpp:7-20).
__device__ __forceinline__ bool sphere_roots(f3 o, f3 d, float radius, float &r0, float &r1) {
    const float a = dot(d, d), b = dot(o, d), c = dot(o, o) - radius * radius;
    const float delta = b * b - a * c;
    if (delta < 0.0f) return false;
    const float ds = sqrtf(delta);
    r0 = (-b - ds) / a;
    r1 = (-b + ds) / a;
    return true;
}

// Image::rgbl (Image.cpp:64-84) on the scattering table.
__device__ __forceinline__ f3 sky_rgbl(const float4 *t, uint32_t w, uint32_t h, float x, float y) {
    const float xi = x * (float)w, yi = y * (float)h;
    const float xb = floorf(xi), yb = floorf(yi);
    const float dx = xi - xb, dy = yi - yb;
    const int x0 = mod_pos(f2i_sat(xb), (int)w), y0 = mod_pos(f2i_sat(yb), (int)h);
    const int x1 = mod_pos(f2i_sat(xb) + 1, (int)w), y1 = mod_pos(f2i_sat(yb) + 1, (int)h);
    const float4 p00 = t[(size_t)y0 * w + x0], p01 = t[(size_t)y1 * w + x0];
    const float4 p10 = t[(size_t)y0 * w + x1], p11 = t[(size_t)y1 * w + x1];
    return mk((1.0f - dx) * ((1.0f - dy) * p00.x + dy * p01.x) + dx * ((1.0f - dy) * p10.x + dy * p11.x),
              (1.0f - dx) * ((1.0f - dy) * p00.y + dy * p01.y) + dx * ((1.0f - dy) * p10.y + dy * p11.y),
              (1.0f - dx) * ((1.0f - dy) * p00.z + dy * p01.z) + dx * ((1.0f - dy) * p10.z + dy * p11.z));
}

__device__ __forceinline__ float rayleigh_phase(float c) {
    const float k = 1.0f / (4.0f * sky::kPi);
    return k * 3.0f / 4.0f * (1.0f + c * c);
}
__device__ __forceinline__ float mie_phase(float c) {
    const float k = 1.0f / (4.0f * sky::kPi);
    const float g2 = sky::kGMie * sky::kGMie;
    return k * 3.0f * (1.0f - g2) / (2.0f * (2.0f + g2)) * (1.0f + c * c) /
           powf(1.0f + g2 - 2.0f * sky::kGMie * c, 3.0f / 2.0f);
}

// MaterialSky::eval: 16-step single-scattering march through the atmosphere along the ray
// (planet centre 6371 km + 1 m below the origin), secondary attenuation from the table,
// plus the sun disc when the ray does not hit the ground.
__device__ __forceinline__ f3 sky_eval(const float4 *table, uint32_t tw, uint32_t th, f3 origin, f3 dir, f3 sun) {
    const f3 planet = (origin + mk(0.0f, sky::kGround, 0.0f)) + mk(0.0f, 1.0f, 0.0f);
    float t0 = 0.0f, t1 = 0.0f, g0 = 0.0f, g1 = 0.0f;
    if (!sphere_roots(planet, dir, sky::kTop, t0, t1)) return mk(0.0f, 0.0f, 0.0f);
    const bool ground = sphere_roots(planet, dir, sky::kGround, g0, g1);
    const float dist = gmin(t1, ground ? g0 : 0.0f);
    const float step = (dist - t0) / (float)sky::kSteps;
    const float cos_vs = dot(dir, sun);
    const f3 kr = sky::rayleigh_k();
    float rd = 0.0f, md = 0.0f;
    f3 rs = mk(0, 0, 0), ms = mk(0, 0, 0), tr = mk(0, 0, 0);
    for (int i = 0; i < sky::kSteps; ++i) {
        const f3 p = planet + (((float)i + 0.5f) * step) * dir;
        float hgt = sqrtf(dot(p, p)) - sky::kGround;
        if (i == sky::kSteps - 1 && hgt < 0.0f) hgt = 0.0f;
        const float rstep = expf(-hgt / sky::kHRayleigh) * step;
        const float mstep = expf(-hgt / sky::kHMie) * step;
        rd += rstep;
        md += mstep;
        const f3 direct = mk(expf(-(md * sky::kMie + rd * kr.x)), expf(-(md * sky::kMie + rd * kr.y)),
                             expf(-(md * sky::kMie + rd * kr.z)));
        const float rel_h = (sqrtf(dot(p, p)) - sky::kGround) / (sky::kTop - sky::kGround);
        const float rel_c = -0.5f * sun.y + 0.5f;
        float u = (511.0f / 512.0f) * rel_h + 0.5f / 512.0f, v = (511.0f / 512.0f) * rel_c + 0.5f / 512.0f;
        u = gmin(gmax(u, 0.5f / 512.0f), 511.0f / 512.0f);  // glm::clamp
        v = gmin(gmax(v, 0.5f / 512.0f), 511.0f / 512.0f);
        const f3 att = direct * sky_rgbl(table, tw, th, u, v);
        rs += rstep * att;
        ms += mstep * att;
        tr += direct;
    }
    const f3 rp = (rayleigh_phase(cos_vs) * kr) * rs;
    const f3 mp = (sky::kMie * mie_phase(cos_vs)) * ms;
    f3 sun_r = mk(0.0f, 0.0f, 0.0f);
    if (!(ground && g1 > 0.0f) && dot(dir, sun) > sky::kSunRadiusCos)
        sun_r = sky::sun_color() / (sky::kPi * sky::kSunRadius * sky::kSunRadius);
    return sky::kSunIntensity * (rp + mp) + tr * sun_r;
}

// PathTracer::evalBackground (PathTracer.cpp:23-55): COLOR and IMAGE only for primary
// misses (IMAGE indexed by the screen position), SKYBOX and ATMOSPHERE (at the ray's
// origin) for every miss.
__device__ __forceinline__ f3 eval_background(const PtScene &s, f3 pos, f3 dir, float ndc_x, float ndc_y,
                                              bool direct) {
    if (s.bg_mode == PT_BG_SKYBOX) return cubemap(s, normalize(dir));
    if (s.bg_mode == PT_BG_ATMOSPHERE)
        return sky_eval(s.sky, s.sky_w, s.sky_h, pos, xnormalize(dir), mk(s.sun[0], s.sun[1], s.sun[2]));
    if (!direct) return mk(0.0f, 0.0f, 0.0f);
    if (s.bg_mode == PT_BG_IMAGE) {
        const float4 c = tex_rgbal(s, s.bg_tex[0], ndc_x, ndc_y);
        return mk(c.x, c.y, c.z);
    }
    return mk(s.bg_color[0], s.bg_color[1], s.bg_color[2]);
}

// ---- MaterialGGX (MaterialGGX.cpp:5-101) --------------------------------------------------
__device__ __forceinline__ f3 ggx_F(f3 F0, float VdotH) {
    const float p = powf(1.0f - VdotH, 5.0f);
    return mk(F0.x + p * (1.0f - F0.x), F0.y + p * (1.0f - F0.y), F0.z + p * (1.0f - F0.z));
}

__device__ __forceinline__ float ggx_D(float NdotH, float alpha) {
    const float halfDenum = NdotH * NdotH * (alpha * alpha - 1.0f) + 1.0f;
    const float halfTerm = alpha / fmaxf(0.0001f, halfDenum);
    return halfTerm * halfTerm * kOneOverPi;
}

__device__ __forceinline__ float ggx_V(float NdotL, float NdotV, float alpha) {
    const float alpha2 = alpha * alpha;
    const float visL = NdotV * sqrtf((-NdotL * alpha2 + NdotL) * NdotL + alpha2);
    const float visV = NdotL * sqrtf((-NdotV * alpha2 + NdotV) * NdotV + alpha2);
    return 0.5f / fmaxf(0.0001f, visV + visL);
}

__device__ __forceinline__ float alpha_from_roughness(float roughness) {
    const float rc = fmaxf(0.045f, roughness);
    return fmaxf(0.0001f, rc * rc);
}

// The reference names wo.z "NdotL" and wi.z "NdotV" (MaterialGGX.cpp:35-36); kept.
__device__ __forceinline__ f3 ggx_brdf(f3 wo, f3 base, float alpha, float metallic, f3 wi, float *pdf) {
    const f3 h = normalize(wi + wo);
    const float NdotH = fmaxf(h.z, 0.0f);
    const float VdotH = fmaxf(dot(wi, h), 0.0f);
    const float NdotL = fmaxf(wo.z, 0.0f);
    const float NdotV = fmaxf(wi.z, 0.0f);
    const float Dh = ggx_D(NdotH, alpha);
    if (pdf) *pdf = Dh * NdotH / (4.0f * fmaxf(0.0001f, VdotH));
    const f3 F0 = mk(0.04f + (base.x - 0.04f) * metallic, 0.04f + (base.y - 0.04f) * metallic,
                     0.04f + (base.z - 0.04f) * metallic);
    const float dv = Dh * ggx_V(NdotL, NdotV, alpha);
    const f3 F = ggx_F(F0, VdotH);
    const float kd = (1.0f - metallic) * kOneOverPi;
    const float ms = 2.0f * alpha * alpha * NdotV;  // multi-scattering adjustment (MaterialGGX.cpp:49)
    f3 r;
    r.x = (kd * base.x * (1.0f - F0.x) + dv * F.x * (1.0f + ms * F0.x)) * NdotV;
    r.y = (kd * base.y * (1.0f - F0.y) + dv * F.y * (1.0f + ms * F0.y)) * NdotV;
    r.z = (kd * base.z * (1.0f - F0.z) + dv * F.z * (1.0f + ms * F0.z)) * NdotV;
    return r;
}

// Random::sampleDisk + sampleCosineHemisphere (Random.cpp:41-70) from two uniforms.
__device__ __forceinline__ f3 cosine_hemisphere(float u0, float u1) {
    const float x = 2.0f * u0 - 1.0f, y = 2.0f * u1 - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(x == 0.0f && y == 0.0f)) {
        float angle, radius;
        if (fabsf(x) > fabsf(y)) {
            radius = x;
            angle = 0.25f * kPi * y / x;
        } else {
            radius = y;
            angle = 0.5f * kPi - 0.25f * kPi * x / y;
        }
        dx = radius * cosf(angle);
        dy = radius * sinf(angle);
    }
    const float z = sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy));
    return mk(dx, dy, z);
}

// MaterialGGX::sampleAndEval (MaterialGGX.cpp:54-92): u0 picks the lobe, u1 and u2 sample it.
__device__ __forceinline__ f3 ggx_sample_eval(f3 wo, f3 base, float roughness, float metallic, float u0, float u1,
                                              float u2, f3 &wi) {
    const float pmean = (base.x + base.y + base.z) / 3.0f;
    const float pdiff = 1.0f / (pmean + 1.0f);
    const float probaSpecular = pdiff + (1.0f - pdiff) * metallic;  // glm::mix(pdiff, 1, metallic)
    const float alpha = alpha_from_roughness(roughness);
    if (u0 < probaSpecular) {
        const float a2 = alpha * alpha;
        const float x = u1;
        const float phiH = u2 * kTwoPi;
        const float cosThetaHSqr = fminf((1.0f - x) / ((a2 - 1.0f) * x + 1.0f), 1.0f);
        const float cosThetaH = sqrtf(cosThetaHSqr);
        const float sinThetaH = sqrtf(1.0f - cosThetaHSqr);
        const f3 lh = mk(sinThetaH * cosf(phiH), sinThetaH * sinf(phiH), cosThetaH);
        const float k = 2.0f * dot(wo, lh);
        wi = mk(k * lh.x - wo.x, k * lh.y - wo.y, k * lh.z - wo.z);
    } else {
        wi = cosine_hemisphere(u1, u2);
        if (wo.z < 0.0f) wi.z = -wi.z;
    }
    if (wi.z < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    float pdfSpec = 0.0f;
    const f3 brdf = ggx_brdf(wo, base, alpha, metallic, wi, &pdfSpec);
    const float pd = kOneOverPi * fmaxf(wi.z, 0.0f);
    const float pdf = pd + (pdfSpec - pd) * probaSpecular;  // glm::mix(pd, pdfSpec, probaSpecular)
    if (pdf == 0.0f) return mk(0.0f, 0.0f, 0.0f);
    return mk(brdf.x / pdf, brdf.y / pdf, brdf.z / pdf);
}

// Mixture pdf of ggx_sample_eval for a given wi (the `pdf` of MaterialGGX.cpp:86-87),
// used by the extended estimator's multiple importance sampling.
__device__ __forceinline__ float ggx_pdf(f3 wo, f3 base, float roughness, float metallic, f3 wi) {
    if (wi.z < 0.0f) return 0.0f;
    const float pmean = (base.x + base.y + base.z) / 3.0f;
    const float pdiff = 1.0f / (pmean + 1.0f);
    const float probaSpecular = pdiff + (1.0f - pdiff) * metallic;
    const float alpha = alpha_from_roughness(roughness);
    const f3 h = normalize(wi + wo);
    const float NdotH = fmaxf(h.z, 0.0f);
    const float VdotH = fmaxf(dot(wi, h), 0.0f);
    const float pdfSpec = ggx_D(NdotH, alpha) * NdotH / (4.0f * fmaxf(0.0001f, VdotH));
    const float pd = kOneOverPi * fmaxf(wi.z, 0.0f);
    return pd + (pdfSpec - pd) * probaSpecular;
}

// MaterialGGX::eval (MaterialGGX.cpp:94-101).
__device__ __forceinline__ f3 ggx_eval(f3 wo, f3 base, float roughness, float metallic, f3 wi) {
    if (wi.z < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    return ggx_brdf(wo, base, alpha_from_roughness(roughness), metallic, wi, nullptr);
}

// ---- lights -------------------------------------------------------------------------------
// Light::sample(position, dist, attenuation) for the three analytic types.
__device__ __forceinline__ f3 light_sample(const PtLight &l, f3 p, float &dist, float &atten) {
    atten = 0.0f;
    if (l.type == PT_LIGHT_DIRECTIONAL) {
        atten = 1.0f;
        dist = FLT_MAX;
        return mk(-l.direction[0], -l.direction[1], -l.direction[2]);
    }
    f3 d = mk(l.position[0] - p.x, l.position[1] - p.y, l.position[2] - p.z);
    dist = sqrtf(dot(d, d));
    if (dist > l.radius) return mk(0.0f, 0.0f, 0.0f);
    if (dist > 0.0f) d = d / dist;
    const float rr = dist / l.radius;
    const float num = fminf(fmaxf(1.0f - rr * rr, 0.0f), 1.0f);
    if (l.type == PT_LIGHT_POINT) {
        atten = num * num;
        return d;
    }
    const float currentCos = -(d.x * l.direction[0] + d.y * l.direction[1] + d.z * l.direction[2]);
    const float outerCos = cosf(l.half_outer);
    // The reference compares with cos(outerCos), not outerCos (SpotLight.cpp:68); kept.
    if (currentCos < cosf(outerCos)) return mk(0.0f, 0.0f, 0.0f);
    const float innerCos = cosf(l.half_inner);
    const float ang = fminf(fmaxf((currentCos - outerCos) / (innerCos - outerCos), 0.0f), 1.0f);
    atten = ang * num * num;
    return d;
}

// ---- extended estimator: environment map and emitters --------------------------------------
__device__ __forceinline__ float luminance(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

__device__ __forceinline__ float mis_power(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

// Direction <-> equirectangular (u, v): d = (sin t cos p, cos t, sin t sin p), u = p / 2pi, v = t / pi.
__device__ __forceinline__ void dir_to_uv(f3 d, float &u, float &v) {
    float phi = atan2f(d.z, d.x);
    if (phi < 0.0f) phi += kTwoPi;
    u = phi * (1.0f / kTwoPi);
    v = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f)) * kOneOverPi;
}

__device__ __forceinline__ f3 env_radiance(const PtScene &s, f3 d) {
    float u, v;
    dir_to_uv(d, u, v);
    const float4 c = tex_rgbal(s, (uint32_t)s.env_tex, u, v);
    return mk(c.x * s.env_intensity, c.y * s.env_intensity, c.z * s.env_intensity);
}

// Solid-angle pdf of env_sample for direction d (piecewise-constant in (u, v)).
__device__ __forceinline__ float env_pdf(const PtScene &s, f3 d) {
    float u, v;
    dir_to_uv(d, u, v);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - d.y * d.y));
    if (st <= 0.0f || s.env_integral <= 0.0f) return 0.0f;
    const uint32_t x = min((uint32_t)(u * s.env_w), s.env_w - 1), y = min((uint32_t)(v * s.env_h), s.env_h - 1);
    const float p_uv = s.env_func[(size_t)y * s.env_w + x] / s.env_integral;
    return p_uv / (2.0f * kPi * kPi * st);
}

// Sample a piecewise-constant 1-D distribution given its cumulative table (n + 1 entries).
__device__ __forceinline__ float sample_cdf(const float *cdf, uint32_t n, float u, uint32_t &idx) {
    uint32_t lo = 0, hi = n;  // largest i with cdf[i] <= u
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid;
        else hi = mid;
    }
    idx = lo;
    const float w = cdf[lo + 1] - cdf[lo];
    const float du = w > 0.0f ? (u - cdf[lo]) / w : 0.0f;
    return ((float)lo + fminf(fmaxf(du, 0.0f), 0.99999994f)) / (float)n;
}

__device__ __forceinline__ f3 env_sample(const PtScene &s, float u0, float u1, float &pdf) {
    uint32_t row, col;
    const float v = sample_cdf(s.env_marg, s.env_h, u0, row);
    const float u = sample_cdf(s.env_cond + (size_t)row * (s.env_w + 1), s.env_w, u1, col);
    const float theta = v * kPi, phi = u * kTwoPi;
    const float st = sinf(theta);
    const f3 d = mk(st * cosf(phi), cosf(theta), st * sinf(phi));
    const float p_uv = s.env_func[(size_t)row * s.env_w + col] / s.env_integral;
    pdf = st > 0.0f ? p_uv / (2.0f * kPi * kPi * st) : 0.0f;
    return d;
}

// Pick an emitter by power (inclusive CDF) and a uniform point on it.
__device__ __forceinline__ int emitter_pick(const PtScene &s, float u) {
    int lo = 0, hi = s.nemitters - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s.emitter_cdf[mid] <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// ---- geometry helpers --------------------------------------------------------------------
__device__ __forceinline__ int find_object(const PtScene &s, uint32_t prim) {
    int lo = 0, hi = s.nobjects - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s.objects[mid].first_tri <= prim) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ f3 ld3(const float *a, uint32_t i) { return mk(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }

__device__ __forceinline__ f3 mat3_mul(const float *m, f3 v) {
    return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

}  // namespace rgb
