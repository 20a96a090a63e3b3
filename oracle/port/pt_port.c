/*
 * CPU restatement of Rendu's offline path tracer -- ORACLE, test infrastructure only.
 *
 * Restates, in plain C and in the reference's float operation order (glm 0.9.9.7; build
 * with -ffp-contract=off), the per-sample algorithm of
 *   src/apps/pathtracer/PathTracer.cpp   render (159-299), evalBackground (23-55),
 *                                        getSampleGrid/getSamplePosition (57-84),
 *                                        buildLocalFrame (86-122), checkVisibility (124-157)
 *   src/apps/pathtracer/MaterialGGX.cpp  F, D, V, alphaFromRoughness, GGX, sampleAndEval, eval (5-101)
 *   src/engine/generation/Random.cpp     sampleDisk, sampleCosineHemisphere (41-70)
 *   src/engine/resources/Image.cpp       rgbl, rgbal (64-106)
 *   src/engine/resources/Texture.cpp     sampleCubemap (141-191)
 *   src/engine/input/Camera.cpp          pose (10-18), pixelShifts (42-49)
 *   src/engine/scene/lights/            PointLight/DirectionalLight/SpotLight::sample
 * on top of the raycaster restatement in rt_port.c, threaded like System::forParallel
 * (System.hpp:72-104) over image rows.
 *
 * One deliberate difference: the reference draws from per-thread std::mt19937 streams
 * seeded in thread-creation order (Random.cpp:72-80), so its renders are not reproducible.
 * This restatement draws from Philox-4x32-10 indexed by (pixel, sample, bounce) exactly as
 * the CUDA path tracer does, so the two can be compared sample by sample; against the
 * reference itself the comparison is statistical.
 */
#include "pt_port.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "rt_port.h"

typedef struct { float x, y, z; } f3;
typedef struct { float x, y, z, w; } f4;

static inline f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 mul3(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline f3 scl3(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross3(f3 x, f3 y) {
    return mk3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
static inline f3 norm3(f3 v) {
    const float s = 1.0f / sqrtf(dot3(v, v));
    return mk3(v.x * s, v.y * s, v.z * s);
}
static inline float fmaxf_g(float x, float y) { return (x < y) ? y : x; } /* std::max */
static inline float fminf_g(float x, float y) { return (y < x) ? y : x; } /* std::min */

/* ---- Philox-4x32-10 (same stream layout as the CUDA path tracer) -------------------- */
typedef struct { uint32_t x, y, z, w; } u4;
static u4 philox(u4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        u4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
static inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
static inline uint32_t uint_below(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }

/* ---- scene ------------------------------------------------------------------------------ */
typedef struct {
    uint32_t w, h;
    float *rgba;
} tex_t;
typedef struct {
    float *pos, *nrm, *tan, *bit, *uv;
    uint32_t *idx;
    size_t nv, ni;
} mesh_t;
typedef struct {
    uint32_t mesh, material;
    float model[16];
    float invtp[9];
    uint32_t first_tri;
    int use_uv;
} obj_t;

struct port_pt {
    tex_t *tex;
    size_t ntex;
    mesh_t *mesh;
    size_t nmesh;
    pt_material_desc *mat;
    size_t nmat;
    obj_t *obj;
    size_t nobj;
    pt_light_desc *light;
    size_t nlight;
    int bg_mode;
    float bg_color[3];
    uint32_t bg_tex[6];
    f3 sun;          /* ATMOSPHERE: normalised sun direction */
    tex_t sky;       /* ATMOSPHERE: the scattering table (computed at commit unless supplied) */
    port_rc *rc;
    int any_masked;
    /* extended estimator */
    int env_tex;
    float env_intensity;
    struct emitter_t *emitters;
    float *ecdf;
    int nemit;
    double epower;
    uint32_t ew, eh;
    float *efunc, *emarg, *econd;
    double eint;
    float p_env;
};

typedef struct emitter_t {
    float v0[3], e1[3], e2[3], emission[3], lum;
} emitter_t;

#define GROW(arr, n) ((arr) = realloc((arr), sizeof(*(arr)) * ((n) + 1)))

port_pt *port_pt_create(void) {
    port_pt *s = (port_pt *)calloc(1, sizeof(port_pt));
    if (s) s->env_tex = -1;
    return s;
}

int port_pt_set_environment(port_pt *s, uint32_t tex, float intensity) {
    s->env_tex = (int)tex;
    s->env_intensity = intensity;
    return 0;
}

void port_pt_destroy(port_pt *s) {
    if (!s) return;
    for (size_t k = 0; k < s->ntex; ++k) free(s->tex[k].rgba);
    for (size_t k = 0; k < s->nmesh; ++k) {
        free(s->mesh[k].pos); free(s->mesh[k].nrm); free(s->mesh[k].tan);
        free(s->mesh[k].bit); free(s->mesh[k].uv); free(s->mesh[k].idx);
    }
    free(s->tex); free(s->mesh); free(s->mat); free(s->obj); free(s->light);
    free(s->emitters); free(s->ecdf); free(s->efunc); free(s->emarg); free(s->econd);
    free(s->sky.rgba);
    if (s->rc) port_rc_destroy(s->rc);
    free(s);
}

/* Textures are kept as 4-channel float images (missing channels 0, alpha 1). */
int port_pt_add_texture(port_pt *s, uint32_t w, uint32_t h, uint32_t ch, const float *px) {
    GROW(s->tex, s->ntex);
    tex_t *t = &s->tex[s->ntex];
    t->w = w;
    t->h = h;
    t->rgba = (float *)malloc(sizeof(float) * 4 * (size_t)w * h);
    for (size_t p = 0; p < (size_t)w * h; ++p)
        for (uint32_t c = 0; c < 4; ++c) t->rgba[4 * p + c] = c < ch ? px[ch * p + c] : (c == 3 ? 1.0f : 0.0f);
    return (int)s->ntex++;
}

static float *dup(const float *a, size_t n) {
    if (!a) return NULL;
    float *r = (float *)malloc(sizeof(float) * (n ? n : 1));
    memcpy(r, a, sizeof(float) * n);
    return r;
}

int port_pt_add_mesh(port_pt *s, const pt_mesh_desc *d) {
    GROW(s->mesh, s->nmesh);
    mesh_t *m = &s->mesh[s->nmesh];
    m->nv = d->vertex_count;
    m->ni = d->index_count;
    m->pos = dup(d->positions, 3 * m->nv);
    m->nrm = dup(d->normals, 3 * m->nv);
    m->tan = dup(d->tangents, 3 * m->nv);
    m->bit = dup(d->bitangents, 3 * m->nv);
    m->uv = dup(d->texcoords, 2 * m->nv);
    m->idx = (uint32_t *)malloc(sizeof(uint32_t) * (m->ni ? m->ni : 1));
    memcpy(m->idx, d->indices, sizeof(uint32_t) * m->ni);
    return (int)s->nmesh++;
}

int port_pt_add_material(port_pt *s, const pt_material_desc *d) {
    GROW(s->mat, s->nmat);
    s->mat[s->nmat] = *d;
    return (int)s->nmat++;
}

/* inverse(transpose(mat3(model))) as a row-major matrix (same computation as the CUDA
 * path tracer; the reference inverts in float per hit, PathTracer.cpp:94). */
static void normal_matrix(const float *m, float out[9]) {
    double a[3][3], inv[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r][c] = m[4 * c + r];
    const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                       a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[3 * r + c] = (float)inv[c][r];
}

int port_pt_add_object(port_pt *s, uint32_t mesh, uint32_t material, const float *model) {
    GROW(s->obj, s->nobj);
    obj_t *o = &s->obj[s->nobj];
    o->mesh = mesh;
    o->material = material;
    for (int k = 0; k < 16; ++k) o->model[k] = model ? model[k] : ((k % 5) == 0 ? 1.0f : 0.0f);
    normal_matrix(o->model, o->invtp);
    return (int)s->nobj++;
}

int port_pt_add_light(port_pt *s, const pt_light_desc *l) {
    GROW(s->light, s->nlight);
    pt_light_desc d = *l;
    if (d.type != PT_LIGHT_POINT) {  /* DirectionalLight / SpotLight normalise at construction */
        const f3 n = norm3(mk3(d.direction[0], d.direction[1], d.direction[2]));
        d.direction[0] = n.x; d.direction[1] = n.y; d.direction[2] = n.z;
    }
    d.inner_angle *= 0.5f; /* SpotLight stores half angles (SpotLight.cpp:8) */
    d.outer_angle *= 0.5f;
    s->light[s->nlight] = d;
    return (int)s->nlight++;
}

int port_pt_set_background(port_pt *s, int mode, const float *color, const uint32_t *tex) {
    s->bg_mode = mode;
    if (color) memcpy(s->bg_color, color, sizeof(s->bg_color));
    if (tex) memcpy(s->bg_tex, tex, sizeof(s->bg_tex));
    if (mode == PT_BG_ATMOSPHERE && color) /* Sky::setDirection normalises (Sky.cpp:35) */
        s->sun = norm3(mk3(color[0], color[1], color[2]));
    return 0;
}

int port_pt_set_sky_table(port_pt *s, const float *rgba, uint32_t w, uint32_t h) {
    free(s->sky.rgba);
    s->sky.rgba = (float *)malloc(sizeof(float) * 4 * (size_t)w * h);
    if (!s->sky.rgba) return -1;
    memcpy(s->sky.rgba, rgba, sizeof(float) * 4 * (size_t)w * h);
    s->sky.w = w;
    s->sky.h = h;
    return 0;
}

/* PathTracer::PathTracer (PathTracer.cpp:11-21): one raycaster mesh per object, in order. */
int port_pt_commit(port_pt *s) {
    if (s->bg_mode == PT_BG_ATMOSPHERE && !s->sky.rgba) {
        s->sky.rgba = (float *)malloc(sizeof(float) * 4 * PORT_SKY_TABLE_RES * PORT_SKY_TABLE_RES);
        if (!s->sky.rgba) return -1;
        port_sky_table(PORT_SKY_TABLE_RES, PORT_SKY_TABLE_SAMPLES, 1, s->sky.rgba);
        s->sky.w = s->sky.h = PORT_SKY_TABLE_RES;
    }
    if (s->rc) port_rc_destroy(s->rc);
    s->rc = port_rc_create();
    s->any_masked = 0;
    for (size_t o = 0; o < s->nobj; ++o) {
        const mesh_t *m = &s->mesh[s->obj[o].mesh];
        if (port_rc_add_mesh(s->rc, m->pos, m->nv, m->idx, m->ni, s->obj[o].model) < 0) return -1;
        s->obj[o].first_tri = port_rc_mesh_first_tri(s->rc, (uint32_t)o);
        s->obj[o].use_uv = m->uv != NULL; /* Object::Object (Object.cpp:4-8) */
        if (s->mat[s->obj[o].material].masked) s->any_masked = 1;
    }
    /* Extended estimator tables: emissive triangles (power CDF) and the environment's
     * piecewise-constant distribution (luminance x sin(theta)), as the CUDA path tracer. */
    free(s->emitters); free(s->ecdf); free(s->efunc); free(s->emarg); free(s->econd);
    s->emitters = NULL; s->ecdf = NULL; s->efunc = NULL; s->emarg = NULL; s->econd = NULL;
    s->nemit = 0;
    s->epower = 0.0;
    for (size_t o = 0; o < s->nobj; ++o) {
        const obj_t *ob = &s->obj[o];
        const pt_material_desc *md = &s->mat[ob->material];
        if (md->type != PT_MAT_EMISSIVE) continue;
        const tex_t *t = &s->tex[md->tex[0]];
        double e[3] = {0, 0, 0};
        const size_t np = (size_t)t->w * t->h;
        for (size_t q = 0; q < np; ++q)
            for (int c = 0; c < 3; ++c) e[c] += t->rgba[4 * q + c];
        for (int c = 0; c < 3; ++c) e[c] /= (double)np;
        const double lum = 0.2126 * e[0] + 0.7152 * e[1] + 0.0722 * e[2];
        if (!(lum > 0.0)) continue;
        const mesh_t *m = &s->mesh[ob->mesh];
        for (size_t tri = 0; tri + 2 < m->ni; tri += 3) {
            double v[3][3];
            for (int k = 0; k < 3; ++k) {
                const float *pp = &m->pos[3 * (size_t)m->idx[tri + k]];
                for (int r2 = 0; r2 < 3; ++r2)
                    v[k][r2] = (double)ob->model[r2] * pp[0] + (double)ob->model[4 + r2] * pp[1] +
                               (double)ob->model[8 + r2] * pp[2] + (double)ob->model[12 + r2];
            }
            const double u[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
            const double w[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
            const double cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            const double area = 0.5 * sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            if (!(area > 0.0)) continue;
            s->emitters = (emitter_t *)realloc(s->emitters, sizeof(emitter_t) * (s->nemit + 1));
            s->ecdf = (float *)realloc(s->ecdf, sizeof(float) * (s->nemit + 1));
            emitter_t *em = &s->emitters[s->nemit];
            for (int q = 0; q < 3; ++q) {
                em->v0[q] = (float)v[0][q];
                em->e1[q] = (float)u[q];
                em->e2[q] = (float)w[q];
                em->emission[q] = (float)e[q];
            }
            em->lum = (float)lum;
            s->epower += area * lum;
            s->ecdf[s->nemit] = (float)s->epower;
            s->nemit++;
        }
    }
    for (int k = 0; k < s->nemit; ++k) s->ecdf[k] = (float)(s->ecdf[k] / s->epower);
    if (s->nemit) s->ecdf[s->nemit - 1] = 1.0f;
    s->eint = 0.0;
    if (s->env_tex >= 0) {
        const tex_t *t = &s->tex[s->env_tex];
        const uint32_t ew = t->w, eh = t->h;
        s->ew = ew;
        s->eh = eh;
        s->efunc = (float *)malloc(sizeof(float) * (size_t)ew * eh);
        s->econd = (float *)malloc(sizeof(float) * (size_t)eh * (ew + 1));
        s->emarg = (float *)malloc(sizeof(float) * (eh + 1));
        double *rows = (double *)malloc(sizeof(double) * eh);
        for (uint32_t y = 0; y < eh; ++y) {
            const double st = sin(3.14159265358979323846 * (y + 0.5) / eh);
            double acc = 0.0;
            float *cr = s->econd + (size_t)y * (ew + 1);
            cr[0] = 0.0f;
            for (uint32_t x = 0; x < ew; ++x) {
                const float *px = &t->rgba[4 * ((size_t)y * ew + x)];
                const double f = (0.2126 * px[0] + 0.7152 * px[1] + 0.0722 * px[2]) * st * s->env_intensity;
                s->efunc[(size_t)y * ew + x] = (float)f;
                acc += f;
                cr[x + 1] = (float)acc;
            }
            for (uint32_t x = 1; x <= ew; ++x) cr[x] = acc > 0.0 ? (float)(cr[x] / acc) : (float)x / ew;
            cr[ew] = 1.0f;
            rows[y] = acc / ew;
            s->eint += acc;
        }
        double racc = 0.0;
        s->emarg[0] = 0.0f;
        for (uint32_t y = 0; y < eh; ++y) {
            racc += rows[y];
            s->emarg[y + 1] = (float)racc;
        }
        for (uint32_t y = 1; y <= eh; ++y) s->emarg[y] = racc > 0.0 ? (float)(s->emarg[y] / racc) : (float)y / eh;
        s->emarg[eh] = 1.0f;
        s->eint /= (double)ew * eh;
        free(rows);
    }
    if (!(s->eint > 0.0)) s->env_tex = s->env_tex >= 0 && s->eint > 0.0 ? s->env_tex : -1;
    s->p_env = s->env_tex >= 0 ? (s->nemit > 0 ? 0.5f : 1.0f) : 0.0f;
    return port_rc_build(s->rc);
}

/* ---- sampling helpers ------------------------------------------------------------------- */
static inline int mod_pos(int x, int w) { return ((x % w) + w) % w; }

/* Image::rgbal (Image.cpp:86-106). */
static f4 rgbal(const tex_t *t, float x, float y) {
    const float xi = x * (float)t->w, yi = y * (float)t->h;
    const float xb = floorf(xi), yb = floorf(yi);
    const float dx = xi - xb, dy = yi - yb;
    const float cxb = fminf(fmaxf(xb, -2147483520.0f), 2147483520.0f);
    const float cyb = fminf(fmaxf(yb, -2147483520.0f), 2147483520.0f);
    const int x0 = mod_pos((int)cxb, (int)t->w), y0 = mod_pos((int)cyb, (int)t->h);
    const int x1 = mod_pos((int)cxb + 1, (int)t->w), y1 = mod_pos((int)cyb + 1, (int)t->h);
    const float *p00 = t->rgba + 4 * ((size_t)y0 * t->w + x0), *p01 = t->rgba + 4 * ((size_t)y1 * t->w + x0);
    const float *p10 = t->rgba + 4 * ((size_t)y0 * t->w + x1), *p11 = t->rgba + 4 * ((size_t)y1 * t->w + x1);
    float r[4];
    for (int c = 0; c < 4; ++c)
        r[c] = (1.0f - dx) * ((1.0f - dy) * p00[c] + dy * p01[c]) + dx * ((1.0f - dy) * p10[c] + dy * p11[c]);
    f4 o = {r[0], r[1], r[2], r[3]};
    return o;
}

/* Texture::sampleCubemap (Texture.cpp:141-191). */
static f3 cubemap(const port_pt *s, f3 dir) {
    const float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
    int face = 0;
    float x = 0.0f, y = 0.0f, denom = 1.0f;
    if (ax >= ay && ax >= az) {
        denom = ax; y = dir.y; face = dir.x >= 0.0f ? 0 : 1; x = dir.x >= 0.0f ? -dir.z : dir.z;
    } else if (ay >= ax && ay >= az) {
        denom = ay; x = dir.x; face = dir.y >= 0.0f ? 2 : 3; y = dir.y >= 0.0f ? -dir.z : dir.z;
    } else if (az >= ax && az >= ay) {
        denom = az; y = dir.y; face = dir.z >= 0.0f ? 4 : 5; x = dir.z >= 0.0f ? dir.x : -dir.x;
    }
    x = 0.5f * (x / denom) + 0.5f;
    y = 0.5f * (-y / denom) + 0.5f;
    const tex_t *t = &s->tex[s->bg_tex[face]];
    const float eps = 1.0f / (float)(t->w < t->h ? t->w : t->h);
    x = fminf(fmaxf(x, eps), 1.0f - eps);
    y = fminf(fmaxf(y, eps), 1.0f - eps);
    const f4 c = rgbal(t, x, y);
    return mk3(c.x, c.y, c.z);
}

/* ---- atmosphere ------------------------------------------------------------------------ */
/* Sky::AtmosphereParameters (Sky.hpp:53-65): an Earth-like atmosphere. */
static const float SKY_SUN_COLOR[3] = {1.474f, 1.8504f, 1.91198f};
static const float SKY_K_RAYLEIGH[3] = {5.5e-6f, 13.0e-6f, 22.4e-6f};
#define SKY_GROUND 6371e3f
#define SKY_TOP 6471e3f
#define SKY_SUN_INTENSITY 20.0f
#define SKY_K_MIE 21e-6f
#define SKY_H_RAYLEIGH 8000.0f
#define SKY_H_MIE 1200.0f
#define SKY_G_MIE 0.758f
#define SKY_SUN_RADIUS 0.04675f
#define SKY_SUN_RADIUS_COS 0.998f
#define SKY_STEPS 16 /* MaterialSky::samplesCount (MaterialSky.hpp) */

/* Intersection::sphere (Intersection.cpp:7-20): roots of |o + t d| = radius. */
static int sphere_roots(f3 o, f3 d, float radius, float *r0, float *r1) {
    const float a = dot3(d, d), b = dot3(o, d), c = dot3(o, o) - radius * radius;
    const float delta = b * b - a * c;
    if (delta < 0.0f) return 0;
    const float ds = sqrtf(delta);
    *r0 = (-b - ds) / a;
    *r1 = (-b + ds) / a;
    return 1;
}

/* AtmosphereApp::precomputeTable (AtmosphereApp.cpp:145-188): secondary attenuation towards
 * the sun, x = relative height, y = cosine of the sun's vertical angle. */
/* Nearest IEEE binary16 value (round to nearest, ties to even), returned as float: the
 * precision of the reference's stored table. Exact for every float (normals, subnormals,
 * overflow to infinity). */
float port_round_half(float x) {
    union { float f; uint32_t u; } v = {x};
    const uint32_t sign = v.u & 0x80000000u;
    uint32_t a = v.u & 0x7FFFFFFFu;
    if (a >= 0x7F800000u) return x;                                  /* inf, nan */
    if (a >= 0x477FF000u) { v.u = sign | 0x7F800000u; return v.f; }  /* rounds past 65504 */
    const int e = (int)(a >> 23) - 127;
    /* spacing of halves around x: 2^(e-10) for normal halves (e >= -14), 2^-24 below */
    const int q = e >= -14 ? e - 10 : -24;
    /* scale so that the spacing is 1, round to even, scale back (exact in double) */
    const double s = ldexp((double)(v.f < 0 ? -v.f : v.f), -q);
    double r = floor(s);
    const double frac = s - r;
    if (frac > 0.5 || (frac == 0.5 && fmod(r, 2.0) != 0.0)) r += 1.0;
    union { float f; uint32_t u; } o;
    o.f = (float)ldexp(r, q);
    o.u |= sign;
    return o.f;
}

void port_sky_table(uint32_t res, uint32_t samples, int half_precision, float *rgba) {
    for (uint32_t y = 0; y < res; ++y)
        for (uint32_t x = 0; x < res; ++x) {
            const float xf = (float)x / ((float)res - 1.0f), yf = (float)y / ((float)res - 1.0f);
            const f3 pos = mk3(0.0f, (SKY_TOP - SKY_GROUND) * xf + SKY_GROUND, 0.0f);
            const float cosA = 2.0f * yf - 1.0f;
            const float sinA = sqrtf(1.0f - cosA * cosA);
            const f3 n = norm3(mk3(sinA, cosA, 0.0f));
            const f3 sun = mk3(-n.x, -n.y, -n.z);
            float r0 = 0.0f, r1 = 0.0f;
            const int hit = sphere_roots(pos, sun, SKY_TOP, &r0, &r1);
            const float step = hit ? r1 / (float)samples : 0.0f;
            float rd = 0.0f, md = 0.0f;
            for (uint32_t j = 0; j < samples; ++j) {
                const f3 p = add3(pos, scl3(((float)j + 0.5f) * step, sun));
                const float hgt = sqrtf(dot3(p, p)) - SKY_GROUND;
                rd += expf(-hgt / SKY_H_RAYLEIGH) * step;
                md += expf(-hgt / SKY_H_MIE) * step;
            }
            float *o = rgba + 4 * ((size_t)y * res + x);
            for (int c = 0; c < 3; ++c) {
                const float att = expf(-(SKY_K_MIE * md + SKY_K_RAYLEIGH[c] * rd));
                o[c] = half_precision ? port_round_half(att) : att;
            }
            o[3] = 1.0f;
        }
}

/* MaterialSky::rayleighPhase / miePhase (MaterialSky.cpp:89-98). */
static float rayleigh_phase(float c) {
    const float k = 1.0f / (4.0f * 3.14159265358979323846f);
    return k * 3.0f / 4.0f * (1.0f + c * c);
}
static float mie_phase(float c) {
    const float k = 1.0f / (4.0f * 3.14159265358979323846f);
    const float g2 = SKY_G_MIE * SKY_G_MIE;
    return k * 3.0f * (1.0f - g2) / (2.0f * (2.0f + g2)) * (1.0f + c * c) /
           powf(1.0f + g2 - 2.0f * SKY_G_MIE * c, 3.0f / 2.0f);
}

/* MaterialSky::eval (MaterialSky.cpp:6-87): single-scattering march of 16 steps through the
 * atmosphere along the ray, secondary attenuation from the table, plus the sun disc. */
static f3 sky_eval(const tex_t *table, f3 origin, f3 dir, f3 sun) {
    const f3 planet = add3(add3(origin, mk3(0.0f, SKY_GROUND, 0.0f)), mk3(0.0f, 1.0f, 0.0f));
    float t0 = 0.0f, t1 = 0.0f, g0 = 0.0f, g1 = 0.0f;
    if (!sphere_roots(planet, dir, SKY_TOP, &t0, &t1)) return mk3(0.0f, 0.0f, 0.0f);
    const int ground = sphere_roots(planet, dir, SKY_GROUND, &g0, &g1);
    const float dist = fminf_g(t1, ground ? g0 : 0.0f);
    const float step = (dist - t0) / (float)SKY_STEPS;
    const float cos_vs = dot3(dir, sun);
    float rd = 0.0f, md = 0.0f;
    f3 rs = mk3(0, 0, 0), ms = mk3(0, 0, 0), tr = mk3(0, 0, 0);
    for (int i = 0; i < SKY_STEPS; ++i) {
        const f3 p = add3(planet, scl3(((float)i + 0.5f) * step, dir));
        float hgt = sqrtf(dot3(p, p)) - SKY_GROUND;
        if (i == SKY_STEPS - 1 && hgt < 0.0f) hgt = 0.0f;
        const float rstep = expf(-hgt / SKY_H_RAYLEIGH) * step;
        const float mstep = expf(-hgt / SKY_H_MIE) * step;
        rd += rstep;
        md += mstep;
        const f3 direct = mk3(expf(-(md * SKY_K_MIE + rd * SKY_K_RAYLEIGH[0])),
                              expf(-(md * SKY_K_MIE + rd * SKY_K_RAYLEIGH[1])),
                              expf(-(md * SKY_K_MIE + rd * SKY_K_RAYLEIGH[2])));
        const float rel_h = (sqrtf(dot3(p, p)) - SKY_GROUND) / (SKY_TOP - SKY_GROUND);
        const float rel_c = -0.5f * sun.y + 0.5f;
        float u = (511.0f / 512.0f) * rel_h + 0.5f / 512.0f, v = (511.0f / 512.0f) * rel_c + 0.5f / 512.0f;
        u = fminf_g(fmaxf_g(u, 0.5f / 512.0f), 511.0f / 512.0f); /* glm::clamp */
        v = fminf_g(fmaxf_g(v, 0.5f / 512.0f), 511.0f / 512.0f);
        const f4 sec = rgbal(table, u, v);
        const f3 att = mul3(direct, mk3(sec.x, sec.y, sec.z));
        rs = add3(rs, scl3(rstep, att));
        ms = add3(ms, scl3(mstep, att));
        tr = add3(tr, direct);
    }
    const f3 rp = mul3(scl3(rayleigh_phase(cos_vs), mk3(SKY_K_RAYLEIGH[0], SKY_K_RAYLEIGH[1], SKY_K_RAYLEIGH[2])), rs);
    const f3 mp = scl3(SKY_K_MIE * mie_phase(cos_vs), ms);
    f3 sun_r = mk3(0.0f, 0.0f, 0.0f);
    const int ground_forward = ground && g1 > 0.0f;
    if (!ground_forward && dot3(dir, sun) > SKY_SUN_RADIUS_COS) {
        const float area = 3.14159265358979323846f * SKY_SUN_RADIUS * SKY_SUN_RADIUS;
        sun_r = mk3(SKY_SUN_COLOR[0] / area, SKY_SUN_COLOR[1] / area, SKY_SUN_COLOR[2] / area);
    }
    return add3(scl3(SKY_SUN_INTENSITY, add3(rp, mp)), mul3(tr, sun_r));
}

void port_sky_eval(const float *table, uint32_t w, uint32_t h, const float *cases, size_t n, float *out) {
    tex_t t = {w, h, (float *)table};
    for (size_t i = 0; i < n; ++i) {
        const float *c = cases + 9 * i;
        const f3 r = sky_eval(&t, mk3(c[0], c[1], c[2]), mk3(c[3], c[4], c[5]), mk3(c[6], c[7], c[8]));
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
}

/* PathTracer::evalBackground (PathTracer.cpp:23-55): SKYBOX and ATMOSPHERE for every miss
 * (the atmosphere at the ray's origin), COLOR and IMAGE for primary misses only. */
static f3 background(const port_pt *s, f3 pos, f3 dir, float nx, float ny, int direct) {
    if (s->bg_mode == PT_BG_SKYBOX) return cubemap(s, norm3(dir));
    if (s->bg_mode == PT_BG_ATMOSPHERE) return sky_eval(&s->sky, pos, norm3(dir), s->sun);
    if (!direct) return mk3(0, 0, 0);
    if (s->bg_mode == PT_BG_IMAGE) {
        const f4 c = rgbal(&s->tex[s->bg_tex[0]], nx, ny);
        return mk3(c.x, c.y, c.z);
    }
    return mk3(s->bg_color[0], s->bg_color[1], s->bg_color[2]);
}

/* ---- MaterialGGX (MaterialGGX.cpp:5-101) ------------------------------------------------- */
static const float ONE_OVER_PI = 0.318309886183790671538f;
static const float TWO_PI = 6.28318530717958647692f;
static const float PI_F = 3.14159265358979323846f;

static f3 ggx_F(f3 F0, float VdotH) {
    const float p = powf(1.0f - VdotH, 5.0f);
    return add3(F0, scl3(p, sub3(mk3(1, 1, 1), F0)));
}
static float ggx_D(float NdotH, float alpha) {
    const float halfDenum = NdotH * NdotH * (alpha * alpha - 1.0f) + 1.0f;
    const float halfTerm = alpha / fmaxf_g(0.0001f, halfDenum);
    return halfTerm * halfTerm * ONE_OVER_PI;
}
static float ggx_V(float NdotL, float NdotV, float alpha) {
    const float alpha2 = alpha * alpha;
    const float visL = NdotV * sqrtf((-NdotL * alpha2 + NdotL) * NdotL + alpha2);
    const float visV = NdotL * sqrtf((-NdotV * alpha2 + NdotV) * NdotV + alpha2);
    return 0.5f / fmaxf_g(0.0001f, visV + visL);
}
static float alpha_from_roughness(float r) {
    const float rc = fmaxf_g(0.045f, r);
    return fmaxf_g(0.0001f, rc * rc);
}
static f3 ggx(f3 wo, f3 base, float alpha, float metal, f3 wi, float *pdf) {
    const f3 h = norm3(add3(wi, wo));
    const float NdotH = fmaxf_g(h.z, 0.0f);
    const float VdotH = fmaxf_g(dot3(wi, h), 0.0f);
    const float NdotL = fmaxf_g(wo.z, 0.0f);
    const float NdotV = fmaxf_g(wi.z, 0.0f);
    const float Dh = ggx_D(NdotH, alpha);
    if (pdf) *pdf = Dh * NdotH / (4.0f * fmaxf_g(0.0001f, VdotH));
    const f3 F0 = add3(mk3(0.04f, 0.04f, 0.04f), scl3(metal, sub3(base, mk3(0.04f, 0.04f, 0.04f))));
    const f3 specular = scl3(Dh * ggx_V(NdotL, NdotV, alpha), ggx_F(F0, VdotH));
    const f3 diffuse = mul3(scl3((1.0f - metal) * ONE_OVER_PI, base), sub3(mk3(1, 1, 1), F0));
    const f3 multiAdj = add3(mk3(1, 1, 1), scl3(2.0f * alpha * alpha * NdotV, F0));
    return scl3(NdotV, add3(diffuse, mul3(specular, multiAdj)));
}
static f3 cosine_hemisphere(float u0, float u1) {
    const float x = 2.0f * u0 - 1.0f, y = 2.0f * u1 - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(x == 0.0f && y == 0.0f)) {
        float angle, radius;
        if (fabsf(x) > fabsf(y)) {
            radius = x;
            angle = (0.25f * PI_F) * y / x;
        } else {
            radius = y;
            angle = 0.5f * PI_F - (0.25f * PI_F) * x / y;
        }
        dx = radius * cosf(angle);
        dy = radius * sinf(angle);
    }
    return mk3(dx, dy, sqrtf(fmaxf_g(0.0f, 1.0f - dx * dx - dy * dy)));
}
static f3 ggx_sample_eval(f3 wo, f3 base, float rough, float metal, float u0, float u1, float u2, f3 *wi) {
    const float pdiff = 1.0f / (dot3(base, mk3(1, 1, 1)) / 3.0f + 1.0f);
    const float probaSpecular = pdiff + metal * (1.0f - pdiff);
    const float alpha = alpha_from_roughness(rough);
    if (u0 < probaSpecular) {
        const float a2 = alpha * alpha;
        const float x = u1;
        const float phiH = u2 * TWO_PI;
        const float cosThetaHSqr = fminf_g((1.0f - x) / ((a2 - 1.0f) * x + 1.0f), 1.0f);
        const float cosThetaH = sqrtf(cosThetaHSqr);
        const float sinThetaH = sqrtf(1.0f - cosThetaHSqr);
        const f3 lh = mk3(sinThetaH * cosf(phiH), sinThetaH * sinf(phiH), cosThetaH);
        *wi = sub3(scl3(2.0f * dot3(wo, lh), lh), wo);
    } else {
        *wi = cosine_hemisphere(u1, u2);
        if (wo.z < 0.0f) wi->z *= -1.0f;
    }
    if (wi->z < 0.0f) return mk3(0, 0, 0);
    float pdfSpec = 0.0f;
    const f3 brdf = ggx(wo, base, alpha, metal, *wi, &pdfSpec);
    const float pd = ONE_OVER_PI * fmaxf_g(wi->z, 0.0f);
    const float pdf = pd + probaSpecular * (pdfSpec - pd);
    if (pdf == 0.0f) return mk3(0, 0, 0);
    return mk3(brdf.x / pdf, brdf.y / pdf, brdf.z / pdf);
}
static f3 ggx_eval(f3 wo, f3 base, float rough, float metal, f3 wi) {
    if (wi.z < 0.0f) return mk3(0, 0, 0);
    return ggx(wo, base, alpha_from_roughness(rough), metal, wi, NULL);
}

void port_ggx_eval(const float *c, size_t n, float *out) {
    for (size_t i = 0; i < n; ++i) {
        const float *q = c + 11 * i;
        const f3 r = ggx_eval(mk3(q[0], q[1], q[2]), mk3(q[3], q[4], q[5]), q[6], q[7], mk3(q[8], q[9], q[10]));
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}

void port_ggx_sample(const float *c, const float *u, size_t n, float *out) {
    for (size_t i = 0; i < n; ++i) {
        const float *q = c + 8 * i;
        f3 wi = mk3(0, 0, 0);
        const f3 r = ggx_sample_eval(mk3(q[0], q[1], q[2]), mk3(q[3], q[4], q[5]), q[6], q[7], u[3 * i], u[3 * i + 1],
                                     u[3 * i + 2], &wi);
        float *o = out + 6 * i;
        o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = wi.x; o[4] = wi.y; o[5] = wi.z;
    }
}

/* ---- lights ------------------------------------------------------------------------------ */
static f3 light_sample(const pt_light_desc *l, f3 p, float *dist, float *atten) {
    *atten = 0.0f;
    if (l->type == PT_LIGHT_DIRECTIONAL) {
        *atten = 1.0f;
        *dist = FLT_MAX;
        return mk3(-l->direction[0], -l->direction[1], -l->direction[2]);
    }
    f3 d = sub3(mk3(l->position[0], l->position[1], l->position[2]), p);
    *dist = sqrtf(dot3(d, d));
    if (*dist > l->radius) return mk3(0, 0, 0);
    if (*dist > 0.0f) d = mk3(d.x / *dist, d.y / *dist, d.z / *dist);
    const float rr = *dist / l->radius;
    const float num = fminf(fmaxf(1.0f - rr * rr, 0.0f), 1.0f);
    if (l->type == PT_LIGHT_POINT) {
        *atten = num * num;
        return d;
    }
    const float currentCos = dot3(mk3(-d.x, -d.y, -d.z), mk3(l->direction[0], l->direction[1], l->direction[2]));
    const float outerCos = cosf(l->outer_angle);
    if (currentCos < cosf(outerCos)) return mk3(0, 0, 0); /* SpotLight.cpp:68 */
    const float innerCos = cosf(l->inner_angle);
    const float ang = fminf(fmaxf((currentCos - outerCos) / (innerCos - outerCos), 0.0f), 1.0f);
    *atten = ang * num * num;
    return d;
}

/* Camera::pose + Camera::pixelShifts. out12 = corner, dx, dy, eye. */
void port_pixel_shifts(const pt_camera_desc *c, float *out) {
    const f3 e = mk3(c->eye[0], c->eye[1], c->eye[2]), ce = mk3(c->center[0], c->center[1], c->center[2]);
    f3 up = norm3(mk3(c->up[0], c->up[1], c->up[2]));
    const f3 view = norm3(sub3(ce, e));
    const f3 right = cross3(view, up);
    up = cross3(right, view);
    const float hs = tanf(0.5f * c->fov);
    const float ws = c->ratio * hs;
    const f3 de = sub3(ce, e);
    const float dist = sqrtf(dot3(de, de));
    const f3 corner = add3(ce, scl3(dist, add3(scl3(-ws, right), scl3(hs, up))));
    const f3 dx = scl3(2.0f * ws * dist, right);
    const f3 dy = scl3(-2.0f * hs * dist, up);
    const float v[12] = {corner.x, corner.y, corner.z, dx.x, dx.y, dx.z, dy.x, dy.y, dy.z, e.x, e.y, e.z};
    memcpy(out, v, sizeof(v));
}

/* ---- extended estimator helpers (same definitions as the CUDA path tracer) ----------- */
static float luminance3(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
static float mis_power(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}
static void dir_to_uv(f3 d, float *u, float *v) {
    float phi = atan2f(d.z, d.x);
    if (phi < 0.0f) phi += TWO_PI;
    *u = phi * (1.0f / TWO_PI);
    *v = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f)) * ONE_OVER_PI;
}
static f3 env_radiance(const port_pt *s, f3 d) {
    float u, v;
    dir_to_uv(d, &u, &v);
    const f4 c = rgbal(&s->tex[s->env_tex], u, v);
    return mk3(c.x * s->env_intensity, c.y * s->env_intensity, c.z * s->env_intensity);
}
static float env_pdf(const port_pt *s, f3 d) {
    float u, v;
    dir_to_uv(d, &u, &v);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - d.y * d.y));
    if (st <= 0.0f || s->eint <= 0.0) return 0.0f;
    uint32_t x = (uint32_t)(u * s->ew), y = (uint32_t)(v * s->eh);
    if (x > s->ew - 1) x = s->ew - 1;
    if (y > s->eh - 1) y = s->eh - 1;
    const float p_uv = s->efunc[(size_t)y * s->ew + x] / (float)s->eint;
    return p_uv / (2.0f * PI_F * PI_F * st);
}
static float sample_cdf(const float *cdf, uint32_t n, float u, uint32_t *idx) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid;
        else hi = mid;
    }
    *idx = lo;
    const float w = cdf[lo + 1] - cdf[lo];
    float du = w > 0.0f ? (u - cdf[lo]) / w : 0.0f;
    du = fminf(fmaxf(du, 0.0f), 0.99999994f);
    return ((float)lo + du) / (float)n;
}
static f3 env_sample(const port_pt *s, float u0, float u1, float *pdf) {
    uint32_t row, col;
    const float v = sample_cdf(s->emarg, s->eh, u0, &row);
    const float u = sample_cdf(s->econd + (size_t)row * (s->ew + 1), s->ew, u1, &col);
    const float theta = v * PI_F, phi = u * TWO_PI;
    const float st = sinf(theta);
    const f3 d = mk3(st * cosf(phi), cosf(theta), st * sinf(phi));
    const float p_uv = s->efunc[(size_t)row * s->ew + col] / (float)s->eint;
    *pdf = st > 0.0f ? p_uv / (2.0f * PI_F * PI_F * st) : 0.0f;
    return d;
}
static int emitter_pick(const port_pt *s, float u) {
    int lo = 0, hi = s->nemit - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s->ecdf[mid] <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
static float ggx_pdf(f3 wo, f3 base, float rough, float metal, f3 wi) {
    if (wi.z < 0.0f) return 0.0f;
    const float pdiff = 1.0f / (dot3(base, mk3(1, 1, 1)) / 3.0f + 1.0f);
    const float ps = pdiff + metal * (1.0f - pdiff);
    const float alpha = alpha_from_roughness(rough);
    const f3 h = norm3(add3(wi, wo));
    const float NdotH = fmaxf_g(h.z, 0.0f);
    const float VdotH = fmaxf_g(dot3(wi, h), 0.0f);
    const float pdfSpec = ggx_D(NdotH, alpha) * NdotH / (4.0f * fmaxf_g(0.0001f, VdotH));
    const float pd = ONE_OVER_PI * fmaxf_g(wi.z, 0.0f);
    return pd + ps * (pdfSpec - pd);
}

/* ---- render ------------------------------------------------------------------------------ */
typedef struct {
    int obj;
    uint32_t i0, i1, i2;
    float u, v, w;
} surf_t;

static surf_t surface(const port_pt *s, const port_hit *h) {
    surf_t r;
    r.obj = (int)port_rc_prim_mesh(s->rc, h->prim);
    const obj_t *o = &s->obj[r.obj];
    const mesh_t *m = &s->mesh[o->mesh];
    const uint32_t local = h->prim - o->first_tri;
    r.i0 = m->idx[3 * local];
    r.i1 = m->idx[3 * local + 1];
    r.i2 = m->idx[3 * local + 2];
    r.u = h->u;
    r.v = h->v;
    r.w = 1.0f - h->u - h->v;
    return r;
}

/* Raycaster::interpolateAttribute: w*A[i0] + u*A[i1] + v*A[i2]. */
static f3 interp3(const float *a, const surf_t *h) {
    const f3 a0 = mk3(a[3 * h->i0], a[3 * h->i0 + 1], a[3 * h->i0 + 2]);
    const f3 a1 = mk3(a[3 * h->i1], a[3 * h->i1 + 1], a[3 * h->i1 + 2]);
    const f3 a2 = mk3(a[3 * h->i2], a[3 * h->i2 + 1], a[3 * h->i2 + 2]);
    return add3(add3(scl3(h->w, a0), scl3(h->u, a1)), scl3(h->v, a2));
}

static void interp_uv(const float *a, const surf_t *h, float *u, float *v) {
    *u = (h->w * a[2 * h->i0] + h->u * a[2 * h->i1]) + h->v * a[2 * h->i2];
    *v = (h->w * a[2 * h->i0 + 1] + h->u * a[2 * h->i1 + 1]) + h->v * a[2 * h->i2 + 1];
}

static f3 mat3mul(const float *m, f3 v) {
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
               m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

static inline void ray8(float *r, f3 o, float tmin, f3 d, float tmax) {
    r[0] = o.x; r[1] = o.y; r[2] = o.z; r[3] = tmin; r[4] = d.x; r[5] = d.y; r[6] = d.z; r[7] = tmax;
}

/* PathTracer::checkVisibility (PathTracer.cpp:124-157). */
static int check_visibility(const port_pt *s, f3 start, f3 dir, float maxd, uint64_t *nrays) {
    f3 lpos = start;
    while (maxd > 0.0f) {
        float r[8];
        ray8(r, lpos, 0.001f, dir, maxd);
        port_hit h;
        (*nrays)++;
        if (!port_rc_closest1(s->rc, r, &h)) return 1;
        const surf_t sh = surface(s, &h);
        const obj_t *o = &s->obj[sh.obj];
        const pt_material_desc *m = &s->mat[o->material];
        if (!m->masked || !o->use_uv) return 0;
        float u, v;
        interp_uv(s->mesh[o->mesh].uv, &sh, &u, &v);
        if (rgbal(&s->tex[m->tex[0]], u, v).w < 0.01f) {
            maxd = maxd - h.t;
            lpos = add3(lpos, scl3(h.t, dir));
        } else {
            return 0;
        }
    }
    return 1;
}

typedef struct {
    const port_pt *s;
    float corner[3], dx[3], dy[3], eye[3];
    uint32_t W, H, spp, depth, cx, cy;
    float cellx, celly;
    uint32_t seed_lo, seed_hi;
    int mode;
    float clamp;
    float *image;
    size_t y0, y1;
    uint64_t rays[3];
} job_t;

static void render_pixel(job_t *j, uint32_t x, uint32_t y) {
    const port_pt *s = j->s;
    const uint32_t pixel = y * j->W + x;
    float *px = j->image + 3 * (size_t)pixel;
    for (uint32_t sid = 0; sid < j->spp; ++sid) {
        const u4 rg = philox((u4){pixel, sid, 0u, 0u}, j->seed_lo, j->seed_hi);
        const float jx = u01(rg.x), jy = u01(rg.y);
        const int sidy = (int)sid / (int)j->cx, sidx = (int)sid % (int)j->cx;
        const float sx = (float)x + ((float)sidx + jx) * j->cellx;
        const float sy = (float)y + ((float)sidy + jy) * j->celly;
        const float nx = sx / (float)j->W, ny = sy / (float)j->H;
        const f3 world = add3(add3(mk3(j->corner[0], j->corner[1], j->corner[2]), scl3(nx, mk3(j->dx[0], j->dx[1], j->dx[2]))),
                              scl3(ny, mk3(j->dy[0], j->dy[1], j->dy[2])));
        const f3 eye = mk3(j->eye[0], j->eye[1], j->eye[2]);
        f3 pos = eye, dir = norm3(sub3(world, eye));
        f3 color = mk3(0, 0, 0), atten = mk3(1, 1, 1);
        const int ext = j->mode == PT_MODE_EXTENDED;
        float prev_pdf = 0.0f;
        for (uint32_t did = 0; did < j->depth; ++did) {
            float r[8];
            ray8(r, pos, 1e-4f, dir, 1e8f);
            port_hit h;
            j->rays[did == 0 ? 0 : 1]++;
            if (!port_rc_closest1(s->rc, r, &h)) {
                if (ext && s->env_tex >= 0) {
                    float wgt = 1.0f;
                    if (did > 0 && prev_pdf > 0.0f) wgt = mis_power(prev_pdf, s->p_env * env_pdf(s, dir));
                    color = add3(color, mul3(atten, scl3(wgt, env_radiance(s, dir))));
                } else {
                    color = add3(color, mul3(atten, background(s, pos, dir, nx, ny, did == 0)));
                }
                break;
            }
            const surf_t sh = surface(s, &h);
            const obj_t *o = &s->obj[sh.obj];
            const mesh_t *mesh = &s->mesh[o->mesh];
            const pt_material_desc *mat = &s->mat[o->material];
            const f3 p = add3(pos, scl3(h.t, dir));
            float u = 0.5f, v = 0.5f;
            if (o->use_uv) interp_uv(mesh->uv, &sh, &u, &v);
            const f4 bcol = rgbal(&s->tex[mat->tex[0]], u, v);
            if (mat->masked && bcol.w < 0.01f) {
                pos = p;
                continue;
            }
            if (mat->type == PT_MAT_EMISSIVE) {
                f3 le = mk3(bcol.x, bcol.y, bcol.z);
                if (ext && did > 0 && prev_pdf > 0.0f && s->nemit > 0) {
                    const f3 p0 = mk3(mesh->pos[3 * sh.i0], mesh->pos[3 * sh.i0 + 1], mesh->pos[3 * sh.i0 + 2]);
                    const f3 p1 = mk3(mesh->pos[3 * sh.i1], mesh->pos[3 * sh.i1 + 1], mesh->pos[3 * sh.i1 + 2]);
                    const f3 p2 = mk3(mesh->pos[3 * sh.i2], mesh->pos[3 * sh.i2 + 1], mesh->pos[3 * sh.i2 + 2]);
                    const f3 ng = norm3(mat3mul(o->invtp, cross3(sub3(p1, p0), sub3(p2, p0))));
                    const float cosl = fabsf(dot3(ng, dir));
                    const float pl = cosl > 0.0f
                                         ? (1.0f - s->p_env) * luminance3(le) * h.t * h.t / ((float)s->epower * cosl)
                                         : 0.0f;
                    le = scl3(mis_power(prev_pdf, pl), le);
                }
                color = add3(color, mul3(atten, le));
                break;
            }
            /* buildLocalFrame */
            const f3 nn = norm3(interp3(mesh->nrm, &sh));
            const f3 tt = norm3(interp3(mesh->tan, &sh));
            const f3 bb = norm3(interp3(mesh->bit, &sh));
            f3 t0 = mat3mul(o->invtp, tt), t1 = mat3mul(o->invtp, bb), t2 = mat3mul(o->invtp, nn);
            if (!(dot3(t2, dir) < 0.0f)) t2 = scl3(-1.0f, t2);
            if (o->use_uv) {
                const f4 img = rgbal(&s->tex[mat->tex[1]], u, v);
                const f3 ln = norm3(sub3(scl3(2.0f, mk3(img.x, img.y, img.z)), mk3(1, 1, 1)));
                t2 = add3(add3(scl3(ln.x, t0), scl3(ln.y, t1)), scl3(ln.z, t2));
            }
            t2 = norm3(t2);
            t1 = norm3(cross3(t2, norm3(t0)));
            t0 = norm3(cross3(t1, t2));
            const f3 md = scl3(-1.0f, dir);
            const f3 wo = norm3(mk3(dot3(t0, md), dot3(t1, md), dot3(t2, md)));
            const f3 base = mk3(powf(bcol.x, 2.2f), powf(bcol.y, 2.2f), powf(bcol.z, 2.2f));
            const f4 rmao = rgbal(&s->tex[mat->tex[2]], u, v);
            const u4 rnd = philox((u4){pixel, sid, did + 1u, 0u}, j->seed_lo, j->seed_hi);
            if (s->nlight > 0) {
                const pt_light_desc *L = &s->light[uint_below(rnd.x, (uint32_t)s->nlight)];
                const f3 ps = add3(p, scl3(0.001f, t2));
                float maxd, fall;
                const f3 ld = light_sample(L, ps, &maxd, &fall);
                int visible = fall > 0.0f;
                if (visible && L->cast_shadows) {
                    j->rays[2]++;
                    uint64_t extra = 0;
                    visible = check_visibility(s, ps, ld, maxd, &extra);
                    j->rays[2] += extra - 1;
                }
                if (visible) {
                    const f3 lwi = norm3(mk3(dot3(t0, ld), dot3(t1, ld), dot3(t2, ld)));
                    const f3 ev = ggx_eval(wo, base, rmao.x, rmao.y, lwi);
                    const float lightPdf = 1.0f / (float)s->nlight;
                    const f3 ill = mk3(fall * ev.x * L->color[0] / lightPdf, fall * ev.y * L->color[1] / lightPdf,
                                       fall * ev.z * L->color[2] / lightPdf);
                    color = add3(color, mul3(atten, ill));
                }
            }
            if (ext && (s->nemit > 0 || s->env_tex >= 0)) {
                const u4 r2 = philox((u4){pixel, sid, did + 1u, 1u}, j->seed_lo, j->seed_hi);
                const float usel = u01(r2.x);
                const f3 ps = add3(p, scl3(0.001f, t2));
                f3 ld = mk3(0, 0, 1), le = mk3(0, 0, 0);
                float pl = 0.0f, dist = 1e8f;
                int ok = 0;
                if (s->env_tex >= 0 && (s->nemit == 0 || usel < s->p_env)) {
                    ld = env_sample(s, u01(r2.y), u01(r2.z), &pl);
                    pl *= s->p_env;
                    le = env_radiance(s, ld);
                    ok = pl > 0.0f;
                } else if (s->nemit > 0) {
                    float ue = s->env_tex >= 0 ? (usel - s->p_env) / (1.0f - s->p_env) : usel;
                    ue = fminf(fmaxf(ue, 0.0f), 0.99999994f);
                    const emitter_t *em = &s->emitters[emitter_pick(s, ue)];
                    const float su = sqrtf(u01(r2.y)), b1 = 1.0f - su, b2 = u01(r2.z) * su;
                    const f3 e1 = mk3(em->e1[0], em->e1[1], em->e1[2]), e2 = mk3(em->e2[0], em->e2[1], em->e2[2]);
                    const f3 q = add3(add3(mk3(em->v0[0], em->v0[1], em->v0[2]), scl3(b1, e1)), scl3(b2, e2));
                    const f3 dq = sub3(q, ps);
                    const float d2 = dot3(dq, dq);
                    dist = sqrtf(d2);
                    ld = mk3(dq.x / dist, dq.y / dist, dq.z / dist);
                    const f3 ng = norm3(cross3(e1, e2));
                    const float cosl = fabsf(dot3(ng, ld));
                    le = mk3(em->emission[0], em->emission[1], em->emission[2]);
                    pl = cosl > 0.0f ? (1.0f - s->p_env) * em->lum * d2 / ((float)s->epower * cosl) : 0.0f;
                    ok = pl > 0.0f && dist > 0.0f;
                }
                if (ok) {
                    const f3 lwi = norm3(mk3(dot3(t0, ld), dot3(t1, ld), dot3(t2, ld)));
                    const f3 ev = ggx_eval(wo, base, rmao.x, rmao.y, lwi);
                    const float pb = ggx_pdf(wo, base, rmao.x, rmao.y, lwi);
                    const float wgt = mis_power(pl, pb) / pl;
                    const f3 contrib = scl3(wgt, mul3(atten, mul3(ev, le)));
                    if (contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f) {
                        j->rays[2]++;
                        uint64_t extra = 0;
                        const int vis = check_visibility(s, ps, ld, dist < 1e8f ? dist * (1.0f - 1e-3f) : 1e8f, &extra);
                        j->rays[2] += extra - 1;
                        if (vis) color = add3(color, contrib);
                    }
                }
            }
            f3 wi;
            const f3 w = ggx_sample_eval(wo, base, rmao.x, rmao.y, u01(rnd.y), u01(rnd.z), u01(rnd.w), &wi);
            if (ext) prev_pdf = (w.x > 0.0f || w.y > 0.0f || w.z > 0.0f) ? ggx_pdf(wo, base, rmao.x, rmao.y, wi) : 0.0f;
            const f3 nd = norm3(add3(add3(scl3(wi.x, t0), scl3(wi.y, t1)), scl3(wi.z, t2)));
            atten = mul3(atten, w);
            if (did < j->depth - 1) {
                pos = p;
                dir = norm3(nd);
            }
        }
        /* render.rgb(x,y) += min(sampleColor, 5.0f) (clamp value: an option of the extended mode) */
        if (j->clamp > 0.0f) {
            const float cl = j->clamp;
            px[0] += (cl < color.x) ? cl : color.x;
            px[1] += (cl < color.y) ? cl : color.y;
            px[2] += (cl < color.z) ? cl : color.z;
        } else {
            px[0] += color.x;
            px[1] += color.y;
            px[2] += color.z;
        }
    }
    px[0] = px[0] / (float)j->spp;
    px[1] = px[1] / (float)j->spp;
    px[2] = px[2] / (float)j->spp;
}

static void *render_rows(void *arg) {
    job_t *j = (job_t *)arg;
    for (size_t y = j->y0; y < j->y1; ++y)
        for (uint32_t x = 0; x < j->W; ++x) render_pixel(j, x, (uint32_t)y);
    return NULL;
}

int port_pt_render(port_pt *s, const pt_camera_desc *cam, uint32_t samples, uint32_t depth, uint64_t seed, float *image,
                   uint32_t W, uint32_t H, int threads, uint64_t *rays_out) {
    return port_pt_render_ex(s, cam, samples, depth, seed, image, W, H, threads, rays_out, PT_MODE_REFERENCE, 5.0f);
}

int port_pt_render_ex(port_pt *s, const pt_camera_desc *cam, uint32_t samples, uint32_t depth, uint64_t seed,
                      float *image, uint32_t W, uint32_t H, int threads, uint64_t *rays_out, int mode, float clamp) {
    if (!s || !s->rc || !cam || !image || samples == 0 || W == 0 || H == 0) return -1;
    job_t base;
    memset(&base, 0, sizeof(base));
    base.s = s;
    float sh[12];
    port_pixel_shifts(cam, sh);
    memcpy(base.corner, sh, 12);
    memcpy(base.dx, sh + 3, 12);
    memcpy(base.dy, sh + 6, 12);
    memcpy(base.eye, sh + 9, 12);
    base.spp = (uint32_t)pow(2.0, round(log2((float)samples)));
    const int k = (int)floor(log2((double)base.spp));
    base.cx = (uint32_t)pow(2, k / 2);
    base.cy = base.cx;
    if (k % 2 == 1) {
        base.cx = (uint32_t)pow(2, (k + 1) / 2);
        base.cy = (uint32_t)pow(2, (k - 1) / 2);
    }
    base.cellx = 1.0f / (float)base.cx;
    base.celly = 1.0f / (float)base.cy;
    base.W = W;
    base.H = H;
    base.depth = depth;
    base.seed_lo = (uint32_t)seed;
    base.seed_hi = (uint32_t)(seed >> 32);
    base.mode = mode;
    base.clamp = clamp;
    base.image = image;
    if (threads <= 0) threads = port_default_threads();
    size_t count = (size_t)threads < H ? (size_t)threads : H;
    const size_t span = H / count > 0 ? H / count : 1;
    pthread_t *th = (pthread_t *)malloc(count * sizeof(pthread_t));
    job_t *jobs = (job_t *)malloc(count * sizeof(job_t));
    for (size_t t = 0; t < count; ++t) {
        jobs[t] = base;
        jobs[t].y0 = t * span;
        jobs[t].y1 = (t == count - 1) ? H : (t + 1) * span;
        pthread_create(&th[t], NULL, render_rows, &jobs[t]);
    }
    uint64_t rays[3] = {0, 0, 0};
    for (size_t t = 0; t < count; ++t) {
        pthread_join(th[t], NULL);
        for (int q = 0; q < 3; ++q) rays[q] += jobs[t].rays[q];
    }
    if (rays_out) memcpy(rays_out, rays, sizeof(rays));
    free(th);
    free(jobs);
    return 0;
}
