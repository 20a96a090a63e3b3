/*
 * CPU restatement of Rendu's PathTracer::render -- ORACLE, test infrastructure only.
 * Declarations for oracle/port/pt_port.c. Scene descriptions use the structs of the
 * product's C-ABI header (pt_mesh_desc, pt_material_desc, pt_light_desc, pt_camera_desc).
 */
#ifndef RENDU_ORACLE_PT_PORT_H
#define RENDU_ORACLE_PT_PORT_H
#include <stddef.h>
#include <stdint.h>

#include "rendu_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_pt port_pt;

port_pt *port_pt_create(void);
void port_pt_destroy(port_pt *s);
int port_pt_add_texture(port_pt *s, uint32_t w, uint32_t h, uint32_t channels, const float *px);
int port_pt_add_mesh(port_pt *s, const pt_mesh_desc *m);
int port_pt_add_material(port_pt *s, const pt_material_desc *m);
int port_pt_add_object(port_pt *s, uint32_t mesh, uint32_t material, const float *model);
int port_pt_add_light(port_pt *s, const pt_light_desc *l);
int port_pt_set_background(port_pt *s, int mode, const float *color, const uint32_t *tex);
int port_pt_commit(port_pt *s);
/* Accumulates into image (h x w x 3) and normalises, as PathTracer::render. rays_out (3
 * counters: primary, bounce, shadow) may be NULL. threads <= 0: hardware threads - 1. */
int port_pt_render(port_pt *s, const pt_camera_desc *cam, uint32_t samples, uint32_t depth, uint64_t seed, float *image,
                   uint32_t w, uint32_t h, int threads, uint64_t *rays_out);
/* Extended estimator (PT_MODE_EXTENDED): environment map and render options. */
int port_pt_set_environment(port_pt *s, uint32_t tex, float intensity);
int port_pt_render_ex(port_pt *s, const pt_camera_desc *cam, uint32_t samples, uint32_t depth, uint64_t seed,
                      float *image, uint32_t w, uint32_t h, int threads, uint64_t *rays_out, int mode, float clamp);
/* ATMOSPHERE background: table override (w x h RGBA floats); by default port_pt_commit
 * computes the 512 x 512 table with 256 samples rounded to half precision, which is the
 * reference's shipped resources/common/scattering-precomputed.exr as loaded. */
#define PORT_SKY_TABLE_RES 512u
#define PORT_SKY_TABLE_SAMPLES 256u
int port_pt_set_sky_table(port_pt *s, const float *rgba, uint32_t w, uint32_t h);
/* AtmosphereApp::precomputeTable: res x res RGBA floats; half_precision rounds every value
 * to the nearest half (as stored in the reference's EXR). */
void port_sky_table(uint32_t res, uint32_t samples, int half_precision, float *rgba);
/* Round to the nearest IEEE half (ties to even), returned as float. */
float port_round_half(float x);
/* MaterialSky::eval for n cases {origin.xyz, direction.xyz (normalised), sun.xyz} with the
 * given table; out = n x 3. */
void port_sky_eval(const float *table, uint32_t w, uint32_t h, const float *cases, size_t n, float *out);
/* MaterialGGX::eval / sampleAndEval with given uniforms (see include/rendu_gb300.h). */
void port_ggx_eval(const float *cases, size_t n, float *out);
void port_ggx_sample(const float *cases, const float *uniforms, size_t n, float *out);
void port_pixel_shifts(const pt_camera_desc *c, float *out12);

#ifdef __cplusplus
}
#endif
#endif
