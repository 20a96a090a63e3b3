/*
 * CPU restatement of Rendu's BVH raycaster -- ORACLE, test infrastructure only.
 * Declarations for oracle/port/rt_port.c. Only tests/, bench.py's CPU-baseline leg and
 * the smoke check may load this library.
 */
#ifndef RENDU_ORACLE_RT_PORT_H
#define RENDU_ORACLE_RT_PORT_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PORT_NO_HIT 0xFFFFFFFFu

/* Same 16-byte layout as the product's hit record: t, u, v, global triangle id. */
typedef struct {
    float t, u, v;
    uint32_t prim;
} port_hit;

typedef struct port_rc port_rc;

port_rc *port_rc_create(void);
void port_rc_destroy(port_rc *rc);
int port_rc_add_mesh(port_rc *rc, const float *pos, size_t nv, const uint32_t *idx, size_t ni, const float *model);
int port_rc_build(port_rc *rc);
size_t port_rc_node_count(const port_rc *rc);
size_t port_rc_tri_count(const port_rc *rc);
uint32_t port_rc_mesh_count(const port_rc *rc);
int port_default_threads(void);
/* rays: n x 8 floats {ox, oy, oz, mini, dx, dy, dz, maxi}. threads <= 0: hardware-1. */
int port_rc_intersect(const port_rc *rc, const float *rays, size_t n, port_hit *hits, int threads, uint64_t *counters);
int port_rc_intersect_any(const port_rc *rc, const float *rays, size_t n, uint8_t *any, int threads);
int port_rc_brute(const port_rc *rc, const float *rays, size_t n, port_hit *hits, int threads);
int port_rc_test_triangle(const port_rc *rc, const float *ray8, uint32_t global_tri, port_hit *out);
int port_rc_closest1(const port_rc *rc, const float *ray8, port_hit *out);
int port_rc_any1(const port_rc *rc, const float *ray8);
uint32_t port_rc_prim_mesh(const port_rc *rc, uint32_t prim);
uint32_t port_rc_mesh_first_tri(const port_rc *rc, uint32_t mesh);
int port_rc_vertices(const port_rc *rc, float *out, size_t cap_floats);

#ifdef __cplusplus
}
#endif
#endif
