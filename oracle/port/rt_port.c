/*
 * CPU restatement of Rendu's BVH raycaster -- ORACLE, test infrastructure only.
 *
 * This file restates, in plain C, the algorithm of the reference's
 *   src/engine/raycaster/Raycaster.cpp      (addMesh, updateHierarchy, intersects, intersectsAny)
 *   src/engine/raycaster/Intersection.cpp   (Ray, Intersection::box)
 *   src/engine/resources/Bounds.cpp         (BoundingBox from triangle, merge, size, centroid)
 * with the reference's own float arithmetic order (glm 0.9.9.7 operator order, no FMA
 * contraction: compile with -ffp-contract=off, never -ffast-math).
 *
 * It is used (a) as the parity checker of the CUDA raycaster in tests/, (b) as the CPU
 * baseline timed by bench.py (kind "port": the reference's own sources cannot travel to
 * the measurement host).  The product path never links or calls it.
 *
 * Parity of this restatement is pinned against the reference compiled from its own sources
 * (oracle/Makefile, target `ref`) through the golden fixtures under tests/golden/.
 */
#include "rt_port.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef struct { float x, y, z; } v3;
typedef struct { v3 lo, hi; } box3;

typedef struct {
    box3 box;
    uint64_t v0, v1, v2;
    uint64_t local_id;
    uint32_t mesh_id;
} tri_info;

typedef struct {
    box3 box;
    uint64_t left, right;
    int leaf;
} bvh_node;

struct port_rc {
    v3 *verts;
    size_t nverts, cap_verts;
    tri_info *tris;
    size_t ntris, cap_tris;
    bvh_node *nodes;
    size_t nnodes, cap_nodes;
    uint32_t mesh_count;
    uint32_t *mesh_tri_offset; /* first global triangle id of each mesh (addMesh order) */
    size_t cap_mesh;
    uint32_t *tri_global; /* per reordered triangle: global id (mesh offset + local/3) */
};

/* ---- glm-order arithmetic ------------------------------------------------------- */
/* glm::min / glm::max on scalars: (y < x) ? y : x and (x < y) ? y : x
 * (glm/detail/func_common.inl:17-29); std::min/std::max have the same operand order. */
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 v3mul(v3 a, v3 b) { v3 r = {a.x * b.x, a.y * b.y, a.z * b.z}; return r; }
static inline v3 v3min(v3 a, v3 b) { v3 r = {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; return r; }
static inline v3 v3max(v3 a, v3 b) { v3 r = {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; return r; }
/* glm::dot on vec3: tmp = a*b; tmp.x + tmp.y + tmp.z (glm/detail/func_geometric.inl:48-55). */
static inline float v3dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* glm::cross (glm/detail/func_geometric.inl:68-79). */
static inline v3 v3cross(v3 x, v3 y) {
    v3 r = {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
    return r;
}
/* glm::normalize = v * inversesqrt(dot(v,v)), inversesqrt = 1/sqrt (func_exponential.inl:136-139). */
static inline v3 v3normalize(v3 v) {
    const float s = 1.0f / sqrtf(v3dot(v, v));
    v3 r = {v.x * s, v.y * s, v.z * s};
    return r;
}

/* BoundingBox(v0,v1,v2) (Bounds.cpp:12-15). */
static inline box3 box_from_tri(v3 a, v3 b, v3 c) {
    box3 r;
    r.lo = v3min(v3min(a, b), c);
    r.hi = v3max(v3max(a, b), c);
    return r;
}
/* BoundingBox::merge (Bounds.cpp:17-20). */
static inline void box_merge(box3 *a, const box3 *b) {
    a->lo = v3min(a->lo, b->lo);
    a->hi = v3max(a->hi, b->hi);
}
/* BoundingBox::getCentroid = 0.5f * (minis + maxis) (Bounds.cpp:61-63). */
static inline float box_centroid(const box3 *b, int axis) {
    const float *lo = &b->lo.x, *hi = &b->hi.x;
    return 0.5f * (lo[axis] + hi[axis]);
}

/* Ray::Ray: dir = normalize(d), invdir = 1 / normalize(d) (Intersection.cpp:3-5). */
typedef struct { v3 pos, dir, invdir; } ray3;
static inline ray3 make_ray(v3 o, v3 d) {
    ray3 r;
    r.pos = o;
    r.dir = v3normalize(d);
    const v3 n = v3normalize(d);
    r.invdir.x = 1.0f / n.x;
    r.invdir.y = 1.0f / n.y;
    r.invdir.z = 1.0f / n.z;
    return r;
}

/* Intersection::box (Intersection.cpp:22-32). */
static inline int ray_box(const ray3 *ray, const box3 *box, float mini, float maxi) {
    const v3 minRatio = v3mul(v3sub(box->lo, ray->pos), ray->invdir);
    const v3 maxRatio = v3mul(v3sub(box->hi, ray->pos), ray->invdir);
    const v3 minFinal = v3min(minRatio, maxRatio);
    const v3 maxFinal = v3max(minRatio, maxRatio);
    const float closest = gmax(minFinal.x, gmax(minFinal.y, minFinal.z));
    const float furthest = gmin(maxFinal.x, gmin(maxFinal.y, maxFinal.z));
    return gmax(closest, mini) <= gmin(furthest, maxi);
}

/* Moller-Trumbore, Raycaster::intersects(const Ray&, const TriangleInfos&, ...)
 * (Raycaster.cpp:232-262). Returns 1 and fills t,u,v on acceptance. */
static inline int ray_tri(const ray3 *ray, v3 v0, v3 v1, v3 v2, float mini, float maxi,
                          float *t_out, float *u_out, float *v_out) {
    const v3 v01 = v3sub(v1, v0);
    const v3 v02 = v3sub(v2, v0);
    const v3 p = v3cross(ray->dir, v02);
    const float det = v3dot(v01, p);
    if (fabsf(det) < FLT_EPSILON) return 0;
    const float invDet = 1.0f / det;
    const v3 q = v3sub(ray->pos, v0);
    const float u = invDet * v3dot(q, p);
    if (u < 0.0f || u > 1.0f) return 0;
    const v3 r = v3cross(q, v01);
    const float v = invDet * v3dot(ray->dir, r);
    if (v < 0.0f || (u + v) > 1.0f) return 0;
    const float t = invDet * v3dot(v02, r);
    if (t > mini && t < maxi) {
        *t_out = t;
        *u_out = u;
        *v_out = v;
        return 1;
    }
    return 0;
}

/* ---- construction ------------------------------------------------------------------ */
static void *grow(void *p, size_t *cap, size_t need, size_t elem) {
    if (need <= *cap) return p;
    size_t nc = *cap ? *cap : 64;
    while (nc < need) nc *= 2;
    void *q = realloc(p, nc * elem);
    if (!q) return NULL;
    *cap = nc;
    return q;
}

port_rc *port_rc_create(void) { return (port_rc *)calloc(1, sizeof(port_rc)); }

void port_rc_destroy(port_rc *rc) {
    if (!rc) return;
    free(rc->verts);
    free(rc->tris);
    free(rc->nodes);
    free(rc->mesh_tri_offset);
    free(rc->tri_global);
    free(rc);
}

/* Raycaster::addMesh (Raycaster.cpp:14-52). `model` is a column-major 4x4 (glm layout) or
 * NULL for identity; the vertex transform follows glm's mat4*vec4 operator order
 * (type_mat4x4.inl:561-572): (m0*x + m1*y) + (m2*z + m3*1). */
int port_rc_add_mesh(port_rc *rc, const float *pos, size_t nv, const uint32_t *idx, size_t ni,
                     const float *model) {
    if (!rc || (nv && !pos) || (ni && !idx) || ni % 3) return -1;
    for (size_t i = 0; i < ni; ++i)
        if (idx[i] >= nv) return -1;
    const uint64_t index_offset = rc->nverts;
    void *p = grow(rc->verts, &rc->cap_verts, rc->nverts + nv, sizeof(v3));
    if (!p) return -2;
    rc->verts = (v3 *)p;
    int identity = 1;
    if (model) {
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r)
                if (model[4 * c + r] != (c == r ? 1.0f : 0.0f)) identity = 0;
    }
    for (size_t i = 0; i < nv; ++i) {
        v3 v = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        if (!identity) {
            const float *m = model;
            float o[3];
            for (int k = 0; k < 3; ++k) {
                const float a0 = m[0 + k] * v.x + m[4 + k] * v.y;
                const float a1 = m[8 + k] * v.z + m[12 + k] * 1.0f;
                o[k] = a0 + a1;
            }
            v.x = o[0];
            v.y = o[1];
            v.z = o[2];
        }
        rc->verts[rc->nverts + i] = v;
    }
    rc->nverts += nv;

    const size_t ntri = ni / 3;
    p = grow(rc->tris, &rc->cap_tris, rc->ntris + ntri, sizeof(tri_info));
    if (!p) return -2;
    rc->tris = (tri_info *)p;
    p = grow(rc->mesh_tri_offset, &rc->cap_mesh, rc->mesh_count + 1, sizeof(uint32_t));
    if (!p) return -2;
    rc->mesh_tri_offset = (uint32_t *)p;
    rc->mesh_tri_offset[rc->mesh_count] = (uint32_t)rc->ntris;
    const size_t start_tri = rc->ntris;
    for (size_t t = 0; t < ntri; ++t) {
        tri_info ti;
        ti.v0 = index_offset + idx[3 * t + 0];
        ti.v1 = index_offset + idx[3 * t + 1];
        ti.v2 = index_offset + idx[3 * t + 2];
        ti.local_id = 3 * t;
        ti.mesh_id = rc->mesh_count;
        ti.box = box_from_tri(rc->verts[ti.v0], rc->verts[ti.v1], rc->verts[ti.v2]);
        rc->tris[rc->ntris + t] = ti;
    }
    rc->ntris += ntri;
    /* One root node per mesh. */
    p = grow(rc->nodes, &rc->cap_nodes, rc->nnodes + 1, sizeof(bvh_node));
    if (!p) return -2;
    rc->nodes = (bvh_node *)p;
    bvh_node *n = &rc->nodes[rc->nnodes++];
    memset(n, 0, sizeof(*n));
    n->leaf = 1;
    n->left = start_tri;
    n->right = ntri;
    rc->mesh_count++;
    return (int)(rc->mesh_count - 1);
}

/* Quickselect on centroids along `axis`: places the k-th smallest at position k with
 * smaller-or-equal elements before it (the contract of std::nth_element used at
 * Raycaster.cpp:120-125; the order inside each side is unspecified there too). */
static void nth_element_axis(tri_info *a, size_t n, size_t k, int axis) {
    size_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const float pivot = box_centroid(&a[lo + (hi - lo) / 2].box, axis);
        size_t i = lo, lt = lo, gt = hi;
        while (i < gt) {
            const float c = box_centroid(&a[i].box, axis);
            if (c < pivot) {
                tri_info t = a[lt]; a[lt] = a[i]; a[i] = t;
                ++lt; ++i;
            } else if (pivot < c) {
                --gt;
                tri_info t = a[gt]; a[gt] = a[i]; a[i] = t;
            } else {
                ++i;
            }
        }
        if (k < lt) hi = lt;
        else if (k >= gt) lo = gt;
        else return;
    }
}

/* Raycaster::updateHierarchy (Raycaster.cpp:54-142): top-down build, explicit LIFO stack
 * seeded with one root per mesh; leaf below 3 triangles; split axis = largest box extent;
 * mean-of-centroids partition when count >= 5, median split otherwise or when degenerate. */
int port_rc_build(port_rc *rc) {
    if (!rc) return -1;
    typedef struct { uint64_t id, begin, count; } set_info;
    size_t scap = 64 + (size_t)rc->mesh_count, ssz = 0;
    set_info *stack = (set_info *)malloc(scap * sizeof(set_info));
    if (!stack) return -2;
    /* Reset any previous hierarchy: keep only the mesh roots (addMesh stored begin/count). */
    rc->nnodes = rc->mesh_count;
    for (uint32_t m = 0; m < rc->mesh_count; ++m) {
        const uint64_t begin = rc->mesh_tri_offset[m];
        const uint64_t end = (m + 1 < rc->mesh_count) ? rc->mesh_tri_offset[m + 1] : rc->ntris;
        rc->nodes[m].left = begin;
        rc->nodes[m].right = end - begin;
        set_info s = {m, begin, end - begin};
        stack[ssz++] = s;
    }
    while (ssz) {
        const set_info cur = stack[--ssz];
        const uint64_t begin = cur.begin, count = cur.count;
        box3 global;
        if (count > 0) {
            global = rc->tris[begin].box;
            for (uint64_t t = 1; t < count; ++t) box_merge(&global, &rc->tris[begin + t].box);
        } else {
            /* An empty mesh keeps a default-constructed (zero) box, as in the reference. */
            memset(&global, 0, sizeof(global));
        }
        rc->nodes[cur.id].box = global;
        if (count < 3) {
            rc->nodes[cur.id].leaf = 1;
            rc->nodes[cur.id].left = begin;
            rc->nodes[cur.id].right = count;
            continue;
        }
        rc->nodes[cur.id].leaf = 0;
        uint64_t split = 0;
        const v3 size = v3sub(global.hi, global.lo);
        const int axis = (size.x >= size.y && size.x >= size.z) ? 0 : (size.y >= size.z ? 1 : 2);
        if (count >= 5) {
            float absc = 0.0f;
            for (uint64_t t = 0; t < count; ++t) absc += box_centroid(&rc->tris[begin + t].box, axis);
            absc /= (float)count;
            /* partition: centroid < mean to the front */
            uint64_t first = begin, last = begin + count;
            while (1) {
                while (first < last && box_centroid(&rc->tris[first].box, axis) < absc) ++first;
                while (first < last && !(box_centroid(&rc->tris[last - 1].box, axis) < absc)) --last;
                if (first >= last) break;
                tri_info t = rc->tris[first];
                rc->tris[first] = rc->tris[last - 1];
                rc->tris[last - 1] = t;
                ++first;
                --last;
            }
            split = first - begin;
        }
        if (split == 0 || split == count || count < 5) {
            split = count / 2;
            nth_element_axis(rc->tris + begin, count, split, axis);
        }
        void *p = grow(rc->nodes, &rc->cap_nodes, rc->nnodes + 2, sizeof(bvh_node));
        if (!p) { free(stack); return -2; }
        rc->nodes = (bvh_node *)p;
        const uint64_t left = rc->nnodes++, right = rc->nnodes++;
        memset(&rc->nodes[left], 0, sizeof(bvh_node));
        memset(&rc->nodes[right], 0, sizeof(bvh_node));
        rc->nodes[cur.id].left = left;
        rc->nodes[cur.id].right = right;
        if (ssz + 2 > scap) {
            scap *= 2;
            set_info *q = (set_info *)realloc(stack, scap * sizeof(set_info));
            if (!q) { free(stack); return -2; }
            stack = q;
        }
        set_info sl = {left, begin, split}, sr = {right, begin + split, count - split};
        stack[ssz++] = sl;
        stack[ssz++] = sr;
    }
    free(stack);
    free(rc->tri_global);
    rc->tri_global = (uint32_t *)malloc((rc->ntris ? rc->ntris : 1) * sizeof(uint32_t));
    if (!rc->tri_global) return -2;
    for (size_t t = 0; t < rc->ntris; ++t)
        rc->tri_global[t] = rc->mesh_tri_offset[rc->tris[t].mesh_id] + (uint32_t)(rc->tris[t].local_id / 3);
    return 0;
}

size_t port_rc_node_count(const port_rc *rc) { return rc ? rc->nnodes : 0; }
size_t port_rc_tri_count(const port_rc *rc) { return rc ? rc->ntris : 0; }
uint32_t port_rc_mesh_count(const port_rc *rc) { return rc ? rc->mesh_count : 0; }

/* ---- queries ------------------------------------------------------------------------- */
static inline v3 ld3(const float *p) { v3 r = {p[0], p[1], p[2]}; return r; }

/* Raycaster::intersects(origin, direction, mini, maxi) (Raycaster.cpp:144-185), with the
 * visit counters of the traversal (inner box tests and triangle tests) added. */
static void closest_one(const port_rc *rc, const float *ray8, port_hit *out, uint64_t *nbox,
                        uint64_t *ntri, uint64_t **stack, size_t *scap) {
    const ray3 ray = make_ray(ld3(ray8), ld3(ray8 + 4));
    const float mini = ray8[3];
    float maxi = ray8[7];
    size_t ssz = 0;
    uint64_t *st = *stack;
    for (uint32_t m = 0; m < rc->mesh_count; ++m) {
        (*nbox)++;
        if (!ray_box(&ray, &rc->nodes[m].box, mini, maxi)) continue;
        st[ssz++] = m;
    }
    port_hit best;
    best.t = FLT_MAX;
    best.u = 0.0f;
    best.v = 0.0f;
    best.prim = PORT_NO_HIT;
    while (ssz) {
        const bvh_node *n = &rc->nodes[st[--ssz]];
        if (n->leaf) {
            for (uint64_t k = 0; k < n->right; ++k) {
                const tri_info *tr = &rc->tris[n->left + k];
                float t, u, v;
                (*ntri)++;
                if (ray_tri(&ray, rc->verts[tr->v0], rc->verts[tr->v1], rc->verts[tr->v2], mini, maxi, &t, &u, &v) &&
                    t < best.t) {
                    best.t = t;
                    best.u = u;
                    best.v = v;
                    best.prim = rc->tri_global[n->left + k];
                    maxi = t;
                }
            }
            continue;
        }
        if (ssz + 2 > *scap) {
            *scap *= 2;
            *stack = (uint64_t *)realloc(*stack, *scap * sizeof(uint64_t));
            st = *stack;
        }
        *nbox += 2;
        if (ray_box(&ray, &rc->nodes[n->left].box, mini, maxi)) st[ssz++] = n->left;
        if (ray_box(&ray, &rc->nodes[n->right].box, mini, maxi)) st[ssz++] = n->right;
    }
    *out = best;
}

/* Raycaster::intersectsAny (Raycaster.cpp:187-224). */
static uint8_t any_one(const port_rc *rc, const float *ray8, uint64_t **stack, size_t *scap) {
    const ray3 ray = make_ray(ld3(ray8), ld3(ray8 + 4));
    const float mini = ray8[3], maxi = ray8[7];
    size_t ssz = 0;
    uint64_t *st = *stack;
    for (uint32_t m = 0; m < rc->mesh_count; ++m)
        if (ray_box(&ray, &rc->nodes[m].box, mini, maxi)) st[ssz++] = m;
    while (ssz) {
        const bvh_node *n = &rc->nodes[st[--ssz]];
        if (n->leaf) {
            for (uint64_t k = 0; k < n->right; ++k) {
                const tri_info *tr = &rc->tris[n->left + k];
                float t, u, v;
                if (ray_tri(&ray, rc->verts[tr->v0], rc->verts[tr->v1], rc->verts[tr->v2], mini, maxi, &t, &u, &v))
                    return 1;
            }
            continue;
        }
        if (ssz + 2 > *scap) {
            *scap *= 2;
            *stack = (uint64_t *)realloc(*stack, *scap * sizeof(uint64_t));
            st = *stack;
        }
        if (ray_box(&ray, &rc->nodes[n->left].box, mini, maxi)) st[ssz++] = n->left;
        if (ray_box(&ray, &rc->nodes[n->right].box, mini, maxi)) st[ssz++] = n->right;
    }
    return 0;
}

/* Exhaustive closest hit over every triangle in addMesh order, with the same per-triangle
 * test; among equal distances the smallest global triangle id wins. Independent of any
 * hierarchy: it is the checker for hits that a hierarchy must not lose. */
static void brute_one(const port_rc *rc, const float *ray8, port_hit *out) {
    const ray3 ray = make_ray(ld3(ray8), ld3(ray8 + 4));
    const float mini = ray8[3], maxi = ray8[7];
    port_hit best;
    best.t = FLT_MAX;
    best.u = best.v = 0.0f;
    best.prim = PORT_NO_HIT;
    for (size_t k = 0; k < rc->ntris; ++k) {
        const tri_info *tr = &rc->tris[k];
        float t, u, v;
        if (!ray_tri(&ray, rc->verts[tr->v0], rc->verts[tr->v1], rc->verts[tr->v2], mini, maxi, &t, &u, &v)) continue;
        const uint32_t g = rc->tri_global[k];
        if (t < best.t || (t == best.t && g < best.prim)) {
            best.t = t;
            best.u = u;
            best.v = v;
            best.prim = g;
        }
    }
    *out = best;
}

/* ---- threading: System::forParallel (System.hpp:72-104) -------------------------------
 * hardware_concurrency()-1 workers (at least 1), contiguous spans, last span takes the rest. */
typedef struct {
    const port_rc *rc;
    const float *rays;
    size_t lo, hi;
    int mode;
    port_hit *hits;
    uint8_t *any;
    uint64_t nbox, ntri;
} work_t;

static void *worker(void *arg) {
    work_t *w = (work_t *)arg;
    size_t scap = 256;
    uint64_t *stack = (uint64_t *)malloc(scap * sizeof(uint64_t));
    if (scap < (size_t)w->rc->mesh_count + 2) {
        scap = (size_t)w->rc->mesh_count + 256;
        stack = (uint64_t *)realloc(stack, scap * sizeof(uint64_t));
    }
    for (size_t i = w->lo; i < w->hi; ++i) {
        const float *r = w->rays + 8 * i;
        if (w->mode == 0) closest_one(w->rc, r, &w->hits[i], &w->nbox, &w->ntri, &stack, &scap);
        else if (w->mode == 1) w->any[i] = any_one(w->rc, r, &stack, &scap);
        else brute_one(w->rc, r, &w->hits[i]);
    }
    free(stack);
    return NULL;
}

int port_default_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 1 ? (int)(n - 1) : 1;
}

static int run_parallel(const port_rc *rc, const float *rays, size_t n, int mode, port_hit *hits,
                        uint8_t *any, int threads, uint64_t *counters) {
    if (!rc || (n && !rays)) return -1;
    if (threads <= 0) threads = port_default_threads();
    size_t count = (size_t)threads < n ? (size_t)threads : n;
    if (count == 0) return 0;
    const size_t span = n / count > 0 ? n / count : 1;
    pthread_t *th = (pthread_t *)malloc(count * sizeof(pthread_t));
    work_t *w = (work_t *)calloc(count, sizeof(work_t));
    for (size_t k = 0; k < count; ++k) {
        w[k].rc = rc;
        w[k].rays = rays;
        w[k].lo = k * span;
        w[k].hi = (k == count - 1) ? n : (k + 1) * span;
        w[k].mode = mode;
        w[k].hits = hits;
        w[k].any = any;
        pthread_create(&th[k], NULL, worker, &w[k]);
    }
    uint64_t nb = 0, nt = 0;
    for (size_t k = 0; k < count; ++k) {
        pthread_join(th[k], NULL);
        nb += w[k].nbox;
        nt += w[k].ntri;
    }
    if (counters) {
        counters[0] = nb;
        counters[1] = nt;
    }
    free(th);
    free(w);
    return 0;
}

int port_rc_intersect(const port_rc *rc, const float *rays, size_t n, port_hit *hits, int threads,
                      uint64_t *counters) {
    return run_parallel(rc, rays, n, 0, hits, NULL, threads, counters);
}

int port_rc_intersect_any(const port_rc *rc, const float *rays, size_t n, uint8_t *any, int threads) {
    return run_parallel(rc, rays, n, 1, NULL, any, threads, NULL);
}

int port_rc_brute(const port_rc *rc, const float *rays, size_t n, port_hit *hits, int threads) {
    return run_parallel(rc, rays, n, 2, hits, NULL, threads, NULL);
}

/* Single-ray triangle test for the given global triangle, exposed so a test can check why
 * two answers differ (tie or grazing miss). */
int port_rc_test_triangle(const port_rc *rc, const float *ray8, uint32_t global_tri, port_hit *out) {
    if (!rc || !out) return -1;
    for (size_t k = 0; k < rc->ntris; ++k) {
        if (rc->tri_global[k] != global_tri) continue;
        const tri_info *tr = &rc->tris[k];
        const ray3 ray = make_ray(ld3(ray8), ld3(ray8 + 4));
        float t, u, v;
        if (ray_tri(&ray, rc->verts[tr->v0], rc->verts[tr->v1], rc->verts[tr->v2], ray8[3], ray8[7], &t, &u, &v)) {
            out->t = t;
            out->u = u;
            out->v = v;
            out->prim = global_tri;
            return 1;
        }
        out->t = FLT_MAX;
        out->u = out->v = 0.0f;
        out->prim = PORT_NO_HIT;
        return 0;
    }
    return -1;
}

/* Single-ray queries for the path-tracer restatement (oracle/port/pt_port.c); each host
 * thread keeps its own traversal stack. */
static _Thread_local uint64_t *tl_stack = NULL;
static _Thread_local size_t tl_cap = 0;

static int ensure_stack(const port_rc *rc) {
    const size_t need = (size_t)rc->mesh_count + 256;
    if (tl_cap >= need) return 0;
    uint64_t *p = (uint64_t *)realloc(tl_stack, need * sizeof(uint64_t));
    if (!p) return -1;
    tl_stack = p;
    tl_cap = need;
    return 0;
}

int port_rc_closest1(const port_rc *rc, const float *ray8, port_hit *out) {
    uint64_t nb = 0, nt = 0;
    if (ensure_stack(rc)) return -1;
    closest_one(rc, ray8, out, &nb, &nt, &tl_stack, &tl_cap);
    return out->prim != PORT_NO_HIT;
}

int port_rc_any1(const port_rc *rc, const float *ray8) {
    if (ensure_stack(rc)) return -1;
    return any_one(rc, ray8, &tl_stack, &tl_cap);
}

uint32_t port_rc_prim_mesh(const port_rc *rc, uint32_t prim) {
    uint32_t lo = 0, hi = rc->mesh_count ? rc->mesh_count - 1 : 0;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (rc->mesh_tri_offset[mid] <= prim) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

uint32_t port_rc_mesh_first_tri(const port_rc *rc, uint32_t mesh) { return rc->mesh_tri_offset[mesh]; }

/* Copy of the transformed, merged vertex soup (addMesh order), for tests. */
int port_rc_vertices(const port_rc *rc, float *out, size_t cap_floats) {
    if (!rc || cap_floats < 3 * rc->nverts) return -1;
    memcpy(out, rc->verts, rc->nverts * sizeof(v3));
    return 0;
}
