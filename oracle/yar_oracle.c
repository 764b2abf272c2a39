/*
 * yar_oracle.c - TEST INFRASTRUCTURE ONLY (see yar_oracle.h).
 *
 * Plain-C restatement of the reference renderer's ray-cast path.  Every
 * function names the reference file:line it follows.  Compiled with
 * -ffp-contract=off and IEEE division/sqrt so every float operation happens
 * in the reference's order and rounding (the reference is built by
 * MSVC /fp:precise, and by oracle/build_ref.sh with g++ -ffp-contract=off).
 */
#include "yar_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAX_TRAVERSAL_DEPTH 40 /* src/ref/kdtree.cpp:10 */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* transform_point / transform_vector, src/lib/matrix.cpp:368-389 */
static void transform_point(const float m[12], const float p[3], float out[3]) {
    for (int r = 0; r < 3; r++)
        out[r] = m[4 * r + 0] * p[0] + m[4 * r + 1] * p[1] + m[4 * r + 2] * p[2] + m[4 * r + 3];
}
static void transform_vector(const float m[12], const float v[3], float out[3]) {
    for (int r = 0; r < 3; r++)
        out[r] = m[4 * r + 0] * v[0] + m[4 * r + 1] * v[1] + m[4 * r + 2] * v[2];
}

/* Bounding_Box::intersect_by_ray_without_NaNs, src/lib/bounding_box.h:63-85 */
static int clip_ray(const float mn[3], const float mx[3], const float o[3], const float d[3],
                    float* t_min, float* t_max) {
    float t0 = 0.f, t1 = INFINITY;
    for (int i = 0; i < 3; i++) {
        if (d[i] != 0.f) {
            float inv = 1.f / d[i];
            float s0 = (mn[i] - o[i]) * inv;
            float s1 = (mx[i] - o[i]) * inv;
            if (inv < 0.f) { float tmp = s0; s0 = s1; s1 = tmp; }
            t0 = s0 > t0 ? s0 : t0;
            t1 = s1 < t1 ? s1 : t1;
            if (t0 > t1) return 0;
        } else if (o[i] < mn[i] || o[i] > mx[i]) {
            return 0;
        }
    }
    *t_min = t0;
    *t_max = t1;
    return 1;
}

/* intersect_triangle_watertight, src/ref/intersection.cpp:53-113 */
float oracle_intersect_triangle_watertight(const float o[3], const float d[3], const float p0[3],
                                           const float p1[3], const float p2[3], float b[3]) {
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    const int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2); /* Vector3::max_dimension */
    const int kx = (kz == 2 ? 0 : kz + 1);
    const int ky = (kz == 0 ? 2 : kz - 1);
    const float dx = d[kx], dy = d[ky], dz = d[kz];
    const float sx = -dx / dz;
    const float sy = -dy / dz;
    const float sz = 1.f / dz;
    const float p0t[3] = {p0[kx] - o[kx], p0[ky] - o[ky], p0[kz] - o[kz]};
    const float p1t[3] = {p1[kx] - o[kx], p1[ky] - o[ky], p1[kz] - o[kz]};
    const float p2t[3] = {p2[kx] - o[kx], p2[ky] - o[ky], p2[kz] - o[kz]};
    const float x0 = p0t[0] + sx * p0t[2];
    const float y0 = p0t[1] + sy * p0t[2];
    const float x1 = p1t[0] + sx * p1t[2];
    const float y1 = p1t[1] + sy * p1t[2];
    const float x2 = p2t[0] + sx * p2t[2];
    const float y2 = p2t[1] + sy * p2t[2];
    float e0 = x1 * y2 - y1 * x2;
    float e1 = x2 * y0 - y2 * x0;
    float e2 = x0 * y1 - y0 * x1;
    if (e0 == 0.f || e1 == 0.f || e2 == 0.f) {
        e0 = (float)((double)x1 * (double)y2 - (double)y1 * (double)x2);
        e1 = (float)((double)x2 * (double)y0 - (double)y2 * (double)x0);
        e2 = (float)((double)x0 * (double)y1 - (double)y0 * (double)x1);
    }
    if ((e0 < 0 || e1 < 0 || e2 < 0) && (e0 > 0 || e1 > 0 || e2 > 0)) return INFINITY;
    const float det = e0 + e1 + e2;
    if (det == 0.f) return INFINITY;
    const float z0 = sz * p0t[2];
    const float z1 = sz * p1t[2];
    const float z2 = sz * p2t[2];
    const float t_scaled = e0 * z0 + e1 * z1 + e2 * z2;
    if ((f2u(det) ^ f2u(t_scaled)) >> 31) return INFINITY;
    const float inv_det = 1.f / det;
    const float t = inv_det * t_scaled;
    b[0] = e0 * inv_det;
    b[1] = e1 * inv_det;
    b[2] = e2 * inv_det;
    return t;
}

static void mesh_positions(const yar_mesh_desc* m, uint32_t tri, const float** p0, const float** p1,
                           const float** p2) {
    const int32_t* i = m->indices + 3 * (size_t)tri;
    *p0 = m->vertices + 3 * (size_t)i[0];
    *p1 = m->vertices + 3 * (size_t)i[1];
    *p2 = m->vertices + 3 * (size_t)i[2];
}

/* cross(p1 - p0, p2 - p0).length_squared() == 0 (src/ref/kdtree.cpp:27-29) */
static int degenerate(const float* p0, const float* p1, const float* p2) {
    const float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const float c[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const float x = a[1] * c[2] - a[2] * c[1];
    const float y = a[2] * c[0] - a[0] * c[2];
    const float z = a[0] * c[1] - a[1] * c[0];
    return x * x + y * y + z * z == 0.f;
}

typedef struct hit_state {
    float t;
    uint32_t prim;
    uint32_t object;
    float b[3];
} hit_state;

typedef struct stack_entry {
    uint32_t node;
    float t_max;
} stack_entry;

/* One kd-tree descent step shared by all four traversals
 * (src/ref/kdtree.cpp:254-298 and :361-406).  Returns the next node. */
static inline uint32_t descend(const yar_kd_node* nodes, uint32_t node, const float o[3], const float d[3],
                               const float inv[3], float* t_min, float* t_max, stack_entry* stack, int* sp) {
    const yar_kd_node n = nodes[node];
    const int axis = (int)(n.word0 & 3u);
    const float distance_to_split_plane = u2f(n.word1) - o[axis];
    const uint32_t below_child = node + 1;
    const uint32_t above_child = n.word0 >> 2;
    if (distance_to_split_plane != 0.0) {
        uint32_t first_child, second_child;
        if (distance_to_split_plane > 0.0) {
            first_child = below_child;
            second_child = above_child;
        } else {
            first_child = above_child;
            second_child = below_child;
        }
        const float t_split = distance_to_split_plane * inv[axis];
        if (t_split > *t_max || t_split < 0.0) return first_child;
        if (t_split < *t_min) return second_child;
        stack[*sp].node = second_child;
        stack[*sp].t_max = *t_max;
        (*sp)++;
        *t_max = t_split;
        return first_child;
    }
    return (d[axis] > 0.0) ? above_child : below_child;
}

/* KdTree::intersect for a triangle-mesh tree with the leaf callback
 * intersect_triangle_mesh_geometry_data (src/ref/kdtree.cpp:12-45, :219-327). */
static int mesh_closest(const yar_mesh_desc* m, const float o[3], const float d[3], hit_state* hit,
                        oracle_ray_stats* st) {
    float t_min, t_max;
    if (!clip_ray(m->kdtree.bounds_min, m->kdtree.bounds_max, o, d, &t_min, &t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    stack_entry stack[MAX_TRAVERSAL_DEPTH + 1];
    int sp = 0;
    const yar_kd_node* nodes = m->kdtree.nodes;
    uint32_t node = 0;
    const float ray_tmax = hit->t;
    while (hit->t > t_min) {
        if (st) st->nodes++;
        if ((nodes[node].word0 & 3u) != 3u) {
            node = descend(nodes, node, o, d, inv, &t_min, &t_max, stack, &sp);
            if (sp > MAX_TRAVERSAL_DEPTH) return -1;
        } else {
            const uint32_t count = nodes[node].word0 >> 2;
            const uint32_t* idx = &nodes[node].word1;
            if (st && count > 1) st->leaf_words += count - 1;
            if (m->visibility != YAR_INVISIBLE) {
                for (uint32_t i = 0; i < count; i++) {
                    const float *p0, *p1, *p2;
                    mesh_positions(m, idx[i], &p0, &p1, &p2);
                    float b[3];
                    if (st) st->triangle_tests++;
                    const float t = oracle_intersect_triangle_watertight(o, d, p0, p1, p2, b);
                    if (t < hit->t) {
                        if (degenerate(p0, p1, p2)) continue;
                        hit->t = t;
                        hit->prim = idx[i];
                        hit->b[0] = b[0];
                        hit->b[1] = b[1];
                        hit->b[2] = b[2];
                    }
                }
            }
            if (sp == 0) break;
            --sp;
            node = stack[sp].node;
            t_min = t_max;
            t_max = stack[sp].t_max;
        }
    }
    return hit->t < ray_tmax;
}

/* KdTree::intersect_any with intersect_any_triangle_mesh_geometry_data
 * (src/ref/kdtree.cpp:47-79, :329-439). */
static int mesh_any(const yar_mesh_desc* m, const float o[3], const float d[3], float ray_tmax,
                    oracle_ray_stats* st) {
    float t_min, t_max;
    if (!clip_ray(m->kdtree.bounds_min, m->kdtree.bounds_max, o, d, &t_min, &t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    stack_entry stack[MAX_TRAVERSAL_DEPTH + 1];
    int sp = 0;
    const yar_kd_node* nodes = m->kdtree.nodes;
    uint32_t node = 0;
    while (ray_tmax > t_min) {
        if (st) st->nodes++;
        if ((nodes[node].word0 & 3u) != 3u) {
            node = descend(nodes, node, o, d, inv, &t_min, &t_max, stack, &sp);
            if (sp > MAX_TRAVERSAL_DEPTH) return -1;
        } else {
            const uint32_t count = nodes[node].word0 >> 2;
            const uint32_t* idx = &nodes[node].word1;
            if (st && count > 1) st->leaf_words += count - 1;
            if (m->visibility == YAR_VISIBLE) {
                for (uint32_t i = 0; i < count; i++) {
                    const float *p0, *p1, *p2;
                    mesh_positions(m, idx[i], &p0, &p1, &p2);
                    float b[3];
                    if (st) st->triangle_tests++;
                    const float t = oracle_intersect_triangle_watertight(o, d, p0, p1, p2, b);
                    if (t >= ray_tmax) continue;
                    if (degenerate(p0, p1, p2)) continue;
                    return 1;
                }
            }
            if (sp == 0) break;
            --sp;
            node = stack[sp].node;
            t_min = t_max;
            t_max = stack[sp].t_max;
        }
    }
    return 0;
}

/* Scene-level KdTree::intersect with intersect_scene_geometry_data
 * (src/ref/kdtree.cpp:81-95, :219-327). */
static int scene_closest(const yar_flat_scene* s, const float o[3], const float d[3], hit_state* hit,
                         oracle_ray_stats* st) {
    float t_min, t_max;
    if (!clip_ray(s->scene_kdtree.bounds_min, s->scene_kdtree.bounds_max, o, d, &t_min, &t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    stack_entry stack[MAX_TRAVERSAL_DEPTH + 1];
    int sp = 0;
    const yar_kd_node* nodes = s->scene_kdtree.nodes;
    uint32_t node = 0;
    const float ray_tmax = hit->t;
    while (hit->t > t_min) {
        if (st) st->nodes++;
        if ((nodes[node].word0 & 3u) != 3u) {
            node = descend(nodes, node, o, d, inv, &t_min, &t_max, stack, &sp);
            if (sp > MAX_TRAVERSAL_DEPTH) return -1;
        } else {
            const uint32_t count = nodes[node].word0 >> 2;
            const uint32_t* idx = &nodes[node].word1;
            if (st && count > 1) st->leaf_words += count - 1;
            for (uint32_t i = 0; i < count; i++) {
                const yar_object_desc* obj = &s->objects[idx[i]];
                float oo[3], od[3];
                transform_point(obj->world_to_object, o, oo);
                transform_vector(obj->world_to_object, d, od);
                if (st) st->object_visits++;
                int r = mesh_closest(&s->meshes[obj->mesh_index], oo, od, hit, st);
                if (r < 0) return -1;
                if (r) hit->object = idx[i];
            }
            if (sp == 0) break;
            --sp;
            node = stack[sp].node;
            t_min = t_max;
            t_max = stack[sp].t_max;
        }
    }
    return hit->t < ray_tmax;
}

static int scene_any(const yar_flat_scene* s, const float o[3], const float d[3], float ray_tmax,
                     oracle_ray_stats* st) {
    float t_min, t_max;
    if (!clip_ray(s->scene_kdtree.bounds_min, s->scene_kdtree.bounds_max, o, d, &t_min, &t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    stack_entry stack[MAX_TRAVERSAL_DEPTH + 1];
    int sp = 0;
    const yar_kd_node* nodes = s->scene_kdtree.nodes;
    uint32_t node = 0;
    while (ray_tmax > t_min) {
        if (st) st->nodes++;
        if ((nodes[node].word0 & 3u) != 3u) {
            node = descend(nodes, node, o, d, inv, &t_min, &t_max, stack, &sp);
            if (sp > MAX_TRAVERSAL_DEPTH) return -1;
        } else {
            const uint32_t count = nodes[node].word0 >> 2;
            const uint32_t* idx = &nodes[node].word1;
            if (st && count > 1) st->leaf_words += count - 1;
            for (uint32_t i = 0; i < count; i++) {
                const yar_object_desc* obj = &s->objects[idx[i]];
                float oo[3], od[3];
                transform_point(obj->world_to_object, o, oo);
                transform_vector(obj->world_to_object, d, od);
                if (st) st->object_visits++;
                int r = mesh_any(&s->meshes[obj->mesh_index], oo, od, ray_tmax, st);
                if (r != 0) return r;
            }
            if (sp == 0) break;
            --sp;
            node = stack[sp].node;
            t_min = t_max;
            t_max = stack[sp].t_max;
        }
    }
    return 0;
}

int oracle_cast_closest(const yar_flat_scene* s, const yar_ray* rays, uint32_t n, float* t, uint32_t* prim,
                        uint32_t* object, float* bary, oracle_ray_stats* stats) {
    if (!s || (!rays && n)) return YAR_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        hit_state hit;
        hit.t = rays[i].tmax;
        hit.prim = 0xffffffffu;
        hit.object = 0xffffffffu;
        hit.b[0] = hit.b[1] = hit.b[2] = 0.f;
        const int r = scene_closest(s, rays[i].origin, rays[i].direction, &hit, stats ? &stats[i] : NULL);
        if (r < 0) return YAR_ERR_CAPACITY;
        if (t) t[i] = hit.t;
        if (prim) prim[i] = r ? hit.prim : 0xffffffffu;
        if (object) object[i] = r ? hit.object : 0xffffffffu;
        if (bary) {
            bary[2 * i] = r ? hit.b[1] : 0.f;
            bary[2 * i + 1] = r ? hit.b[2] : 0.f;
        }
    }
    return YAR_OK;
}

int oracle_cast_any(const yar_flat_scene* s, const yar_ray* rays, uint32_t n, uint8_t* occluded,
                    oracle_ray_stats* stats) {
    if (!s || (!rays && n)) return YAR_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        const int r = scene_any(s, rays[i].origin, rays[i].direction, rays[i].tmax, stats ? &stats[i] : NULL);
        if (r < 0) return YAR_ERR_CAPACITY;
        occluded[i] = (uint8_t)(r ? 1 : 0);
    }
    return YAR_OK;
}

/* ---- pcg32, third-party/pcg/pcg_basic.c:46-75 and src/lib/random.h:7-74 ---- */
uint32_t oracle_pcg32_next(oracle_pcg32* rng) {
    const uint64_t oldstate = rng->state;
    rng->state = oldstate * 6364136223846793005ULL + rng->inc;
    const uint32_t xorshifted = (uint32_t)(((oldstate >> 18u) ^ oldstate) >> 27u);
    const uint32_t rot = (uint32_t)(oldstate >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((-rot) & 31));
}

void oracle_pcg32_seed(oracle_pcg32* rng, uint64_t initstate, uint64_t initseq) {
    rng->state = 0u;
    rng->inc = (initseq << 1u) | 1u;
    oracle_pcg32_next(rng);
    rng->state += initstate;
    oracle_pcg32_next(rng);
}

float oracle_pcg32_float(oracle_pcg32* rng) {
    const uint32_t i = (oracle_pcg32_next(rng) >> 9) | 0x3f800000u;
    return u2f(i) - 1.0f;
}

static uint32_t pcg32_bounded_fast(oracle_pcg32* rng, uint32_t bound) {
    /* RNG::get_bounded_uint_fast_and_biased, src/lib/random.h:58-62 */
    const uint64_t r = oracle_pcg32_next(rng);
    return (uint32_t)((r * bound) >> 32);
}

#define ONE_MINUS_EPSILON 0x1.fffffep-1f /* src/lib/math.h:14 */

/* generate_stratified_sequence_1d/2d, src/ref/sampling.cpp:79-96 */
static void stratified_1d(oracle_pcg32* rng, int n, float* out) {
    const float dx = 1.f / (float)n;
    for (int x = 0; x < n; x++) {
        float v = ((float)x + oracle_pcg32_float(rng)) * dx;
        out[x] = v < ONE_MINUS_EPSILON ? v : ONE_MINUS_EPSILON;
    }
}
static void stratified_2d(oracle_pcg32* rng, int nx, int ny, float* out) {
    const float dx = 1.f / (float)nx;
    const float dy = 1.f / (float)ny;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            float a = ((float)x + oracle_pcg32_float(rng)) * dx;
            *out++ = a < ONE_MINUS_EPSILON ? a : ONE_MINUS_EPSILON;
            float b = ((float)y + oracle_pcg32_float(rng)) * dy;
            *out++ = b < ONE_MINUS_EPSILON ? b : ONE_MINUS_EPSILON;
        }
}
/* shuffle, src/lib/math.h:138-145 (elements of `width` floats) */
static void shuffle(float* data, int n, int width, oracle_pcg32* rng) {
    for (int i = n; i > 1; i--) {
        const uint32_t k = pcg32_bounded_fast(rng, (uint32_t)i);
        for (int c = 0; c < width; c++) {
            float tmp = data[(i - 1) * width + c];
            data[(i - 1) * width + c] = data[k * width + c];
            data[k * width + c] = tmp;
        }
    }
}

void oracle_pixel_samples(uint32_t stream_id, int nx, int ny, int n1d, int n2d, float* image, float* s1d,
                          float* s2d) {
    oracle_pcg32 rng;
    oracle_pcg32_seed(&rng, 0, stream_id);
    const int spp = nx * ny;
    stratified_2d(&rng, nx, ny, image);
    float* tmp = (float*)malloc(sizeof(float) * 2 * (size_t)spp);
    for (int i = 0; i < n1d; i++) {
        stratified_1d(&rng, spp, tmp);
        shuffle(tmp, spp, 1, &rng);
        for (int k = 0; k < spp; k++) s1d[k * n1d + i] = tmp[k];
    }
    for (int i = 0; i < n2d; i++) {
        stratified_2d(&rng, nx, ny, tmp);
        shuffle(tmp, spp, 2, &rng);
        for (int k = 0; k < spp; k++) {
            s2d[2 * (k * n2d + i) + 0] = tmp[2 * k + 0];
            s2d[2 * (k * n2d + i) + 1] = tmp[2 * k + 1];
        }
    }
    free(tmp);
}

int oracle_render(const yar_flat_scene* scene, float* rgb, double* variance, int32_t row_begin, int32_t row_end,
                  int32_t thread_count) {
    (void)scene; (void)rgb; (void)variance; (void)row_begin; (void)row_end; (void)thread_count;
    return YAR_ERR_UNSUPPORTED;
}
