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

/* The alpha test of both leaf callbacks (src/ref/kdtree.cpp:31-38, :69-77):
 * Triangle_Mesh::get_uv (barycentric_interpolate, src/lib/math.h:146-153),
 * then Image_Texture::sample_bilinear of mip 0 with repeat wrapping
 * (image_texture.cpp:441-476); 1 when the red channel is 0 (skip). */
static float alpha_texel_r(const yar_flat_scene* s, const yar_texture_mip_desc* mip, int x, int y) {
    const int w = (int)mip->width, h = (int)mip->height;
    if (x >= 0) x &= w - 1;
    else { x %= w; x += (x >> 31) & w; }
    if (y >= 0) y &= h - 1;
    else { y %= h; y += (y >> 31) & h; }
    return s->texels[3 * (mip->texel_offset + (uint64_t)y * (uint64_t)w + (uint64_t)x)];
}
static int alpha_rejects(const yar_flat_scene* s, const yar_mesh_desc* m, uint32_t prim, const float b[3]) {
    if (!s || !m->alpha_texture) return 0;
    const int32_t* vi = &m->indices[3 * (size_t)prim];
    const float* uv0 = &m->uvs[2 * (size_t)vi[0]];
    const float* uv1 = &m->uvs[2 * (size_t)vi[1]];
    const float* uv2 = &m->uvs[2 * (size_t)vi[2]];
    const float u = b[0] * uv0[0] + b[1] * uv1[0] + b[2] * uv2[0];
    const float v = b[0] * uv0[1] + b[1] * uv1[1] + b[2] * uv2[1];
    const yar_texture_mip_desc* mip = &s->texture_mips[s->textures[m->alpha_texture - 1].first_mip];
    const float x = u * (float)mip->width - 0.5f, y = v * (float)mip->height - 0.5f;
    const float x_floor = floorf(x), y_floor = floorf(y);
    const float wx = x - x_floor, wy = y - y_floor;
    const int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    float r = alpha_texel_r(s, mip, x0, y0) * ((1 - wy) * (1 - wx));
    r = r + alpha_texel_r(s, mip, x1, y0) * ((1 - wy) * wx);
    r = r + alpha_texel_r(s, mip, x0, y1) * (wy * (1 - wx));
    r = r + alpha_texel_r(s, mip, x1, y1) * (wy * wx);
    return r == 0.f;
}

/* KdTree::intersect for a triangle-mesh tree with the leaf callback
 * intersect_triangle_mesh_geometry_data (src/ref/kdtree.cpp:12-45, :219-327). */
static int mesh_closest(const yar_flat_scene* s, const yar_mesh_desc* m, const float o[3], const float d[3],
                        hit_state* hit, oracle_ray_stats* st) {
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
                        if (alpha_rejects(s, m, idx[i], b)) continue;
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
static int mesh_any(const yar_flat_scene* s, const yar_mesh_desc* m, const float o[3], const float d[3],
                    float ray_tmax, oracle_ray_stats* st) {
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
                    if (alpha_rejects(s, m, idx[i], b)) continue;
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
                int r = mesh_closest(s, &s->meshes[obj->mesh_index], oo, od, hit, st);
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
                int r = mesh_any(s, &s->meshes[obj->mesh_index], oo, od, ray_tmax, st);
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


/* ======================================================================
 * Render path: camera, shading context, BSDFs, MIS direct lighting from
 * rectangular lights, the path loop and the film, restated from
 * src/ref/{camera,shading_context,bsdf,scattering,sampling,direct_lighting,
 * path_tracing,reference_renderer,film}.cpp and src/lib/math.cpp.
 * ==================================================================== */
#include <pthread.h>

typedef struct v3 { float x, y, z; } v3;
typedef struct col { float r, g, b; } col;

static inline v3 mk3(float x, float y, float z) { v3 v = {x, y, z}; return v; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3s(v3 v, float t) { return mk3(v.x * t, v.y * t, v.z * t); }   /* Vector3 * float */
static inline v3 div3s(v3 v, float t) { return mk3(v.x / t, v.y / t, v.z / t); }   /* Vector3 / float */
static inline v3 neg3(v3 v) { return mk3(-v.x, -v.y, -v.z); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float len2_3(v3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
static inline float len3(v3 v) { return sqrtf(len2_3(v)); }
static inline v3 norm3(v3 v) { return div3s(v, len3(v)); }
static inline float get3(v3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline v3 ld3(const float* p) { return mk3(p[0], p[1], p[2]); }

static inline col mkc(float r, float g, float b) { col c = {r, g, b}; return c; }
static inline col addc(col a, col b) { return mkc(a.r + b.r, a.g + b.g, a.b + b.b); }
static inline col mulc(col a, col b) { return mkc(a.r * b.r, a.g * b.g, a.b * b.b); }
static inline col mulcs(col c, float k) { return mkc(c.r * k, c.g * k, c.b * k); }   /* ColorRGB * float */
static inline col divc(col a, col b) { return mkc(a.r / b.r, a.g / b.g, a.b / b.b); }
static inline col subc(col a, col b) { return mkc(a.r - b.r, a.g - b.g, a.b - b.b); }
static inline col sqrtc(col c) { return mkc(sqrtf(c.r), sqrtf(c.g), sqrtf(c.b)); }
static inline int blackc(col c) { return c.r == 0 && c.g == 0 && c.b == 0; }
static inline float fmaxf_std(float a, float b) { return (a < b) ? b : a; }       /* std::max */
static inline float fminf_std(float a, float b) { return (b < a) ? b : a; }       /* std::min */
static inline float maxcomp(col c) { return fmaxf_std(c.r, fmaxf_std(c.g, c.b)); }
static inline col ldc(const float* p) { return mkc(p[0], p[1], p[2]); }

#define PI_F 3.14159265f              /* src/lib/math.h:7 */
static const float PI_INV_F = 1.f / PI_F;

static v3 xform_point(const float m[12], v3 p) {
    float in[3] = {p.x, p.y, p.z}, out[3];
    transform_point(m, in, out);
    return mk3(out[0], out[1], out[2]);
}
static v3 xform_vector(const float m[12], v3 v) {
    float in[3] = {v.x, v.y, v.z}, out[3];
    transform_vector(m, in, out);
    return mk3(out[0], out[1], out[2]);
}

/* barycentric_interpolate, src/lib/math.h:146-153 */
static v3 bary3(const v3 p[3], const float b[3]) {
    return add3(add3(mul3s(p[0], b[0]), mul3s(p[1], b[1])), mul3s(p[2], b[2]));
}

/* coordinate_system_from_vector, src/lib/math.cpp:21-25 */
static void coordinate_system(v3 v, v3* v1, v3* v2) {
    *v1 = (fabsf(v.x) > fabsf(v.y)) ? mk3(-v.z, 0, v.x) : mk3(0, -v.z, v.y);
    *v1 = div3s(*v1, len3(*v1));
    *v2 = cross3(v, *v1);
}

/* project_vector_onto_plane_and_get_direction, src/lib/math.cpp:33-39 */
static v3 project_direction(v3 v, v3 n) {
    v3 t = cross3(v, n);
    v3 d = cross3(n, t);
    return norm3(d);
}

/* reflect / refract, src/lib/math.h:108-125 */
static v3 reflect3(v3 w, v3 n) { return sub3(mul3s(n, 2.f * dot3(w, n)), w); }
static int refract3(v3 wi, v3 n, float eta, v3* wt) {
    float cos_i = dot3(wi, n);
    float sin_t2 = eta * eta * fmaxf_std(0.f, 1.f - cos_i * cos_i);
    if (sin_t2 >= 1.f) return 0;
    float cos_t = sqrtf(1.f - sin_t2);
    *wt = add3(mul3s(wi, -eta), mul3s(n, eta * cos_i - cos_t));
    return 1;
}

static inline int f2i(float f) { int i; memcpy(&i, &f, 4); return i; }
static inline float i2f(int i) { float f; memcpy(&f, &i, 4); return f; }

/* offset_ray_origin_in_both_directions, src/lib/math.cpp:81-120 */
static void offset_origins(v3 p, v3 n, v3* pos, v3* neg) {
    const float int_scale = 256.f, origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f;
    const float pc[3] = {p.x, p.y, p.z}, nc[3] = {n.x, n.y, n.z};
    float po[3], ne[3];
    for (int k = 0; k < 3; k++) {
        int di = (int)(int_scale * nc[k]);
        int i1 = f2i(pc[k]) - di, i2 = f2i(pc[k]) + di;
        po[k] = i2f(pc[k] < 0 ? i1 : i2);
        ne[k] = i2f(pc[k] < 0 ? i2 : i1);
        if (fabsf(pc[k]) < origin) {
            float d = float_scale * nc[k];
            po[k] = pc[k] + d;
            ne[k] = pc[k] - d;
        }
    }
    *pos = mk3(po[0], po[1], po[2]);
    *neg = mk3(ne[0], ne[1], ne[2]);
}

typedef struct shading_ctx {
    v3 wo, position, geometric_normal, normal, dpdu_shading;
    v3 origin_pos, origin_neg;
    int flipped;
    uint32_t material_type;
    int material_index;
    uint32_t light_type;
    int light_index;
    /* uv parameterization and its screen-space derivatives (zero without differential rays) */
    int has_uv;
    float uv[2];
    v3 dpdu, dpdv;              /* world space */
    float dudx, dvdx, dudy, dvdy;
    /* for bump mapping: the normal's uv derivatives (world space, flipped
     * with the normal) and the shading frame's second tangent */
    v3 dndu, dndv, dpdv_shading;
    /* has_dxdy_derivatives and the position and direction derivatives along
     * the differential rays (the specular differential rays start from them) */
    int has_dxdy;
    v3 dpdx, dpdy, dwo_dx, dwo_dy;
} shading_ctx;

/* adjust_shading_normal, src/ref/shading_context.cpp:17-63 */
static void adjust_shading_normal(v3 wo, v3 ng, v3* n) {
    v3 R = reflect3(wo, *n);
    float a = dot3(R, ng);
    if (a >= 0.f) return;
    const float cos_threshold = 0.0017453f;
    if (dot3(wo, ng) < cos_threshold) { *n = ng; return; }
    float b = dot3(*n, ng);
    v3 tangent;
    if (b > 1e-4f) {
        float dist = fabsf(a) / b;
        tangent = add3(R, mul3s(*n, dist));
        tangent = div3s(tangent, len3(tangent));
    } else {
        tangent = *n;
    }
    tangent = add3(tangent, mul3s(ng, 1e-4f));
    *n = norm3(add3(wo, tangent));
}

/* Shading_Context::initialize_local_geometry + init_from_triangle_mesh_intersection
 * (src/ref/shading_context.cpp:65-172, :188-240) for constant-parameter
 * materials (no bump, no differentials). */
static void init_shading(const yar_flat_scene* s, v3 ray_d, uint32_t object_index, uint32_t tri, const float b[3],
                         shading_ctx* sc) {
    const yar_object_desc* obj = &s->objects[object_index];
    const yar_mesh_desc* m = &s->meshes[obj->mesh_index];
    memset(sc, 0, sizeof(*sc));
    sc->wo = neg3(norm3(ray_d));
    const int32_t* vi = m->indices + 3 * (size_t)tri;
    v3 p[3] = {ld3(m->vertices + 3 * (size_t)vi[0]), ld3(m->vertices + 3 * (size_t)vi[1]),
               ld3(m->vertices + 3 * (size_t)vi[2])};
    v3 position = bary3(p, b);
    v3 gn = norm3(cross3(sub3(p[1], p[0]), sub3(p[2], p[0])));
    if (m->reverse_geometric_normal_orientation) gn = neg3(gn);
    v3 normal = gn;
    if (m->normals) {
        v3 n[3] = {ld3(m->normals + 3 * (size_t)vi[0]), ld3(m->normals + 3 * (size_t)vi[1]),
                   ld3(m->normals + 3 * (size_t)vi[2])};
        v3 in = bary3(n, b);
        if (len2_3(in) != 0) normal = norm3(in);
    }
    int has_uv = 0;
    v3 dpdu = mk3(0, 0, 0), dpdv = mk3(0, 0, 0), dndu = mk3(0, 0, 0), dndv = mk3(0, 0, 0);
    if (m->uvs) {
        has_uv = 1;
        const float* u0 = m->uvs + 2 * (size_t)vi[0];
        const float* u1 = m->uvs + 2 * (size_t)vi[1];
        const float* u2 = m->uvs + 2 * (size_t)vi[2];
        /* barycentric_interpolate (src/lib/math.h:146-153) of the vertex uvs */
        sc->uv[0] = u0[0] * b[0] + u1[0] * b[1] + u2[0] * b[2];
        sc->uv[1] = u0[1] * b[0] + u1[1] * b[1] + u2[1] * b[2];
        float a00 = u1[0] - u0[0], a01 = u1[1] - u0[1], a10 = u2[0] - u0[0], a11 = u2[1] - u0[1];
        v3 bp0 = sub3(p[1], p[0]), bp1 = sub3(p[2], p[0]);
        /* solve_linear_system_2x2 (src/lib/math.cpp:8-16) */
        float det = a00 * a11 - a01 * a10;
        if (det != 0.f) {
            float inv_det = 1.f / det;
            dpdu = mul3s(sub3(mul3s(bp0, a11), mul3s(bp1, a01)), inv_det);
            dpdv = mul3s(add3(mul3s(bp0, -a10), mul3s(bp1, a00)), inv_det);
        }
        if (fabsf(det) < 1e-9f) coordinate_system(gn, &dpdu, &dpdv);
        /* the normals' derivatives (zero vertex normals without them) */
        v3 n[3] = {mk3(0, 0, 0), mk3(0, 0, 0), mk3(0, 0, 0)};
        if (m->normals)
            for (int k = 0; k < 3; k++) n[k] = ld3(m->normals + 3 * (size_t)vi[k]);
        v3 bn0 = sub3(n[1], n[0]), bn1 = sub3(n[2], n[0]);
        if (det != 0.f) {
            float inv_det = 1.f / det;
            dndu = mul3s(sub3(mul3s(bn0, a11), mul3s(bn1, a01)), inv_det);
            dndv = mul3s(add3(mul3s(bn0, -a10), mul3s(bn1, a00)), inv_det);
        }
        if (fabsf(det) < 1e-9f) {  /* pbrt's approximation */
            v3 dn = cross3(bn1, bn0);
            if (len2_3(dn) == 0.f) {
                dndu = mk3(0, 0, 0);
                dndv = mk3(0, 0, 0);
            } else {
                coordinate_system(dn, &dndu, &dndv);
            }
        }
    }
    /* to world space */
    position = xform_point(obj->object_to_world, position);
    normal = xform_vector(obj->object_to_world_normal, normal);
    const float length_of_scaled_normal = len3(normal);
    normal = div3s(normal, length_of_scaled_normal);
    gn = xform_vector(obj->object_to_world_normal, gn);
    gn = div3s(gn, len3(gn));
    dpdu = xform_vector(obj->object_to_world, dpdu);
    dpdv = xform_vector(obj->object_to_world, dpdv);
    {
        const float inv_length = 1 / length_of_scaled_normal;
        dndu = mul3s(xform_vector(obj->object_to_world_normal, dndu), inv_length);
        dndv = mul3s(xform_vector(obj->object_to_world_normal, dndv), inv_length);
    }
    sc->has_uv = has_uv;
    sc->dpdu = dpdu;
    sc->dpdv = dpdv;
    if (dot3(normal, gn) == 0.f) gn = normal;
    if (dot3(gn, sc->wo) < 0) gn = neg3(gn);
    if (dot3(normal, gn) < 0) {
        normal = neg3(normal);
        dndu = neg3(dndu);
        dndv = neg3(dndv);
        sc->flipped = 1;
    }
    offset_origins(position, gn, &sc->origin_pos, &sc->origin_neg);
    adjust_shading_normal(sc->wo, gn, &normal);
    v3 dpdu_shading, dpdv_shading;
    if (!has_uv) {
        coordinate_system(normal, &dpdu_shading, &dpdv_shading);
    } else if (fabsf(dot3(normal, gn) - 1.f) < 1e-6f) {
        dpdu_shading = dpdu;
        dpdv_shading = dpdv;
    } else {
        dpdu_shading = mul3s(project_direction(dpdu, normal), len3(dpdu));
        dpdv_shading = mul3s(project_direction(dpdv, normal), len3(dpdv));
    }
    sc->dndu = dndu;
    sc->dndv = dndv;
    sc->dpdv_shading = dpdv_shading;
    sc->position = position;
    sc->geometric_normal = gn;
    sc->normal = normal;
    sc->dpdu_shading = dpdu_shading;
    sc->material_type = obj->material_type;
    sc->material_index = obj->material_index;
    sc->light_type = obj->area_light_type;
    sc->light_index = obj->area_light_index;
}

/* get_ray_origin_using_control_direction / _point, src/ref/shading_context.cpp:405-417 */
static v3 origin_for_direction(const shading_ctx* sc, v3 dir) {
    return dot3(dir, sc->geometric_normal) > 0.f ? sc->origin_pos : sc->origin_neg;
}
static v3 origin_for_point(const shading_ctx* sc, v3 point) {
    return origin_for_direction(sc, sub3(point, sc->position));
}

/* ---------------- BSDFs (src/ref/bsdf.cpp, src/ref/scattering.cpp, src/ref/sampling.cpp) */
typedef struct bsdf_t {
    uint32_t type;
    v3 n, t, bt;  /* normal, tangent, bitangent */
    int reflection, transmission;
    col reflectance, transmittance; /* plastic, coated diffuse: diffuse reflectance and r0 */
    float alpha_x, alpha_y, alpha;  /* metal, coated diffuse: alpha_x/y; glass, plastic: alpha */
    float eta_i_metal;
    col eta_t, k_t;
    float eta_o, eta_i;             /* glass */
    int pbrt3_plastic, flipped;     /* plastic: Pbrt3_Plastic_BRDF, original shading normal flipped */
    col diffuse_coeff, specular_coeff; /* pbrt3 translucent: Kd, Ks */
    const struct bsdf_t* sub[2];    /* mix: the two BSDFs; scaled: sub[0] */
    col mix_coeff;                  /* mix: White - amount */
    float p_coeff, scale;           /* mix: 1 - luminance(mix_coeff); scaled: the factor */
    /* pbrt3 fourier: zenith cosines, coefficients, (offset, length) per node pair */
    const float *fourier_nodes, *fourier_coeffs;
    const uint32_t* fourier_series;
    uint32_t fourier_node_count, fourier_channels;
} bsdf_t;

#define ORACLE_BSDF_SCALED 0x100u   /* Scaled_BSDF: a mix whose other material is pure delta */

/* ColorRGB::luminance, src/lib/color.h:74-76 with sRGB_to_XYZ (src/lib/color.cpp:18-24) */
static float luminance(col c) { return 0.2126729f * c.r + 0.7151522f * c.g + 0.0721750f * c.b; }
static int is_pure_delta(uint32_t type) { /* !material_has_bsdf, src/lib/material.h:27-30 */
    return type == YAR_MATERIAL_PERFECT_REFLECTOR || type == YAR_MATERIAL_PERFECT_REFRACTOR;
}

static col clamp_unit(col c) { /* ColorRGB::clamp_to_unit_range, src/lib/color.h:83-88 */
    c.r = c.r < 0.f ? 0.f : (1.f < c.r ? 1.f : c.r);
    c.g = c.g < 0.f ? 0.f : (1.f < c.g ? 1.f : c.g);
    c.b = c.b < 0.f ? 0.f : (1.f < c.b ? 1.f : c.b);
    return c;
}

static float pbrt3_roughness_to_alpha(float roughness) {
    /* src/ref/scattering.cpp:240-251 */
    roughness = fmaxf_std(roughness, 1e-3f);
    float x = logf(roughness);
    return 1.621420000f + 0.819955000f * x + 0.173400000f * x * x + 0.017120100f * x * x * x +
           0.000640711f * x * x * x * x;
}
static float roughness_to_alpha(const yar_flat_scene* s, float r, int no_remap) {
    if (no_remap) return r;
    if (s->config.pbrt3_scene) return pbrt3_roughness_to_alpha(r);
    return r * r;
}

static v3 local_to_world(const bsdf_t* f, v3 l) {
    return mk3(f->t.x * l.x + f->bt.x * l.y + f->n.x * l.z, f->t.y * l.x + f->bt.y * l.y + f->n.y * l.z,
               f->t.z * l.x + f->bt.z * l.y + f->n.z * l.z);
}
static v3 world_to_local(const bsdf_t* f, v3 w) { return mk3(dot3(w, f->t), dot3(w, f->bt), dot3(w, f->n)); }

static col texture_reflectance(const yar_flat_scene* s, const shading_ctx* sc, const yar_material_desc* m);
static col texture_transmittance(const yar_flat_scene* s, const shading_ctx* sc, const yar_material_desc* m);

static int make_leaf_bsdf(const yar_flat_scene* s, const shading_ctx* sc, uint32_t type, const yar_material_desc* m,
                          bsdf_t* f) {
    memset(f, 0, sizeof(*f));
    f->n = sc->normal;
    f->bt = norm3(cross3(sc->normal, sc->dpdu_shading));
    f->t = cross3(f->bt, sc->normal);
    f->type = type;
    if (f->type == YAR_MATERIAL_DIFFUSE) {
        f->reflection = 1;
        f->reflectance = m->reflectance_texture ? texture_reflectance(s, sc, m) : ldc(m->reflectance);
    } else if (f->type == YAR_MATERIAL_METAL) {
        f->reflection = 1;
        f->alpha_x = roughness_to_alpha(s, m->u_roughness, m->roughness_is_alpha);
        f->alpha_y = roughness_to_alpha(s, m->v_roughness, m->roughness_is_alpha);
        f->eta_i_metal = m->eta_i;
        f->eta_t = ldc(m->eta);
        f->k_t = ldc(m->k);
    } else if (f->type == YAR_MATERIAL_GLASS) {
        f->reflection = f->transmission = 1;
        f->reflectance = m->reflectance_texture ? texture_reflectance(s, sc, m) : ldc(m->reflectance);
        f->transmittance = m->transmittance_texture ? texture_transmittance(s, sc, m) : ldc(m->transmittance);
        f->alpha = roughness_to_alpha(s, m->u_roughness, m->roughness_is_alpha);
        int enter = !sc->flipped;
        f->eta_o = enter ? 1.f : m->index_of_refraction;
        f->eta_i = enter ? m->index_of_refraction : 1.f;
    } else if (f->type == YAR_MATERIAL_PLASTIC || f->type == YAR_MATERIAL_COATED_DIFFUSE) {
        /* Plastic_BRDF / Pbrt3_Plastic_BRDF / Ashikhmin_Shirley_Phong_BRDF constructors,
         * src/ref/bsdf.cpp:205-213, :427-438, src/ref/bsdf_pbrt.cpp:258-262 */
        f->reflection = 1;
        f->reflectance = m->reflectance_texture ? texture_reflectance(s, sc, m) : ldc(m->reflectance);
        f->transmittance = ldc(m->transmittance);
        f->alpha_x = roughness_to_alpha(s, m->u_roughness, m->roughness_is_alpha);
        f->alpha_y = roughness_to_alpha(s, m->v_roughness, m->roughness_is_alpha);
        f->alpha = f->alpha_x;
        f->pbrt3_plastic = f->type == YAR_MATERIAL_PLASTIC && s->config.pbrt3_scene;
        f->flipped = sc->flipped;
    } else if (f->type == YAR_MATERIAL_PBRT3_UBER) {
        /* Pbrt3_Uber_BRDF, src/ref/bsdf_pbrt.cpp:14-32: Kd, Ks, opacity; roughness always remapped */
        f->reflection = 1;
        f->reflectance = ldc(m->reflectance);
        f->specular_coeff = ldc(m->specular);
        f->diffuse_coeff = ldc(m->opacity);
        f->alpha_x = roughness_to_alpha(s, m->u_roughness, 0);
        f->alpha_y = roughness_to_alpha(s, m->v_roughness, 0);
        f->eta_i = !sc->flipped ? m->index_of_refraction : 1.f / m->index_of_refraction;
    } else if (f->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) {
        /* Diffuse_Transmission_BSDF, src/ref/bsdf.cpp:89-103 */
        f->reflection = f->transmission = 1;
        const col r = m->reflectance_texture ? texture_reflectance(s, sc, m) : ldc(m->reflectance);
        const col t = m->transmittance_texture ? texture_transmittance(s, sc, m) : ldc(m->transmittance);
        f->reflectance = clamp_unit(mulc(ldc(m->diffuse), r));
        f->transmittance = clamp_unit(mulc(ldc(m->diffuse), t));
    } else if (f->type == YAR_MATERIAL_PBRT3_TRANSLUCENT) {
        /* Pbrt3_Translucent_BSDF, src/ref/bsdf_pbrt.cpp:94-115 */
        f->reflectance = ldc(m->reflectance);
        f->transmittance = ldc(m->transmittance);
        f->diffuse_coeff = ldc(m->diffuse);
        f->specular_coeff = ldc(m->specular);
        f->alpha = roughness_to_alpha(s, m->u_roughness, 0);
        int enter = !sc->flipped;
        f->eta_o = enter ? 1.f : 1.5f;
        f->eta_i = enter ? 1.5f : 1.f;
        f->reflection = !blackc(f->reflectance);
        f->transmission = !blackc(f->transmittance);
    } else if (f->type == YAR_MATERIAL_PBRT3_FOURIER) {
        /* Pbrt3_Fourier_BSDF, src/ref/bsdf_pbrt.cpp:297-303: reflection only */
        const yar_fourier_desc* t = &s->fourier_tables[m->fourier_table - 1];
        f->reflection = 1;
        f->fourier_nodes = s->fourier_floats + t->nodes;
        f->fourier_coeffs = s->fourier_floats + t->coeffs;
        f->fourier_series = s->fourier_uints + t->series;
        f->fourier_node_count = t->node_count;
        f->fourier_channels = t->channel_count;
    } else {
        return YAR_ERR_UNSUPPORTED;
    }
    return YAR_OK;
}

/* create_bsdf (src/ref/bsdf.cpp:631-714) with create_mix_bsdf (:599-629): a mix of
 * two BSDF materials is a Mix_BSDF, a mix with a pure delta material the Scaled_BSDF
 * of the other one.  sub holds the mix's leaf BSDFs. */
static int make_bsdf(const yar_flat_scene* s, const shading_ctx* sc, bsdf_t* f, bsdf_t sub[2]) {
    const yar_material_desc* m = &s->materials[sc->material_index];
    if (sc->material_type != YAR_MATERIAL_MIX) return make_leaf_bsdf(s, sc, sc->material_type, m, f);
    const yar_material_desc* m1 = &s->materials[m->mix_materials[0]];
    const yar_material_desc* m2 = &s->materials[m->mix_materials[1]];
    const int has1 = !is_pure_delta(m1->type), has2 = !is_pure_delta(m2->type);
    if (!has1 && !has2) return YAR_ERR_UNSUPPORTED;
    const float amount = luminance(ldc(m->mix_amount));
    int rc = make_leaf_bsdf(s, sc, YAR_MATERIAL_DIFFUSE, m, f); /* the frame */
    if (rc != YAR_OK) return rc;
    f->sub[0] = &sub[0];
    if (!has1 || !has2) {
        rc = make_leaf_bsdf(s, sc, has1 ? m1->type : m2->type, has1 ? m1 : m2, &sub[0]);
        f->type = ORACLE_BSDF_SCALED;
        f->scale = has1 ? amount : 1.f - amount;
        f->reflection = sub[0].reflection;
        f->transmission = sub[0].transmission;
        return rc;
    }
    rc = make_leaf_bsdf(s, sc, m1->type, m1, &sub[0]);
    if (rc == YAR_OK) rc = make_leaf_bsdf(s, sc, m2->type, m2, &sub[1]);
    f->sub[1] = &sub[1];
    f->type = YAR_MATERIAL_MIX;
    f->mix_coeff = subc(mkc(1, 1, 1), ldc(m->mix_amount));
    f->p_coeff = 1.f - luminance(f->mix_coeff);
    f->reflection = sub[0].reflection || sub[1].reflection;
    f->transmission = sub[0].transmission || sub[1].transmission;
    return rc;
}

/* The sine and cosine of sampled angles.  The reference calls the C library's
 * sinf/cosf (std::sin/std::cos on floats), which is what this oracle does by
 * default.  oracle_render_trig can switch to the correctly rounded values
 * (double evaluation rounded to float), which is what the CUDA path computes:
 * with it, the two must agree bit for bit.  Set per render, not reentrant. */
static int g_correctly_rounded_trig = 0;
static float sin_sample(float x) { return g_correctly_rounded_trig ? (float)sin((double)x) : sinf(x); }
static float cos_sample(float x) { return g_correctly_rounded_trig ? (float)cos((double)x) : cosf(x); }
static float atan2_sample(float y, float x) {
    return g_correctly_rounded_trig ? (float)atan2((double)y, (double)x) : atan2f(y, x);
}
static float acos_sample(float x) { return g_correctly_rounded_trig ? (float)acos((double)x) : acosf(x); }
/* log2 of the EWA footprint: the C library's log2f, or correctly rounded like the device */
/* The film filters (src/ref/film.cpp:123-142) at offset (x, y) from the pixel
 * center: box 1; gaussian max(0, exp(-alpha |p|^2) - exp(-alpha r^2)), the
 * zero level from expf as the reference's constructor computes it; triangle
 * max(0, r - |x|) max(0, r - |y|). */
static float film_filter_weight(const yar_render_config* c, float x, float y) {
    if (c->pixel_filter_type == 1) {
        const float zero_level = expf(-c->pixel_filter_alpha * c->pixel_filter_radius * c->pixel_filter_radius);
        const float a = -c->pixel_filter_alpha * (x * x + y * y);
        const float e = g_correctly_rounded_trig ? (float)exp((double)a) : expf(a);
        const float v = e - zero_level;
        return 0.f < v ? v : 0.f;
    }
    if (c->pixel_filter_type == 2) {
        const float ax = c->pixel_filter_radius - fabsf(x), ay = c->pixel_filter_radius - fabsf(y);
        return (0.f < ax ? ax : 0.f) * (0.f < ay ? ay : 0.f);
    }
    return 1.f;
}
static float log2_lod(float x) { return g_correctly_rounded_trig ? (float)log2((double)x) : log2f(x); }

/* ---------------- image textures (src/ref/image_texture.cpp, src/ref/parameter_evaluation.cpp:10-31) */

/* do_EWA's filter weights (src/ref/image_texture.cpp:503-512), exp(-2 x) over
 * 256 steps, with the C library's expf [0] or correctly rounded [1] */
static float g_ewa_weights[2][256];
static void init_ewa_weights(void) {
    for (int i = 0; i < 256; i++) {
        const float x = (float)i / (float)(256 - 1);
        g_ewa_weights[0][i] = expf(-2.f * x);
        g_ewa_weights[1][i] = (float)exp((double)(-2.f * x));
    }
}

/* get_texel_repeat (image_texture.cpp:386-410): power-of-two mips */
static col texel_repeat(const yar_flat_scene* s, const yar_texture_mip_desc* mip, int x, int y) {
    const int w = (int)mip->width, h = (int)mip->height;
    if (x >= 0) x &= w - 1;
    else { x %= w; x += (x >> 31) & w; }
    if (y >= 0) y &= h - 1;
    else { y %= h; y += (y >> 31) & h; }
    const float* t = s->texels + 3 * (mip->texel_offset + (uint64_t)y * (uint64_t)w + (uint64_t)x);
    return mkc(t[0], t[1], t[2]);
}

/* Image_Texture::sample_bilinear with Wrap_Mode::repeat (image_texture.cpp:436-477) */
static col texture_bilinear(const yar_flat_scene* s, const yar_texture_mip_desc* mip, float u, float v) {
    const float x = u * (float)mip->width - 0.5f, y = v * (float)mip->height - 0.5f;
    const float x_floor = floorf(x), y_floor = floorf(y);
    const float wx = x - x_floor, wy = y - y_floor;
    const int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    col c = mulcs(texel_repeat(s, mip, x0, y0), (1 - wy) * (1 - wx));
    c = addc(c, mulcs(texel_repeat(s, mip, x1, y0), (1 - wy) * wx));
    c = addc(c, mulcs(texel_repeat(s, mip, x0, y1), wy * (1 - wx)));
    return addc(c, mulcs(texel_repeat(s, mip, x1, y1), wy * wx));
}

/* do_EWA (image_texture.cpp:501-578): the elliptical Gaussian footprint on one mip */
static col texture_ewa_level(const yar_flat_scene* s, const yar_texture_mip_desc* mip, float u, float v,
                             const float a1[2], const float a2[2]) {
    const float* weights = g_ewa_weights[g_correctly_rounded_trig ? 1 : 0];
    const float w = (float)mip->width, h = (float)mip->height;
    u = u * w - 0.5f;
    v = v * h - 0.5f;
    const float a1x = a1[0] * w, a1y = a1[1] * h, a2x = a2[0] * w, a2y = a2[1] * h;
    float A = a1y * a1y + a2y * a2y + 1;
    float B = -2 * (a1x * a1y + a2x * a2y);
    float C = a1x * a1x + a2x * a2x + 1;
    const float F = A * C - 0.25f * B * B;
    const float inv_F = 1.f / F;
    A *= inv_F;
    B *= inv_F;
    C *= inv_F;
    const float inv_det = 0.25f * F;
    const float u_delta = 2 * sqrtf(C * inv_det);
    const float x0 = ceilf(u - u_delta), x1 = floorf(u + u_delta);
    const float v_delta = 2 * sqrtf(A * inv_det);
    const float y0 = ceilf(v - v_delta), y1 = floorf(v + v_delta);
    col sum = mkc(0, 0, 0);
    float weight_sum = 0.f;
    for (float y = y0; y <= y1; y++) {
        const float yy = y - v;
        for (float x = x0; x <= x1; x++) {
            const float xx = x - u;
            const float r2 = A * xx * xx + B * xx * yy + C * yy * yy;
            if (r2 < 1.f) {
                const float wt = weights[(int)(r2 * 256)];
                sum = addc(sum, mulcs(texel_repeat(s, mip, (int)x, (int)y), wt));
                weight_sum += wt;
            }
        }
    }
    return mulcs(sum, 1.f / weight_sum);
}

/* Image_Texture::sample_EWA (image_texture.cpp:580-615), max anisotropy 32 */
static col texture_ewa(const yar_flat_scene* s, const yar_texture_desc* t, float u, float v, float a1[2], float a2[2]) {
    const yar_texture_mip_desc* mips = s->texture_mips + t->first_mip;
    float l1 = a1[0] * a1[0] + a1[1] * a1[1], l2 = a2[0] * a2[0] + a2[1] * a2[1];
    if (l1 < l2) {
        float tmp[2] = {a1[0], a1[1]};
        a1[0] = a2[0]; a1[1] = a2[1];
        a2[0] = tmp[0]; a2[1] = tmp[1];
        const float tl = l1; l1 = l2; l2 = tl;
    }
    const float major_length = sqrtf(l1);
    float minor_length = sqrtf(l2);
    if (minor_length < 1e-6f) return texture_bilinear(s, &mips[0], u, v);
    if (minor_length * 32.f < major_length) {
        const float scale = major_length / (minor_length * 32.f);
        minor_length *= scale;
        a2[0] *= scale;
        a2[1] *= scale;
    }
    const float lod = fmaxf_std(0.f, (float)((int)t->mip_count - 1) + log2_lod(minor_length));
    float lod_floor;
    const float frac = modff(lod, &lod_floor);
    const int level0 = (int)lod_floor;
    if (level0 >= (int)t->mip_count - 1) {
        const float* c = s->texels + 3 * mips[t->mip_count - 1].texel_offset;
        return mkc(c[0], c[1], c[2]);
    }
    const col c0 = texture_ewa_level(s, &mips[level0], u, v, a1, a2);
    const col c1 = texture_ewa_level(s, &mips[level0 + 1], u, v, a1, a2);
    return addc(mulcs(c0, 1.f - frac), mulcs(c1, frac));  /* lerp, src/lib/math.h:82-85 */
}

/* evaluate_texture_parameter (parameter_evaluation.cpp:10-31): uv and its
 * derivatives scaled, then EWA with repeat wrapping */
static col texture_parameter(const yar_flat_scene* s, uint32_t texture, const float uv_scale[2], float u, float v,
                             const shading_ctx* sc) {
    const yar_texture_desc* t = &s->textures[texture - 1];
    const float su = uv_scale[0], sv = uv_scale[1];
    float a1[2] = {sc->dudx * su, sc->dvdx * sv}, a2[2] = {sc->dudy * su, sc->dvdy * sv};
    return texture_ewa(s, t, u * su, v * sv, a1, a2);
}
static col texture_reflectance(const yar_flat_scene* s, const shading_ctx* sc, const yar_material_desc* m) {
    return texture_parameter(s, m->reflectance_texture, m->reflectance_uv_scale, sc->uv[0], sc->uv[1], sc);
}
static col texture_transmittance(const yar_flat_scene* s, const shading_ctx* sc, const yar_material_desc* m) {
    return texture_parameter(s, m->transmittance_texture, m->transmittance_uv_scale, sc->uv[0], sc->uv[1], sc);
}

/* evaluate_float_parameter of a bump map at (u, v): the constant, or the
 * luminance of the texture (parameter_evaluation.cpp:46-55) */
static float bump_height_at(const yar_flat_scene* s, const yar_material_desc* m, float u, float v,
                            const shading_ctx* sc) {
    if (m->bump == 1) return m->bump_height;
    return luminance(texture_parameter(s, m->bump_texture, m->bump_uv_scale, u, v, sc));
}

/* Shading_Context::apply_bump_map (src/ref/shading_context.cpp:419-462): the
 * height and its finite differences along u and v perturb the shading
 * tangents; the shading normal is rebuilt from them, turned into the
 * geometric normal's hemisphere and adjusted. */
static void apply_bump_map(const yar_flat_scene* s, const yar_material_desc* m, shading_ctx* sc) {
    if (!m->bump) return;
    const float height = bump_height_at(s, m, sc->uv[0], sc->uv[1], sc);
    float du = 0.5f * (fabsf(sc->dudx) + fabsf(sc->dudy));
    if (du == 0.f) du = 0.0005f;
    const float height_du = bump_height_at(s, m, sc->uv[0] + du, sc->uv[1] + 0.f, sc);
    float dv = 0.5f * (fabsf(sc->dvdx) + fabsf(sc->dvdy));
    if (dv == 0.f) dv = 0.0005f;
    const float height_dv = bump_height_at(s, m, sc->uv[0] + 0.f, sc->uv[1] + dv, sc);
    const v3 original_shading_normal = sc->flipped ? neg3(sc->normal) : sc->normal;
    float du_scale = 1.f, dv_scale = 1.f;
    if (m->bump == 2) {
        du_scale = m->bump_uv_scale[0];
        dv_scale = m->bump_uv_scale[1];
    }
    const v3 dpdu_shading = add3(add3(sc->dpdu_shading, mul3s(original_shading_normal, (height_du - height) / (du * du_scale))),
                                 mul3s(mul3s(sc->dndu, du_scale), height));
    const v3 dpdv_shading = add3(add3(sc->dpdv_shading, mul3s(original_shading_normal, (height_dv - height) / (dv * dv_scale))),
                                 mul3s(mul3s(sc->dndv, dv_scale), height));
    v3 normal = norm3(cross3(dpdu_shading, dpdv_shading));
    if (dot3(normal, sc->geometric_normal) < 0) normal = neg3(normal);
    adjust_shading_normal(sc->wo, sc->geometric_normal, &normal);
    sc->normal = normal;
    sc->dpdu_shading = dpdu_shading;
    sc->dpdv_shading = dpdv_shading;
}

/* ray_plane_intersection, src/lib/math.cpp:27-31 */
static float ray_plane_t(v3 o, v3 d, v3 n, float plane_d) {
    const float k = -dot3(o, n) - plane_d;
    if (k == 0) return 0.f;
    return k / dot3(d, n);
}

/* Shading_Context::calculate_dxdy_derivatives + calculate_uv_derivates
 * (src/ref/shading_context.cpp:242-333) for the differential rays (ox, dx_dir)
 * and (oy, dy_dir) */
static void uv_derivatives(shading_ctx* sc, v3 ox, v3 dx_dir, v3 oy, v3 dy_dir) {
    if (!sc->has_uv) return;
    sc->has_dxdy = 1;
    const v3 gn = sc->geometric_normal;
    const float plane_d = -dot3(gn, sc->position);
    v3 dpdx = mk3(0, 0, 0), dpdy = mk3(0, 0, 0);
    const float tx = ray_plane_t(ox, dx_dir, gn, plane_d);
    if (fabsf(tx) != INFINITY) dpdx = sub3(add3(ox, mul3s(dx_dir, tx)), sc->position);
    const float ty = ray_plane_t(oy, dy_dir, gn, plane_d);
    if (fabsf(ty) != INFINITY) dpdy = sub3(add3(oy, mul3s(dy_dir, ty)), sc->position);
    sc->dpdx = dpdx;
    sc->dpdy = dpdy;
    sc->dwo_dx = sub3(neg3(dx_dir), sc->wo);
    sc->dwo_dy = sub3(neg3(dy_dir), sc->wo);
    int dim0, dim1;
    {
        const float ax = fabsf(gn.x), ay = fabsf(gn.y), az = fabsf(gn.z);
        if (ax > ay && ax > az) { dim0 = 1; dim1 = 2; }
        else if (ay > az) { dim0 = 0; dim1 = 2; }
        else { dim0 = 0; dim1 = 1; }
    }
    const float pu[3] = {sc->dpdu.x, sc->dpdu.y, sc->dpdu.z}, pv[3] = {sc->dpdv.x, sc->dpdv.y, sc->dpdv.z};
    const float px[3] = {dpdx.x, dpdx.y, dpdx.z}, py[3] = {dpdy.x, dpdy.y, dpdy.z};
    const float a00 = pu[dim0], a01 = pv[dim0], a10 = pu[dim1], a11 = pv[dim1];
    const float det = a00 * a11 - a01 * a10;  /* solve_linear_system_2x2, src/lib/math.cpp:8-16 */
    sc->dudx = sc->dvdx = sc->dudy = sc->dvdy = 0.f;
    if (det != 0.f) {
        const float inv_det = 1.f / det;
        sc->dudx = (a11 * px[dim0] - a01 * px[dim1]) * inv_det;
        sc->dvdx = (-a10 * px[dim0] + a00 * px[dim1]) * inv_det;
        sc->dudy = (a11 * py[dim0] - a01 * py[dim1]) * inv_det;
        sc->dvdy = (-a10 * py[dim0] + a00 * py[dim1]) * inv_det;
    }
    if (fabsf(sc->dudx) > 1e9f || fabsf(sc->dvdx) > 1e9f || fabsf(sc->dudy) > 1e9f || fabsf(sc->dvdy) > 1e9f) {
        sc->has_dxdy = 0;
        sc->dpdx = sc->dpdy = sc->dwo_dx = sc->dwo_dy = mk3(0, 0, 0);
        sc->dudx = sc->dvdx = sc->dudy = sc->dvdy = 0.f;
    }
}

/* Raytracer_Config::max_differential_ray_specular_bounces (src/lib/raytracer_config.h:33);
 * no scene format sets it */
#define MAX_DIFFERENTIAL_RAY_SPECULAR_BOUNCES 4

/* Shading_Context::compute_differential_rays_for_specular_reflection (eta 0)
 * and _for_specular_transmission (eta = etaI / etaT), src/ref/shading_context.cpp:357-403:
 * the differential rays of the delta ray from the hit position in direction
 * dir; ray[0], ray[1] the dx ray's origin and direction, ray[2], ray[3] the dy ray's. */
static void specular_differentials(const shading_ctx* sc, v3 dir, float eta, v3 ray[4]) {
    const v3 n = sc->normal, wo = sc->wo;
    const v3 dndx = add3(mul3s(sc->dndu, sc->dudx), mul3s(sc->dndv, sc->dvdx));
    const v3 dndy = add3(mul3s(sc->dndu, sc->dudy), mul3s(sc->dndv, sc->dvdy));
    const float d_wo_dot_n_dx = dot3(sc->dwo_dx, n) + dot3(wo, dndx);
    const float d_wo_dot_n_dy = dot3(sc->dwo_dy, n) + dot3(wo, dndy);
    v3 dwi_dx, dwi_dy;
    if (eta == 0.f) {
        const float dot_wo_n = dot3(wo, n);
        dwi_dx = sub3(mul3s(add3(mul3s(n, d_wo_dot_n_dx), mul3s(dndx, dot_wo_n)), 2.f), sc->dwo_dx);
        dwi_dy = sub3(mul3s(add3(mul3s(n, d_wo_dot_n_dy), mul3s(dndy, dot_wo_n)), 2.f), sc->dwo_dy);
    } else {
        const float cos_o = dot3(wo, n);
        const float cos_t = -dot3(dir, n);
        const float k1 = eta * eta * cos_o / cos_t;
        const float k2 = eta * cos_o - cos_t;
        const float d_cos_t_dx = k1 * d_wo_dot_n_dx, d_cos_t_dy = k1 * d_wo_dot_n_dy;
        dwi_dx = add3(add3(mul3s(sc->dwo_dx, -eta), mul3s(dndx, k2)), mul3s(n, eta * d_wo_dot_n_dx - d_cos_t_dx));
        dwi_dy = add3(add3(mul3s(sc->dwo_dy, -eta), mul3s(dndy, k2)), mul3s(n, eta * d_wo_dot_n_dy - d_cos_t_dy));
    }
    ray[0] = add3(sc->position, sc->dpdx);
    ray[1] = norm3(add3(dir, dwi_dx));
    ray[2] = add3(sc->position, sc->dpdy);
    ray[3] = norm3(add3(dir, dwi_dy));
}

static v3 sample_hemisphere_cosine(float u0, float u1) {
    float z = sqrtf(1.f - u0);
    float r = sqrtf(u0);
    float phi = 2.f * PI_F * u1;
    return mk3(r * cos_sample(phi), r * sin_sample(phi), z);
}

static float dielectric_fresnel(float cos_i, float eta) {
    cos_i = fminf_std(fabsf(cos_i), 1.f);
    float sin_i = sqrtf(1.f - cos_i * cos_i);
    float sin_t = (1.f / eta) * sin_i;
    if (sin_t >= 1.f) return 1.f;
    float cos_t = sqrtf(1.f - sin_t * sin_t);
    float Rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    float Rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (Rp * Rp + Rs * Rs);
}

/* schlick_fresnel, src/ref/scattering.cpp:10-15 */
static col schlick_fresnel(col r0, float cos_i) {
    float k = 1.f - fabsf(cos_i);
    float k5 = (k * k) * (k * k) * k;
    return addc(r0, mulcs(subc(mkc(1, 1, 1), r0), k5));
}

static col conductor_fresnel(float cos_i, float eta_i, col eta_t, col k_t) {
    cos_i = fabsf(cos_i < -1.f ? -1.f : (cos_i > 1.f ? 1.f : cos_i));
    float c2 = cos_i * cos_i;
    float s2 = 1.f - c2;
    col eta = mulcs(eta_t, 1.f / eta_i);           /* ColorRGB / float = c * (1/k) */
    col k = mulcs(k_t, 1.f / eta_i);
    col eta2 = mulc(eta, eta);
    col k2 = mulc(k, k);
    col t0 = subc(subc(eta2, k2), mkc(s2, s2, s2));
    col a2b2 = sqrtc(addc(mulc(t0, t0), mulc(mulcs(eta2, 4.f), k2)));
    col t1 = addc(a2b2, mkc(c2, c2, c2));
    col a = sqrtc(mulcs(addc(a2b2, t0), 0.5f));
    col t2 = mulcs(a, 2.f * cos_i);
    col Rs = divc(subc(t1, t2), addc(t1, t2));
    col t3 = addc(mulcs(a2b2, c2), mkc(s2 * s2, s2 * s2, s2 * s2));
    col t4 = mulcs(t2, s2);
    col Rp = divc(mulc(Rs, subc(t3, t4)), addc(t3, t4));
    return mulcs(addc(Rp, Rs), 0.5f);
}

static float ggx_D(v3 wh, v3 n, float alpha) {
    float c = dot3(wh, n);
    if (c <= 0.f) return 0.f;
    float c2 = c * c;
    float a2 = alpha * alpha;
    float k = c2 * (a2 - 1) + 1;
    return a2 / (PI_F * k * k);
}
static float clamp1(float x) { return x < -1.f ? -1.f : (x > 1.f ? 1.f : x); }
static float ggx_D_aniso(v3 wh, float ax, float ay) {
    float c = clamp1(wh.z);
    float c2 = c * c;
    float s2 = 1.f - c2;
    float s2inv = 1.f / s2;
    float cos2_phi = (s2 == 0.f) ? 1.f : (wh.x * wh.x) * s2inv;
    float sin2_phi = (s2 == 0.f) ? 0.f : (wh.y * wh.y) * s2inv;
    float k = c2 + s2 * (cos2_phi / (ax * ax) + sin2_phi / (ay * ay));
    return 1.f / (PI_F * ax * ay * k * k);
}
static float ggx_lambda(v3 v, v3 n, float alpha) {
    float c = dot3(v, n);
    float c2 = c * c;
    float tan2 = fmaxf_std(0.f, (1.f - c2) / c2);
    return 0.5f * (-1.f + sqrtf(1.f + alpha * alpha * tan2));
}
static float ggx_lambda_aniso(v3 v, float ax, float ay) {
    float c = clamp1(v.z);
    float c2 = c * c;
    float s2 = 1.f - c2;
    float tan2 = s2 / c2;
    float s2inv = 1.f / s2;
    float cos2_phi = (s2 == 0.f) ? 1.f : (v.x * v.x) * s2inv;
    float sin2_phi = (s2 == 0.f) ? 0.f : (v.y * v.y) * s2inv;
    float alpha2 = cos2_phi * ax * ax + sin2_phi * ay * ay;
    return 0.5f * (-1.f + sqrtf(1.f + alpha2 * tan2));
}
static float ggx_G(v3 wi, v3 wo, v3 n, float a) { return 1.f / (1.f + ggx_lambda(wi, n, a) + ggx_lambda(wo, n, a)); }
static float ggx_G1(v3 v, v3 n, float a) { return 1.f / (1.f + ggx_lambda(v, n, a)); }
static float ggx_G_aniso(v3 wi, v3 wo, float ax, float ay) {
    return 1.f / (1.f + ggx_lambda_aniso(wi, ax, ay) + ggx_lambda_aniso(wo, ax, ay));
}
static float ggx_G1_aniso(v3 v, float ax, float ay) { return 1.f / (1.f + ggx_lambda_aniso(v, ax, ay)); }

/* GGX_sample_visible_microfacet_normal, src/ref/sampling.cpp:310-335 */
static v3 ggx_sample_vndf(float u0, float u1, v3 wo, float ax, float ay) {
    v3 N = norm3(mk3(ax * wo.x, ay * wo.y, wo.z));
    float len_sq = N.x * N.x + N.y * N.y;
    v3 T1 = len_sq > 0.f ? div3s(mk3(-N.y, N.x, 0), sqrtf(len_sq)) : mk3(1, 0, 0);
    v3 T2 = cross3(N, T1);
    float r = sqrtf(u0);
    float phi = 2.f * PI_F * u1;
    float t1 = r * cos_sample(phi);
    float t2 = r * sin_sample(phi);
    float s = 0.5f * (1.f + N.z);
    t2 = (1.f - s) * sqrtf(1.f - t1 * t1) + s * t2;
    v3 nh = add3(add3(mul3s(T1, t1), mul3s(T2, t2)), mul3s(N, sqrtf(fmaxf_std(0.f, 1.f - t1 * t1 - t2 * t2))));
    return norm3(mk3(ax * nh.x, ay * nh.y, fmaxf_std(1e-6f, nh.z)));
}
static float vndf_pdf(v3 wo, v3 wh, v3 n, float alpha) {
    float G1 = ggx_G1(wo, n, alpha);
    float D = ggx_D(wh, n, alpha);
    return G1 * D * fmaxf_std(0.f, dot3(wo, wh)) / dot3(wo, n);
}
static float vndf_pdf_aniso(v3 wo, v3 wh, float ax, float ay) {
    float G1 = ggx_G1_aniso(wo, ax, ay);
    float D = ggx_D_aniso(wh, ax, ay);
    return G1 * D * fmaxf_std(0.f, dot3(wo, wh)) / wo.z;
}
static float refl_pdf(v3 wo, v3 wh, v3 n, float a) { return vndf_pdf(wo, wh, n, a) / (4 * dot3(wh, wo)); }
static float refl_pdf_aniso(v3 wo, v3 wh, float ax, float ay) {
    return vndf_pdf_aniso(wo, wh, ax, ay) / (4 * dot3(wh, wo));
}
static float trans_pdf(v3 wo, v3 wi, v3 wh, v3 n, float a, float eta_o, float eta_i) {
    float wh_pdf = vndf_pdf(wo, wh, n, a);
    float denom = eta_o * dot3(wo, wh) + eta_i * dot3(wi, wh);
    float dwh = eta_i * eta_i * fabsf(dot3(wi, wh)) / (denom * denom);
    return wh_pdf * dwh;
}
static v3 refraction_half(float eta_o, v3 wo, float eta_i, v3 wi, v3 n) {
    v3 wh = neg3(norm3(add3(mul3s(wo, eta_o), mul3s(wi, eta_i))));
    if (dot3(wh, n) < 0.f) wh = neg3(wh);
    return wh;
}

static float pow5(float v) { return (v * v) * (v * v) * v; }

/* cos_delta_phi (src/lib/math.h:87-104): the cosine of the azimuth between a
 * and b in the tangent plane (1 for a direction along the normal). */
static float cos_delta_phi(v3 a, v3 b, v3 t1, v3 t2) {
    const float ax = dot3(a, t1), ay = dot3(a, t2), bx = dot3(b, t1), by = dot3(b, t2);
    const float a_len_sq = ax * ax + ay * ay, b_len_sq = bx * bx + by * by;
    if (a_len_sq == 0.f || b_len_sq == 0.f) return 1.f;
    const float cosine = (ax * bx + ay * by) / sqrtf(a_len_sq * b_len_sq);
    return cosine < -1.f ? -1.f : (1.f < cosine ? 1.f : cosine);
}

/* The first zenith node not below c (std::lower_bound over increasing nodes). */
static uint32_t fourier_node(const bsdf_t* f, float c) {
    uint32_t lo = 0, n = f->fourier_node_count;
    while (n > 0) {
        const uint32_t half = n / 2;
        if (f->fourier_nodes[lo + half] < c) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

/* Pbrt3_Fourier_BSDF::evaluate (src/ref/bsdf_pbrt.cpp:305-358): the nearest
 * node pair's Fourier series in the azimuth (no interpolation), divided by
 * |cos_i|; three channels store Y, R, B. */
static col fourier_evaluate(const bsdf_t* f, v3 wo, v3 wi) {
    const v3 nwi = neg3(wi);
    float cos_i = dot3(f->n, nwi);
    cos_i = cos_i < -1.f ? -1.f : (1.f < cos_i ? 1.f : cos_i);
    float cos_o = dot3(f->n, wo);
    cos_o = cos_o < -1.f ? -1.f : (1.f < cos_o ? 1.f : cos_o);
    const uint32_t index = fourier_node(f, cos_o) * f->fourier_node_count + fourier_node(f, cos_i);
    const uint32_t offset = f->fourier_series[2 * index], count = f->fourier_series[2 * index + 1];
    const float* coeffs = f->fourier_coeffs + offset;
    const float cos_phi = cos_delta_phi(wo, nwi, f->t, f->bt);
    const float phi = acos_sample(cos_phi);
    const float scale = cos_i != 0.f ? 1.f / fabsf(cos_i) : 0.f;
    if (f->fourier_channels == 1) {
        float y = 0.f;
        for (uint32_t i = 0; i < count; i++) y += coeffs[i] * cos_sample((float)i * phi);
        const float v = y * scale;
        return mkc(v, v, v);
    }
    float y = 0.f, r = 0.f, b = 0.f;
    for (uint32_t i = 0; i < count; i++) {
        const float c = cos_sample((float)i * phi);
        y += coeffs[i + 0 * count] * c;
        r += coeffs[i + 1 * count] * c;
        b += coeffs[i + 2 * count] * c;
    }
    const float g = 1.398304f * y - 0.297381f * r - 0.100923f * b; /* get_green_from_YRB, src/lib/color.cpp:26-29 */
    return mkc(r * scale, g * scale, b * scale);
}

static col leaf_evaluate(const bsdf_t* f, v3 wo, v3 wi) {
    if (f->type == YAR_MATERIAL_DIFFUSE) return mulcs(f->reflectance, PI_INV_F);
    if (f->type == YAR_MATERIAL_PBRT3_FOURIER) return fourier_evaluate(f, wo, wi);
    if (f->type == YAR_MATERIAL_PBRT3_UBER) { /* src/ref/bsdf_pbrt.cpp:34-52; diffuse_coeff holds the opacity */
        col diffuse = mulc(mulcs(f->reflectance, PI_INV_F), f->diffuse_coeff);
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        v3 wh_l = norm3(add3(wo_l, wi_l));
        float F = dielectric_fresnel(dot3(wi_l, wh_l), f->eta_i);
        float G = ggx_G_aniso(wi_l, wo_l, f->alpha_x, f->alpha_y);
        float D = ggx_D_aniso(wh_l, f->alpha_x, f->alpha_y);
        float mf = (F * G * D) / (4.f * wo_l.z * wi_l.z);
        return addc(diffuse, mulcs(mulc(f->specular_coeff, f->diffuse_coeff), mf));
    }
    if (f->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) { /* src/ref/bsdf.cpp:105-112 */
        int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
        return mulcs(same ? f->reflectance : f->transmittance, PI_INV_F);
    }
    if (f->type == YAR_MATERIAL_PBRT3_TRANSLUCENT) { /* src/ref/bsdf_pbrt.cpp:117-158 */
        int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
        if (same) {
            col diffuse = mulc(mulcs(f->diffuse_coeff, PI_INV_F), f->reflectance);
            v3 wh = norm3(add3(wo, wi));
            float F = dielectric_fresnel(dot3(wi, wh), f->eta_i / f->eta_o);
            float G = ggx_G(wi, wo, f->n, f->alpha);
            float D = ggx_D(wh, f->n, f->alpha);
            float base = (F * G * D) / (4.f * dot3(wo, f->n) * dot3(wi, f->n));
            return addc(diffuse, mulcs(mulc(f->specular_coeff, f->reflectance), base));
        }
        col diffuse = mulc(mulcs(f->diffuse_coeff, PI_INV_F), f->transmittance);
        col specular = mkc(0, 0, 0);
        v3 wh = refraction_half(f->eta_o, wo, f->eta_i, wi, f->n);
        float wo_wh = dot3(wo, wh), wi_wh = dot3(wi, wh);
        if (wo_wh * wi_wh <= 0.f) {
            float F = dielectric_fresnel(wi_wh, f->eta_o / f->eta_i);
            if (F < 1.f) {
                float G = ggx_G(wi, wo, f->n, f->alpha);
                float D = ggx_D(wh, f->n, f->alpha);
                float wo_n = dot3(wo, f->n), wi_n = dot3(wi, f->n);
                float k = fabsf((wo_wh * wi_wh) / (wo_n * wi_n));
                float k2 = f->eta_o * wo_wh + f->eta_i * wi_wh;
                float base = (f->eta_o * f->eta_o * k * G * D * (1.f - F)) / (k2 * k2);
                specular = mulcs(mulc(f->specular_coeff, f->transmittance), base);
            }
        }
        return addc(diffuse, specular);
    }
    if (f->type == YAR_MATERIAL_PLASTIC) {
        /* Plastic_BRDF::evaluate, src/ref/bsdf.cpp:215-234; Pbrt3_Plastic_BRDF::evaluate,
         * src/ref/bsdf_pbrt.cpp:264-290 (pbrt3's swapped 1.0/1.5 IOR pair) */
        v3 wh = norm3(add3(wo, wi));
        float cos_i = dot3(wi, wh);
        col F;
        if (f->pbrt3_plastic) {
            v3 original_n = f->flipped ? neg3(f->n) : f->n;
            float relative_ior = dot3(original_n, wi) < 0.f ? 1.5f / 1.f : 1.f / 1.5f;
            float fr = dielectric_fresnel(cos_i, relative_ior);
            F = mkc(fr, fr, fr);
        } else {
            F = schlick_fresnel(mkc(0.04f, 0.04f, 0.04f), cos_i);
        }
        float G = ggx_G(wi, wo, f->n, f->alpha);
        float D = ggx_D(wh, f->n, f->alpha);
        float wo_n = dot3(wo, f->n), wi_n = dot3(wi, f->n);
        col base = mulcs(F, (G * D) / (4.f * wo_n * wi_n));
        col specular = mulcs(base, f->transmittance.r);
        return addc(mulcs(f->reflectance, PI_INV_F), specular);
    }
    if (f->type == YAR_MATERIAL_COATED_DIFFUSE) {
        /* Ashikhmin_Shirley_Phong_BRDF::evaluate, src/ref/bsdf.cpp:440-460 */
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        v3 wh_l = norm3(add3(wo_l, wi_l));
        float cos_i = dot3(wi_l, wh_l);
        col F = schlick_fresnel(f->transmittance, cos_i);
        float D = ggx_D_aniso(wh_l, f->alpha_x, f->alpha_y);
        col specular = mulcs(F, D / (4.f * cos_i * fmaxf_std(wo_l.z, wi_l.z)));
        col diffuse = mulcs(mulc(f->reflectance, subc(mkc(1, 1, 1), f->transmittance)),
                            28.f / (23.f * PI_F) * (1.f - pow5(1.f - 0.5f * wi_l.z)) *
                                (1.f - pow5(1.f - 0.5f * wo_l.z)));
        return addc(diffuse, specular);
    }
    if (f->type == YAR_MATERIAL_METAL) {
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        v3 wh_l = norm3(add3(wo_l, wi_l));
        float cos_i = dot3(wi_l, wh_l);
        col F = conductor_fresnel(cos_i, f->eta_i_metal, f->eta_t, f->k_t);
        float G = ggx_G_aniso(wi_l, wo_l, f->alpha_x, f->alpha_y);
        float D = ggx_D_aniso(wh_l, f->alpha_x, f->alpha_y);
        return mulcs(F, (G * D) / (4.f * wo_l.z * wi_l.z));
    }
    /* rough glass */
    int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
    if (same) {
        v3 wh = norm3(add3(wo, wi));
        float cos_i = dot3(wi, wh);
        float F = dielectric_fresnel(cos_i, f->eta_i / f->eta_o);
        float G = ggx_G(wi, wo, f->n, f->alpha);
        float D = ggx_D(wh, f->n, f->alpha);
        float base = (F * G * D) / (4.f * dot3(wo, f->n) * dot3(wi, f->n));
        return mulcs(f->reflectance, base);
    }
    v3 wh = refraction_half(f->eta_o, wo, f->eta_i, wi, f->n);
    float wo_wh = dot3(wo, wh), wi_wh = dot3(wi, wh);
    if (wo_wh * wi_wh > 0.f) return mkc(0, 0, 0);
    float cos_i = dot3(wi, wh);
    float F = dielectric_fresnel(cos_i, f->eta_o / f->eta_i);
    if (F == 1.f) return mkc(0, 0, 0);
    float G = ggx_G(wi, wo, f->n, f->alpha);
    float D = ggx_D(wh, f->n, f->alpha);
    float wo_n = dot3(wo, f->n), wi_n = dot3(wi, f->n);
    float k = fabsf((wo_wh * wi_wh) / (wo_n * wi_n));
    float k2 = f->eta_o * wo_wh + f->eta_i * wi_wh;
    float base = (f->eta_o * f->eta_o * k * G * D * (1.f - F)) / (k2 * k2);
    return mulcs(f->transmittance, base);
}

static float glass_reflection_probability(const bsdf_t* f, float fresnel) {
    float max_r = maxcomp(f->reflectance), max_t = maxcomp(f->transmittance);
    float ratio = max_r / (max_r + max_t);
    float r = fresnel * ratio;
    float t = (1.f - fresnel) * (1 - ratio);
    return ((r + t) == 0) ? 0.f : r / (r + t);
}

static float leaf_pdf(const bsdf_t* f, v3 wo, v3 wi) {
    /* Pbrt3_Fourier_BSDF::pdf (src/ref/bsdf_pbrt.cpp:368-372): cosine-weighted */
    if (f->type == YAR_MATERIAL_DIFFUSE || f->type == YAR_MATERIAL_PBRT3_FOURIER) return dot3(f->n, wi) / PI_F;
    if (f->type == YAR_MATERIAL_PBRT3_UBER) { /* src/ref/bsdf_pbrt.cpp:74-87 */
        float diffuse_pdf = dot3(f->n, wi) / PI_F;
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        float spec_pdf = refl_pdf_aniso(wo_l, norm3(add3(wo_l, wi_l)), f->alpha_x, f->alpha_y);
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (f->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) { /* src/ref/bsdf.cpp:128-141 */
        float max_r = maxcomp(f->reflectance), max_t = maxcomp(f->transmittance);
        float pdf = fabsf(dot3(f->n, wi)) * PI_INV_F;
        int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
        return same ? (max_r / (max_r + max_t)) * pdf : (max_t / (max_r + max_t)) * pdf;
    }
    if (f->type == YAR_MATERIAL_PBRT3_TRANSLUCENT) { /* src/ref/bsdf_pbrt.cpp:211-250 */
        float max_r = maxcomp(f->reflectance), max_t = maxcomp(f->transmittance);
        float rp = max_r / (max_r + max_t);
        int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
        if (same) {
            float diffuse_pdf = dot3(wi, f->n) * PI_INV_F;
            float spec_pdf = refl_pdf(wo, norm3(add3(wo, wi)), f->n, f->alpha);
            return rp * 0.5f * (diffuse_pdf + spec_pdf);
        }
        float diffuse_pdf = -dot3(wi, f->n) * PI_INV_F;
        float spec_pdf = 0.f;
        v3 wh = refraction_half(f->eta_o, wo, f->eta_i, wi, f->n);
        if (dot3(wo, wh) * dot3(wi, wh) <= 0.f) spec_pdf = trans_pdf(wo, wi, wh, f->n, f->alpha, f->eta_o, f->eta_i);
        return (1.f - rp) * 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (f->type == YAR_MATERIAL_PLASTIC) {
        /* Plastic_BRDF::pdf, src/ref/bsdf.cpp:253-263 */
        float diffuse_pdf = dot3(f->n, wi) / PI_F;
        float spec_pdf = refl_pdf(wo, norm3(add3(wo, wi)), f->n, f->alpha);
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (f->type == YAR_MATERIAL_COATED_DIFFUSE) {
        /* Ashikhmin_Shirley_Phong_BRDF::pdf, src/ref/bsdf.cpp:480-492 */
        float diffuse_pdf = dot3(f->n, wi) / PI_F;
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        float spec_pdf = refl_pdf_aniso(wo_l, norm3(add3(wo_l, wi_l)), f->alpha_x, f->alpha_y);
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (f->type == YAR_MATERIAL_METAL) {
        v3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        v3 wh_l = norm3(add3(wo_l, wi_l));
        return refl_pdf_aniso(wo_l, wh_l, f->alpha_x, f->alpha_y);
    }
    int same = dot3(wo, f->n) * dot3(wi, f->n) > 0.f;
    if (same) {
        v3 wh = norm3(add3(wo, wi));
        float rp = refl_pdf(wo, wh, f->n, f->alpha);
        float cos_i = dot3(wi, wh);
        float fr = dielectric_fresnel(cos_i, f->eta_i / f->eta_o);
        return rp * glass_reflection_probability(f, fr);
    }
    v3 wh = refraction_half(f->eta_o, wo, f->eta_i, wi, f->n);
    float wo_wh = dot3(wo, wh), wi_wh = dot3(wi, wh);
    if (wo_wh * wi_wh > 0.f) return 0.f;
    float cos_t = dot3(wo, wh);
    float fr = dielectric_fresnel(cos_t, f->eta_i / f->eta_o);
    float rprob = glass_reflection_probability(f, fr);
    return trans_pdf(wo, wi, wh, f->n, f->alpha, f->eta_o, f->eta_i) * (1.f - rprob);
}

/* BSDF::sample; returns black when no direction is produced. */
static col leaf_sample(const bsdf_t* f, float u0, float u1, float u_scatter, v3 wo, v3* wi, float* pdf) {
    if (f->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) { /* src/ref/bsdf.cpp:114-126 */
        float max_r = maxcomp(f->reflectance), max_t = maxcomp(f->transmittance);
        float sign = u_scatter < max_r / (max_r + max_t) ? 1.f : -1.f;
        *wi = local_to_world(f, mul3s(sample_hemisphere_cosine(u0, u1), sign));
        *pdf = leaf_pdf(f, wo, *wi);
        return leaf_evaluate(f, wo, *wi);
    }
    if (f->type == YAR_MATERIAL_PBRT3_TRANSLUCENT) { /* src/ref/bsdf_pbrt.cpp:160-209 */
        float max_r = maxcomp(f->reflectance), max_t = maxcomp(f->transmittance);
        float rp = max_r / (max_r + max_t);
        if (u_scatter < rp) {
            float u = u_scatter / rp;
            u = u < ONE_MINUS_EPSILON ? u : ONE_MINUS_EPSILON;
            if (u < 0.5f) {
                *wi = local_to_world(f, sample_hemisphere_cosine(u0, u1));
            } else {
                v3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, world_to_local(f, wo), f->alpha, f->alpha));
                v3 c = reflect3(wo, wh);
                if (dot3(c, f->n) <= 0.f) return mkc(0, 0, 0);
                *wi = c;
            }
        } else {
            float u = (u_scatter - rp) / (1.f - rp);
            u = u < ONE_MINUS_EPSILON ? u : ONE_MINUS_EPSILON;
            if (u < 0.5f) {
                *wi = local_to_world(f, neg3(sample_hemisphere_cosine(u0, u1)));
            } else {
                v3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, world_to_local(f, wo), f->alpha, f->alpha));
                if (dot3(wh, wo) < 0.f) return mkc(0, 0, 0);
                v3 c;
                if (!refract3(wo, wh, f->eta_o / f->eta_i, &c)) return mkc(0, 0, 0);
                if (dot3(c, f->n) >= 0.f) return mkc(0, 0, 0);
                *wi = c;
            }
        }
        *pdf = leaf_pdf(f, wo, *wi);
        if (*pdf == 0.f) return mkc(0, 0, 0);
        return leaf_evaluate(f, wo, *wi);
    }
    if (f->type == YAR_MATERIAL_DIFFUSE || f->type == YAR_MATERIAL_PBRT3_FOURIER) {
        /* Pbrt3_Fourier_BSDF::sample (src/ref/bsdf_pbrt.cpp:360-366) samples as Diffuse_BRDF */
        v3 l = sample_hemisphere_cosine(u0, u1);
        *wi = local_to_world(f, l);
        *pdf = leaf_pdf(f, wo, *wi);
        return leaf_evaluate(f, wo, *wi);
    }
    if (f->type == YAR_MATERIAL_PLASTIC || f->type == YAR_MATERIAL_COATED_DIFFUSE ||
        f->type == YAR_MATERIAL_PBRT3_UBER) {
        /* Pbrt3_Uber_BRDF::sample (src/ref/bsdf_pbrt.cpp:54-72) has the same shape.
         * Plastic_BRDF::sample, src/ref/bsdf.cpp:236-251; Ashikhmin_Shirley_Phong_BRDF::sample,
         * :462-478: the first 1D sample picks the diffuse or the specular lobe */
        if (u_scatter < 0.5f) {
            *wi = local_to_world(f, sample_hemisphere_cosine(u0, u1));
        } else {
            v3 wo_l = world_to_local(f, wo);
            if (f->type == YAR_MATERIAL_PLASTIC) {
                v3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, wo_l, f->alpha, f->alpha));
                *wi = reflect3(wo, wh);
            } else {
                v3 wh_l = ggx_sample_vndf(u0, u1, wo_l, f->alpha_x, f->alpha_y);
                *wi = local_to_world(f, reflect3(wo_l, wh_l));
            }
        }
        if (dot3(f->n, *wi) <= 0.f) return mkc(0, 0, 0);
        *pdf = leaf_pdf(f, wo, *wi);
        return leaf_evaluate(f, wo, *wi);
    }
    if (f->type == YAR_MATERIAL_METAL) {
        v3 wo_l = world_to_local(f, wo);
        v3 wh_l = ggx_sample_vndf(u0, u1, wo_l, f->alpha_x, f->alpha_y);
        v3 wi_l = reflect3(wo_l, wh_l);
        if (wi_l.z <= 0.f) return mkc(0, 0, 0);
        *wi = local_to_world(f, wi_l);
        *pdf = refl_pdf_aniso(wo_l, wh_l, f->alpha_x, f->alpha_y);
        return leaf_evaluate(f, wo, *wi);
    }
    /* rough glass, src/ref/bsdf.cpp:336-370 */
    v3 wo_l = world_to_local(f, wo);
    v3 wh_l = ggx_sample_vndf(u0, u1, wo_l, f->alpha, f->alpha);
    v3 wh = local_to_world(f, wh_l);
    v3 rwi = reflect3(wo, wh);
    if (dot3(rwi, f->n) <= 0.f) return mkc(0, 0, 0);
    float cos_i = dot3(wo, wh);
    float fresnel = dielectric_fresnel(cos_i, f->eta_i / f->eta_o);
    float rprob = glass_reflection_probability(f, fresnel);
    if (u_scatter < rprob) {
        *wi = rwi;
    } else {
        if (!refract3(wo, wh, f->eta_o / f->eta_i, wi)) return mkc(0, 0, 0);
        if (dot3(*wi, f->n) >= 0.f) return mkc(0, 0, 0);
    }
    *pdf = leaf_pdf(f, wo, *wi);
    if (*pdf == 0.f) return mkc(0, 0, 0);
    return leaf_evaluate(f, wo, *wi);
}

/* Mix_BSDF (src/ref/bsdf.cpp:497-567) and Scaled_BSDF (:572-592) over leaf
 * BSDFs; every other BSDF forwards to its own functions. */
static int possible_for(const bsdf_t* f, float n_dot_wi) {
    return (n_dot_wi > 0 && f->reflection) || (n_dot_wi < 0 && f->transmission);
}
static col bsdf_evaluate(const bsdf_t* f, v3 wo, v3 wi) {
    if (f->type == ORACLE_BSDF_SCALED) return mulcs(leaf_evaluate(f->sub[0], wo, wi), f->scale);
    if (f->type != YAR_MATERIAL_MIX) return leaf_evaluate(f, wo, wi);
    col f1 = mkc(0, 0, 0), f2 = mkc(0, 0, 0);
    float n_dot_wi = dot3(f->n, wi);
    if (possible_for(f->sub[0], n_dot_wi)) f1 = leaf_evaluate(f->sub[0], wo, wi);
    if (possible_for(f->sub[1], n_dot_wi)) f2 = leaf_evaluate(f->sub[1], wo, wi);
    return addc(mulc(subc(mkc(1, 1, 1), f->mix_coeff), f1), mulc(f->mix_coeff, f2));
}
static float bsdf_pdf(const bsdf_t* f, v3 wo, v3 wi) {
    if (f->type == ORACLE_BSDF_SCALED) return leaf_pdf(f->sub[0], wo, wi);
    if (f->type != YAR_MATERIAL_MIX) return leaf_pdf(f, wo, wi);
    float n_dot_wi = dot3(f->n, wi);
    float pdf1 = 0.f, pdf2 = 0.f;
    if (possible_for(f->sub[0], n_dot_wi)) pdf1 = leaf_pdf(f->sub[0], wo, wi);
    if (possible_for(f->sub[1], n_dot_wi)) pdf2 = leaf_pdf(f->sub[1], wo, wi);
    return (1.f - f->p_coeff) * pdf1 + f->p_coeff * pdf2;
}
static col bsdf_sample(const bsdf_t* f, float u0, float u1, float u_scatter, v3 wo, v3* wi, float* pdf) {
    if (f->type == ORACLE_BSDF_SCALED) return mulcs(leaf_sample(f->sub[0], u0, u1, u_scatter, wo, wi, pdf), f->scale);
    if (f->type != YAR_MATERIAL_MIX) return leaf_sample(f, u0, u1, u_scatter, wo, wi, pdf);
    col f1 = mkc(0, 0, 0), f2 = mkc(0, 0, 0);
    float pdf1 = 0.f, pdf2 = 0.f;
    if (u_scatter < f->p_coeff) {
        f2 = leaf_sample(f->sub[1], u0, u1, u_scatter / f->p_coeff, wo, wi, &pdf2);
        float n_dot_wi = dot3(f->n, *wi);
        if (possible_for(f->sub[0], n_dot_wi)) {
            pdf1 = leaf_pdf(f->sub[0], wo, *wi);
            f1 = leaf_evaluate(f->sub[0], wo, *wi);
        }
    } else {
        f1 = leaf_sample(f->sub[0], u0, u1, (u_scatter - f->p_coeff) / (1.f - f->p_coeff), wo, wi, &pdf1);
        float n_dot_wi = dot3(f->n, *wi);
        if (possible_for(f->sub[1], n_dot_wi)) {
            pdf2 = leaf_pdf(f->sub[1], wo, *wi);
            f2 = leaf_evaluate(f->sub[1], wo, *wi);
        }
    }
    *pdf = (1.f - f->p_coeff) * pdf1 + f->p_coeff * pdf2;
    return addc(mulc(subc(mkc(1, 1, 1), f->mix_coeff), f1), mulc(f->mix_coeff, f2));
}

/* ---------------- ray queries on the flat scene */
static int trace_closest(const yar_flat_scene* s, v3 o, v3 d, hit_state* hit) {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    hit->t = INFINITY;
    hit->prim = hit->object = 0xffffffffu;
    return scene_closest(s, oo, dd, hit, NULL);
}
static int trace_any(const yar_flat_scene* s, v3 o, v3 d, float tmax) {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    return scene_any(s, oo, dd, tmax, NULL);
}

/* mis_power_heuristic, src/ref/direct_lighting.cpp:18-24 */
static float mis_power(float p1, float p2) {
    if (p1 == INFINITY) return 1.f;
    return p1 * p1 / (p1 * p1 + p2 * p2);
}

/* direct_lighting_from_rectangular_light, src/ref/direct_lighting.cpp:109-194 */
static col direct_rect(const yar_flat_scene* s, const shading_ctx* sc, const bsdf_t* f, int light_index, float ul0,
                       float ul1, float ub0, float ub1, float u_scatter) {
    const yar_rect_light_desc* L = &s->rect_lights[light_index];
    const float* m = L->light_to_world;
    v3 light_n = mk3(m[2], m[6], m[10]);
    col Le = ldc(L->emitted_radiance);
    col out = mkc(0, 0, 0);
    int have = 0;
    {
        v3 local = mk3(L->size[0] * (ul0 - 0.5f), L->size[1] * (ul1 - 0.5f), 0.0f);
        v3 lp = xform_point(m, local);
        v3 position = origin_for_point(sc, lp);
        v3 lv = sub3(lp, position);
        float dist = len3(lv);
        v3 wi = div3s(lv, dist);
        float lndw = dot3(light_n, neg3(wi));
        if (lndw > 1e-4f) {
            float ndw = dot3(sc->normal, wi);
            int possible = (ndw > 0.f && f->reflection) || (ndw < 0.f && f->transmission);
            if (possible) {
                col fv = bsdf_evaluate(f, sc->wo, wi);
                if (!blackc(fv)) {
                    if (!trace_any(s, position, wi, dist * (1.f - 1e-5f))) {
                        float light_pdf = (dist * dist) / (L->size[0] * L->size[1] * lndw);
                        float bpdf = bsdf_pdf(f, sc->wo, wi);
                        float w = mis_power(light_pdf, bpdf);
                        col c = mulcs(mulc(Le, fv), w * fabsf(ndw) / light_pdf);
                        out = have ? addc(out, c) : addc(mkc(0, 0, 0), c);
                        have = 1;
                    }
                }
            }
        }
    }
    {
        v3 wi = mk3(0, 0, 0); /* Vector3 default: a BSDF sample may leave it unset */
        float bpdf;
        col fv = bsdf_sample(f, ub0, ub1, u_scatter, sc->wo, &wi, &bpdf);
        if (!blackc(fv)) {
            float lndw = dot3(light_n, neg3(wi));
            if (lndw > 1e-4f) {
                v3 position = origin_for_direction(sc, wi);
                hit_state h;
                if (trace_closest(s, position, wi, &h) > 0) {
                    const yar_object_desc* o = &s->objects[h.object];
                    if (o->area_light_type == YAR_LIGHT_DIFFUSE_RECTANGULAR && o->area_light_index == light_index) {
                        const yar_mesh_desc* mm = &s->meshes[o->mesh_index];
                        const int32_t* vi = mm->indices + 3 * (size_t)h.prim;
                        v3 p[3] = {ld3(mm->vertices + 3 * (size_t)vi[0]), ld3(mm->vertices + 3 * (size_t)vi[1]),
                                   ld3(mm->vertices + 3 * (size_t)vi[2])};
                        v3 hp = bary3(p, h.b);
                        float d = len3(sub3(hp, position));
                        float light_pdf = (d * d) / (L->size[0] * L->size[1] * lndw);
                        float w = mis_power(bpdf, light_pdf);
                        float ndw = dot3(sc->normal, wi);
                        col c = mulcs(mulc(Le, fv), w * fabsf(ndw) / bpdf);
                        out = have ? addc(out, c) : addc(mkc(0, 0, 0), c);
                        have = 1;
                    }
                }
            }
        }
    }
    return out;
}

/* direct_lighting_from_point_light / _spot_light / _directional_light,
 * src/ref/direct_lighting.cpp:26-107: one shadow ray, no MIS. */
static col direct_delta(const yar_flat_scene* s, const shading_ctx* sc, const bsdf_t* f, const yar_delta_light_desc* L) {
    const col black = mkc(0, 0, 0);
    const col I = ldc(L->intensity);
    const v3 ldir = ld3(L->direction);
    if (L->type == YAR_LIGHT_DIRECTIONAL) {
        float n_dot_l = dot3(sc->normal, ldir);
        if (n_dot_l <= 0.f) return black;
        v3 position = origin_for_direction(sc, ldir);
        if (trace_any(s, position, ldir, INFINITY)) return black;
        return mulcs(mulc(I, bsdf_evaluate(f, sc->wo, ldir)), n_dot_l);
    }
    const v3 lpos = ld3(L->position);
    v3 position = origin_for_point(sc, lpos);
    v3 lv = sub3(lpos, position);
    float dist = len3(lv);
    v3 wi = div3s(lv, dist);
    if (L->type == YAR_LIGHT_POINT) {
        float n_dot_l = dot3(sc->normal, wi);
        if (n_dot_l <= 0.f) return black;
        if (trace_any(s, position, wi, dist * (1.f - 1e-5f))) return black;
        return mulcs(mulc(I, bsdf_evaluate(f, sc->wo, wi)), n_dot_l / (dist * dist));
    }
    float cone_cos = cosf(L->cone_angle);
    float wi_cos = dot3(neg3(wi), ldir);
    if (wi_cos < cone_cos) return black;
    float penumbra_attenuation = 1.f;
    float penumbra_cos = cosf(fmaxf_std(0.f, L->cone_angle - L->penumbra_angle));
    if (wi_cos < penumbra_cos) {
        float k = (wi_cos - cone_cos) / (penumbra_cos - cone_cos);
        penumbra_attenuation = (k * k) * (k * k);
    }
    float n_dot_wi = dot3(sc->normal, wi);
    int possible = (n_dot_wi > 0.f && f->reflection) || (n_dot_wi < 0.f && f->transmission);
    if (!possible) return black;
    col fv = bsdf_evaluate(f, sc->wo, wi);
    if (blackc(fv)) return black;
    if (trace_any(s, position, wi, dist * (1.f - 1e-5f))) return black;
    return mulcs(mulc(I, fv), penumbra_attenuation * fabsf(n_dot_wi) / (dist * dist));
}

/* Diffuse_Triangle_Mesh_Light_Sampler with its Distribution_1D over triangle
 * areas, built as init_triangle_mesh_light_samplers does
 * (src/ref/reference_renderer.cpp:131-151). */
typedef struct mesh_light_sampler {
    const yar_mesh_desc* mesh;
    float mesh_area;
    float interval_length;
    float* cdf; /* triangle_count entries */
} mesh_light_sampler;

static v3 mesh_vertex(const yar_mesh_desc* m, uint32_t tri, int k) {
    return ld3(m->vertices + 3 * (size_t)m->indices[3 * (size_t)tri + k]);
}
/* Triangle_Mesh::get_triangle_area, src/lib/triangle_mesh.h:103-109 */
static float triangle_area(const yar_mesh_desc* m, uint32_t tri) {
    v3 p0 = mesh_vertex(m, tri, 0), p1 = mesh_vertex(m, tri, 1), p2 = mesh_vertex(m, tri, 2);
    return len3(cross3(sub3(p1, p0), sub3(p2, p0))) * 0.5f;
}
static void free_mesh_samplers(mesh_light_sampler* ms, uint32_t n) {
    if (!ms) return;
    for (uint32_t i = 0; i < n; i++) free(ms[i].cdf);
    free(ms);
}
/* Triangle_Mesh::get_area (:111-118) and Distribution_1D::initialize (src/ref/sampling.cpp:149-166) */
static int build_mesh_samplers(const yar_flat_scene* s, mesh_light_sampler** out) {
    *out = NULL;
    if (!s->mesh_light_count) return YAR_OK;
    mesh_light_sampler* ms = (mesh_light_sampler*)calloc(s->mesh_light_count, sizeof(mesh_light_sampler));
    if (!ms) return YAR_ERR_CAPACITY;
    for (uint32_t i = 0; i < s->mesh_light_count; i++) {
        const uint32_t mi = s->mesh_lights[i].triangle_mesh_index;
        if (mi >= s->mesh_count || s->meshes[mi].triangle_count == 0) {
            free_mesh_samplers(ms, s->mesh_light_count);
            return YAR_ERR_INVALID;
        }
        const yar_mesh_desc* m = &s->meshes[mi];
        const uint32_t n = m->triangle_count;
        ms[i].mesh = m;
        ms[i].cdf = (float*)malloc(sizeof(float) * n);
        if (!ms[i].cdf) {
            free_mesh_samplers(ms, s->mesh_light_count);
            return YAR_ERR_CAPACITY;
        }
        float area = 0.f;
        for (uint32_t t = 0; t < n; t++) area += triangle_area(m, t);
        ms[i].mesh_area = area;
        ms[i].interval_length = 1.f / (float)n;
        float total = 0.f, sum = 0.f;
        for (uint32_t t = 0; t < n; t++) total += triangle_area(m, t);
        for (uint32_t t = 0; t < n; t++) {
            sum += triangle_area(m, t);
            ms[i].cdf[t] = sum / total;
        }
    }
    *out = ms;
    return YAR_OK;
}

/* The light's normal at a point of triangle tri: the interpolated vertex normal
 * (not normalised) or the geometric normal (Triangle_Mesh::get_normal /
 * get_geometric_normal, src/lib/triangle_mesh.h:61-77). */
static v3 mesh_light_normal(const yar_mesh_desc* m, uint32_t tri, const float b[3]) {
    if (m->normals) {
        const int32_t* vi = m->indices + 3 * (size_t)tri;
        v3 n[3] = {ld3(m->normals + 3 * (size_t)vi[0]), ld3(m->normals + 3 * (size_t)vi[1]),
                   ld3(m->normals + 3 * (size_t)vi[2])};
        return bary3(n, b);
    }
    v3 p0 = mesh_vertex(m, tri, 0), p1 = mesh_vertex(m, tri, 1), p2 = mesh_vertex(m, tri, 2);
    v3 gn = norm3(cross3(sub3(p1, p0), sub3(p2, p0)));
    return m->reverse_geometric_normal_orientation ? neg3(gn) : gn;
}

/* Diffuse_Triangle_Mesh_Light_Sampler::sample (src/ref/light_sampling.cpp:126-161) with
 * sample_from_CDF (src/ref/sampling.cpp:98-147) and uniform_sample_triangle_baricentrics (:69-77) */
static v3 mesh_light_sample(const mesh_light_sampler* ms, float u0, float u1, v3 shading_pos, float* pdf) {
    const uint32_t n = ms->mesh->triangle_count;
    uint32_t k = 0;
    while (k < n - 1 && ms->cdf[k] < u0) k++; /* std::lower_bound */
    const float cdf_a = k == 0 ? 0.f : ms->cdf[k - 1], cdf_b = ms->cdf[k];
    const float fraction = (u0 - cdf_a) / (cdf_b - cdf_a);
    float x = ((float)k + fraction) * ms->interval_length;
    x = x < ONE_MINUS_EPSILON ? x : ONE_MINUS_EPSILON;
    const float remapped = fraction < ONE_MINUS_EPSILON ? fraction : ONE_MINUS_EPSILON;
    uint32_t tri = (uint32_t)(x * (float)n);
    if (tri > n - 1) tri = n - 1;
    const float a = sqrtf(remapped);
    float b[3];
    b[0] = 1 - a;
    b[1] = u1 * a;
    b[2] = 1.f - b[0] - b[1];
    v3 p[3] = {mesh_vertex(ms->mesh, tri, 0), mesh_vertex(ms->mesh, tri, 1), mesh_vertex(ms->mesh, tri, 2)};
    v3 light_p = bary3(p, b);
    v3 light_n = mesh_light_normal(ms->mesh, tri, b);
    v3 lv = sub3(light_p, shading_pos);
    float d2 = len2_3(lv);
    v3 wi = div3s(lv, sqrtf(d2));
    float lndw = dot3(light_n, neg3(wi));
    *pdf = lndw <= 0.f ? 0.f : d2 / (lndw * ms->mesh_area);
    return light_p;
}

/* direct_lighting_from_triangle_mesh_light, src/ref/direct_lighting.cpp:262-322 */
static col direct_mesh(const yar_flat_scene* s, const shading_ctx* sc, const bsdf_t* f, const mesh_light_sampler* ms,
                       int light_index, float ul0, float ul1, float ub0, float ub1, float u_scatter) {
    const col Le = ldc(s->mesh_lights[light_index].emitted_radiance);
    col out = mkc(0, 0, 0);
    int have = 0;
    {
        float light_pdf;
        v3 lp = mesh_light_sample(ms, ul0, ul1, sc->position, &light_pdf);
        if (light_pdf != 0.f) {
            v3 position = origin_for_point(sc, lp);
            v3 lv = sub3(lp, position);
            float dist = len3(lv);
            v3 wi = div3s(lv, dist);
            float ndw = dot3(sc->normal, wi);
            int possible = (ndw > 0.f && f->reflection) || (ndw < 0.f && f->transmission);
            if (possible) {
                col fv = bsdf_evaluate(f, sc->wo, wi);
                if (!blackc(fv) && !trace_any(s, position, wi, dist * (1.f - 1e-5f))) {
                    float bpdf = bsdf_pdf(f, sc->wo, wi);
                    float w = mis_power(light_pdf, bpdf);
                    out = addc(out, mulcs(mulc(Le, fv), w * fabsf(ndw) / light_pdf));
                    have = 1;
                }
            }
        }
    }
    {
        v3 wi = mk3(0, 0, 0);
        float bpdf;
        col fv = bsdf_sample(f, ub0, ub1, u_scatter, sc->wo, &wi, &bpdf);
        if (!blackc(fv)) {
            v3 position = origin_for_direction(sc, wi);
            hit_state h;
            if (trace_closest(s, position, wi, &h) > 0) {
                const yar_object_desc* o = &s->objects[h.object];
                if (o->area_light_type == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH && o->area_light_index == light_index) {
                    /* Diffuse_Triangle_Mesh_Light_Sampler::pdf (light_sampling.cpp:163-184) */
                    v3 light_n = mesh_light_normal(ms->mesh, h.prim, h.b);
                    float lndw = dot3(light_n, neg3(wi));
                    float light_pdf = lndw <= 0.f ? 0.f : (h.t * h.t) / (lndw * ms->mesh_area);
                    float w = mis_power(bpdf, light_pdf);
                    col c = mulcs(mulc(Le, fv), w * fabsf(dot3(sc->normal, wi)) / bpdf);
                    out = have ? addc(out, c) : addc(mkc(0, 0, 0), c);
                    have = 1;
                }
            }
        }
    }
    return out;
}

/* Diffuse_Sphere_Light_Sampler (src/ref/light_sampling.cpp:76-123), built per
 * shading point, and direct_lighting_from_sphere_light (direct_lighting.cpp:196-260). */
typedef struct sphere_sampler {
    v3 center, axes[3];
    float radius, d_center, cos_theta_max, cone_pdf;
} sphere_sampler;

static void sphere_sampler_init(sphere_sampler* ss, const yar_sphere_light_desc* L, v3 shading_pos) {
    ss->center = ld3(L->position);
    ss->radius = L->radius;
    v3 a2 = sub3(shading_pos, ss->center);
    ss->d_center = len3(a2);
    a2 = div3s(a2, ss->d_center);
    /* coordinate_system_from_vector, src/lib/math.cpp:21-25 */
    v3 a0 = fabsf(a2.x) > fabsf(a2.y) ? mk3(-a2.z, 0, a2.x) : mk3(0, -a2.z, a2.y);
    a0 = div3s(a0, len3(a0));
    ss->axes[0] = a0;
    ss->axes[1] = cross3(a2, a0);
    ss->axes[2] = a2;
    float sin_theta_max = ss->radius / ss->d_center;
    ss->cos_theta_max = sqrtf(fmaxf_std(0.f, 1.f - sin_theta_max * sin_theta_max));
    ss->cone_pdf = 1.f / (2.f * PI_F * (1.f - ss->cos_theta_max));
}

static v3 sphere_sampler_sample(const sphere_sampler* ss, float u0, float u1) {
    float radius2 = ss->radius * ss->radius;
    float d_center2 = ss->d_center * ss->d_center;
    float cos_theta = (1.f - u0) + u0 * ss->cos_theta_max;
    float phi = 2.f * PI_F * u1;
    float sin_theta2 = fmaxf_std(0.f, 1.f - cos_theta * cos_theta);
    float d_sample = ss->d_center * cos_theta - sqrtf(fmaxf_std(0.f, radius2 - d_center2 * sin_theta2));
    float cos_alpha = (d_center2 + radius2 - d_sample * d_sample) / (2.f * ss->d_center * ss->radius);
    float sin_alpha = sqrtf(fmaxf_std(0.f, 1.f - cos_alpha * cos_alpha));
    v3 dir = add3(add3(mul3s(ss->axes[0], sin_alpha * cos_sample(phi)), mul3s(ss->axes[1], sin_alpha * sin_sample(phi))),
                  mul3s(ss->axes[2], cos_alpha));
    return add3(mul3s(dir, ss->radius), ss->center);
}

static col direct_sphere(const yar_flat_scene* s, const shading_ctx* sc, const bsdf_t* f, int light_index, float ul0,
                         float ul1, float ub0, float ub1, float u_scatter) {
    const yar_sphere_light_desc* L = &s->sphere_lights[light_index];
    const col Le = ldc(L->emitted_radiance);
    sphere_sampler ss;
    sphere_sampler_init(&ss, L, sc->position);
    col out = mkc(0, 0, 0);
    int have = 0;
    {
        v3 lp = sphere_sampler_sample(&ss, ul0, ul1);
        v3 position = origin_for_point(sc, lp);
        v3 lv = sub3(lp, position);
        float dist = len3(lv);
        v3 wi = div3s(lv, dist);
        float ndw = dot3(sc->normal, wi);
        int possible = (ndw > 0.f && f->reflection) || (ndw < 0.f && f->transmission);
        if (possible) {
            col fv = bsdf_evaluate(f, sc->wo, wi);
            if (!blackc(fv) && !trace_any(s, position, wi, dist * (1.f - 1e-5f))) {
                float bpdf = bsdf_pdf(f, sc->wo, wi);
                float w = mis_power(ss.cone_pdf, bpdf);
                out = addc(out, mulcs(mulc(Le, fv), w * fabsf(ndw) / ss.cone_pdf));
                have = 1;
            }
        }
    }
    {
        v3 wi = mk3(0, 0, 0);
        float bpdf;
        col fv = bsdf_sample(f, ub0, ub1, u_scatter, sc->wo, &wi, &bpdf);
        if (!blackc(fv) && dot3(neg3(ss.axes[2]), wi) >= ss.cos_theta_max) {
            v3 position = origin_for_direction(sc, wi);
            hit_state h;
            if (trace_closest(s, position, wi, &h) > 0) {
                const yar_object_desc* o = &s->objects[h.object];
                if (o->area_light_type == YAR_LIGHT_DIFFUSE_SPHERE && o->area_light_index == light_index) {
                    float w = mis_power(bpdf, ss.cone_pdf);
                    col c = mulcs(mulc(Le, fv), w * fabsf(dot3(sc->normal, wi)) / bpdf);
                    out = have ? addc(out, c) : addc(mkc(0, 0, 0), c);
                    have = 1;
                }
            }
        }
    }
    return out;
}

/* Environment_Light_Sampler (src/ref/light_sampling.cpp:11-71) over the map's
 * mip 0, with Distribution_2D (src/ref/sampling.cpp:185-276) built by
 * initialize_from_latitude_longitude_radiance_map (:236-259). */
#define PI2_F 6.2831853f /* src/lib/math.h:10 */
typedef struct env_sampler {
    const yar_environment_desc* e;
    int nx, ny;
    float x_interval, y_interval;
    float* marginal; /* ny */
    float* cdfs;     /* nx * ny */
} env_sampler;

static col env_texel(const yar_environment_desc* e, int x, int y) { /* get_texel_clamp, image_texture.cpp:417-421 */
    x = x < 0 ? 0 : ((int)e->width - 1 < x ? (int)e->width - 1 : x);
    y = y < 0 ? 0 : ((int)e->height - 1 < y ? (int)e->height - 1 : y);
    return ldc(e->radiance + 3 * ((size_t)y * e->width + x));
}
static col env_nearest(const yar_environment_desc* e, float u, float v) { /* sample_nearest, :423-439 */
    return env_texel(e, (int)(u * (float)e->width), (int)(v * (float)e->height));
}
static col env_bilinear(const yar_environment_desc* e, float u, float v) { /* sample_bilinear, :441-480 */
    float x = u * (float)e->width - 0.5f, y = v * (float)e->height - 0.5f;
    float x_floor = floorf(x), y_floor = floorf(y);
    float wx = x - x_floor, wy = y - y_floor;
    int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    col c = addc(addc(addc(mulcs(env_texel(e, x0, y0), (1 - wy) * (1 - wx)), mulcs(env_texel(e, x1, y0), (1 - wy) * wx)),
                      mulcs(env_texel(e, x0, y1), wy * (1 - wx))),
                 mulcs(env_texel(e, x1, y1), wy * wx));
    return c;
}
static v3 xform_vec(const float m[12], v3 v) { /* transform_vector, src/lib/matrix.cpp:376-382 */
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
               m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
static void env_uv(v3 d, float* u, float* v) { /* get_uv_from_direction, light_sampling.cpp:15-25 */
    float phi = atan2_sample(d.y, d.x);
    phi = phi < 0 ? phi + PI2_F : phi;
    float z = d.z < -1.f ? -1.f : (1.f < d.z ? 1.f : d.z);
    float theta = acos_sample(z);
    float a = phi * (1.f / PI2_F);
    *u = a < 0.f ? 0.f : (ONE_MINUS_EPSILON < a ? ONE_MINUS_EPSILON : a);
    float b = theta * PI_INV_F;
    *v = b < ONE_MINUS_EPSILON ? b : ONE_MINUS_EPSILON;
}
static void free_env_sampler(env_sampler* es) {
    free(es->marginal);
    free(es->cdfs);
}
static int build_env_sampler(const yar_flat_scene* s, env_sampler* es) {
    memset(es, 0, sizeof(*es));
    const yar_environment_desc* e = s->environment;
    if (!e) return YAR_OK;
    if (!e->radiance || e->width == 0 || e->height == 0) return YAR_ERR_INVALID;
    const int nx = (int)e->width, ny = (int)e->height;
    es->e = e;
    es->nx = nx;
    es->ny = ny;
    es->x_interval = 1.f / (float)nx;
    es->y_interval = 1.f / (float)ny;
    float* values = (float*)malloc(sizeof(float) * (size_t)nx * ny);
    float* row_sums = (float*)malloc(sizeof(float) * (size_t)ny);
    es->marginal = (float*)malloc(sizeof(float) * (size_t)ny);
    es->cdfs = (float*)calloc((size_t)nx * ny, sizeof(float));
    if (!values || !row_sums || !es->marginal || !es->cdfs) {
        free(values);
        free(row_sums);
        free_env_sampler(es);
        return YAR_ERR_CAPACITY;
    }
    for (int y = 0; y < ny; y++) {
        float sin_theta = sinf((y + 0.5f) / (float)ny * PI_F);
        float v = (y + 0.5f) / (float)ny;
        for (int x = 0; x < nx; x++) {
            float u = (x + 0.5f) / (float)nx;
            values[(size_t)y * nx + x] = luminance(env_nearest(e, u, v)) * sin_theta;
        }
    }
    float total = 0.f;
    int last_nonzero = -1;
    for (int y = 0; y < ny; y++) {
        float row = 0.f;
        for (int x = 0; x < nx; x++) row += values[(size_t)y * nx + x];
        row_sums[y] = row;
        total += row;
        if (row != 0.f) last_nonzero = y;
    }
    int rc = YAR_OK;
    if (last_nonzero < 0) {
        rc = YAR_ERR_UNSUPPORTED; /* the reference asserts on an all-black map */
    } else {
        for (int y = 0; y < last_nonzero; y++) es->marginal[y] = (y == 0 ? 0.f : es->marginal[y - 1]) + row_sums[y] / total;
        for (int y = last_nonzero; y < ny; y++) es->marginal[y] = 1.f;
        for (int y = 0; y < ny; y++) {
            float* cdf = es->cdfs + (size_t)y * nx;
            if (row_sums[y] == 0.f) continue;
            for (int x = 0; x < nx - 1; x++) cdf[x] = (x == 0 ? 0.f : cdf[x - 1]) + values[(size_t)y * nx + x] / row_sums[y];
            cdf[nx - 1] = 1.f;
        }
    }
    free(values);
    free(row_sums);
    if (rc != YAR_OK) free_env_sampler(es);
    return rc;
}
/* sample_from_CDF (src/ref/sampling.cpp:98-147) returning the interval too */
static float cdf_sample(const float* cdf, int n, float interval, float u, float* pdf, int* index) {
    int k = 0;
    while (k < n - 1 && cdf[k] < u) k++;
    float a = k == 0 ? 0.f : cdf[k - 1], b = cdf[k];
    float fraction = (u - a) / (b - a);
    float x = ((float)k + fraction) * interval;
    *pdf = (b - a) * (float)n;
    *index = k;
    return x < ONE_MINUS_EPSILON ? x : ONE_MINUS_EPSILON;
}
static float env_pdf_uv(const env_sampler* es, float u, float v) { /* Distribution_2D::pdf_uv, :278-291 */
    int x = (int)(u * (float)es->nx), y = (int)(v * (float)es->ny);
    float pdf_y = (es->marginal[y] - (y == 0 ? 0.f : es->marginal[y - 1])) * (float)es->ny;
    const float* c = es->cdfs + (size_t)y * es->nx;
    float pdf_x = (c[x] - (x == 0 ? 0.f : c[x - 1])) * (float)es->nx;
    return pdf_y * pdf_x;
}
static col env_radiance(const env_sampler* es, v3 world_dir, int filtered) {
    float u, v;
    env_uv(xform_vec(es->e->world_to_light, world_dir), &u, &v);
    col c = filtered ? env_bilinear(es->e, u, v) : env_nearest(es->e, u, v);
    return mulc(c, ldc(es->e->scale));
}
static float env_light_pdf(const env_sampler* es, v3 world_dir) { /* Environment_Light_Sampler::pdf, :61-71 */
    v3 d = xform_vec(es->e->world_to_light, world_dir);
    float u, v;
    env_uv(d, &u, &v);
    float pdf_uv = env_pdf_uv(es, u, v);
    float sin_theta = sqrtf(fmaxf_std(0.f, 1.f - d.z * d.z));
    return pdf_uv / (2 * PI_F * PI_F * sin_theta);
}
static col env_light_sample(const env_sampler* es, float u0, float u1, v3* wi, float* pdf) { /* :29-49 */
    float pdf_y, pdf_x;
    int y, x;
    float ky = cdf_sample(es->marginal, es->ny, es->y_interval, u0, &pdf_y, &y);
    float kx = cdf_sample(es->cdfs + (size_t)y * es->nx, es->nx, es->x_interval, u1, &pdf_x, &x);
    float pdf_uv = pdf_y * pdf_x;
    float phi = kx * PI2_F, theta = ky * PI_F;
    float sin_theta = sin_sample(theta);
    *pdf = pdf_uv / (2 * PI_F * PI_F * sin_theta);
    *wi = xform_vec(es->e->light_to_world, mk3(sin_theta * cos_sample(phi), sin_theta * sin_sample(phi), cos_sample(theta)));
    return mulc(env_nearest(es->e, kx, ky), ldc(es->e->scale));
}

/* direct_lighting_from_environment_light, src/ref/direct_lighting.cpp:324-384 */
static col direct_env(const yar_flat_scene* s, const shading_ctx* sc, const bsdf_t* f, const env_sampler* es,
                      float ul0, float ul1, float ub0, float ub1, float u_scatter) {
    col out = mkc(0, 0, 0);
    int have = 0;
    {
        v3 wi;
        float light_pdf;
        col Le = env_light_sample(es, ul0, ul1, &wi, &light_pdf);
        float ndw = dot3(sc->normal, wi);
        int possible = (ndw > 0.f && f->reflection) || (ndw < 0.f && f->transmission);
        if (possible) {
            col fv = bsdf_evaluate(f, sc->wo, wi);
            if (!blackc(fv)) {
                v3 position = origin_for_direction(sc, wi);
                if (!trace_any(s, position, wi, INFINITY)) {
                    float bpdf = bsdf_pdf(f, sc->wo, wi);
                    float w = mis_power(light_pdf, bpdf);
                    out = addc(out, mulcs(mulc(Le, fv), w * fabsf(ndw) / light_pdf));
                    have = 1;
                }
            }
        }
    }
    {
        v3 wi = mk3(0, 0, 0);
        float bpdf;
        col fv = bsdf_sample(f, ub0, ub1, u_scatter, sc->wo, &wi, &bpdf);
        if (!blackc(fv)) {
            col Le = env_radiance(es, wi, 0);
            if (!blackc(Le)) {
                v3 position = origin_for_direction(sc, wi);
                if (!trace_any(s, position, wi, INFINITY)) {
                    float light_pdf = env_light_pdf(es, wi);
                    float w = mis_power(bpdf, light_pdf);
                    col c = mulcs(mulc(Le, fv), w * fabsf(dot3(sc->normal, wi)) / bpdf);
                    out = have ? addc(out, c) : addc(mkc(0, 0, 0), c);
                    have = 1;
                }
            }
        }
    }
    return out;
}

typedef struct sampler_view {
    const float* s1d;   /* this sample's 1d dims */
    const float* s2d;   /* this sample's 2d dims (pairs) */
    int n1d, n2d, i1d, i2d;
    oracle_pcg32* rng;  /* the pixel rng for dims beyond the budget */
} sampler_view;

static float next1d(sampler_view* sv) {
    if (sv->i1d < sv->n1d) return sv->s1d[sv->i1d++];
    return oracle_pcg32_float(sv->rng);
}
static void next2d(sampler_view* sv, float* a, float* b) {
    if (sv->i2d < sv->n2d) {
        *a = sv->s2d[2 * sv->i2d];
        *b = sv->s2d[2 * sv->i2d + 1];
        sv->i2d++;
        return;
    }
    *a = oracle_pcg32_float(sv->rng);
    *b = oracle_pcg32_float(sv->rng);
}

/* Camera::generate_ray, src/ref/camera.cpp:16-31 */
static void camera_ray(const yar_camera_desc* c, float fx, float fy, v3* o, v3* d) {
    float u = 2.f * (fx / c->image_extent[0]) - 1.f;
    float v = 2.f * (fy / c->image_extent[1]) - 1.f;
    float right = u * c->horz_half_dist;
    float up = -v * c->vert_half_dist;
    v3 dir = mk3(right, c->z_is_up ? 1.f : up, c->z_is_up ? up : -1.f);
    dir = div3s(dir, len3(dir));
    *o = xform_point(c->camera_to_world, mk3(0, 0, 0));
    *d = xform_vector(c->camera_to_world, dir);
}

/* The material's bump map, applied once per hit before the delta check and
 * the BSDF: check_for_delta_scattering_event (src/ref/delta_scattering.cpp:252-257)
 * applies it for the delta-capable materials and create_bsdf (src/ref/bsdf.cpp:631-714)
 * for the others; applying it twice gives the same shading frame.  Mix
 * materials have none (their sub-materials' bump maps are refused). */
static void apply_material_bump(const yar_flat_scene* s, shading_ctx* sc) {
    if (sc->material_type == YAR_MATERIAL_NULL || sc->material_type == YAR_MATERIAL_MIX) return;
    apply_bump_map(s, &s->materials[sc->material_index], sc);
}

/* check_for_delta_scattering_event / get_*_info, src/ref/delta_scattering.cpp:27-97, :252-324
 * (perfect reflector, perfect refractor, smooth glass; no nested dielectrics).  Returns 1 and the delta direction and attenuation for a delta
 * material, 2 for a delta material without a direction, 0 otherwise.  *kind: the
 * Delta_Scattering_Type of the event, 0 reflection, etaI_over_etaT (> 0)
 * transmission, -1 passthrough. */
static int delta_scattering(const yar_flat_scene* s, const shading_ctx* sc, float* u_ptr, v3* dir, col* atten,
                            float* bsdf_prob, float* kind) {
    const yar_material_desc* m = &s->materials[sc->material_index];
    *atten = mkc(1, 1, 1);
    *kind = 0.f;
    if (sc->material_type == YAR_MATERIAL_PBRT3_UBER) {
        /* get_pbrt_uber_info, src/ref/delta_scattering.cpp:102-150 */
        const float fp = *u_ptr * (float)m->component_count;
        const int k = (int)fp;
        const uint32_t comp = m->components[k];
        const float r = fp - (float)k;
        *u_ptr = r < 0.f ? 0.f : (ONE_MINUS_EPSILON < r ? ONE_MINUS_EPSILON : r);
        float delta_terms = 0.f;
        for (uint32_t c = 0; c < m->component_count; c++)
            if (m->components[c] >= YAR_UBER_DELTA_REFLECTION) delta_terms += 1.f;
        *bsdf_prob = 1.f - delta_terms / (float)m->component_count;
        if (comp == YAR_UBER_DELTA_REFLECTION) {
            const int enter = !sc->flipped;
            float fresnel = dielectric_fresnel(dot3(sc->normal, sc->wo),
                                               enter ? m->index_of_refraction : 1.f / m->index_of_refraction);
            *atten = mulcs(ldc(m->delta_reflectance), (float)m->component_count * fresnel);
            *dir = reflect3(sc->wo, sc->normal);
            return 1;
        }
        if (comp == YAR_UBER_OPACITY) {
            *atten = mulcs(subc(mkc(1, 1, 1), ldc(m->opacity)), (float)m->component_count);
            *dir = neg3(sc->wo);
            *kind = -1.f;
            return 1;
        }
        return 0;
    }
    if (sc->material_type == YAR_MATERIAL_MIX) {
        /* get_mix_info, src/ref/delta_scattering.cpp:154-189, with sub-materials that are
         * pure delta or have no delta event */
        const yar_material_desc* m1 = &s->materials[m->mix_materials[0]];
        const yar_material_desc* m2 = &s->materials[m->mix_materials[1]];
        const float amount = fminf_std(luminance(ldc(m->mix_amount)), 1.f);
        const int has1 = !is_pure_delta(m1->type), has2 = !is_pure_delta(m2->type);
        const yar_material_desc* pick;
        if (*u_ptr < amount) {
            *u_ptr /= amount;
            pick = m1;
        } else {
            *u_ptr = (*u_ptr - amount) / (1.f - amount);
            pick = m2;
        }
        int event = 0;
        float prob = 0.f;
        if (pick->type == YAR_MATERIAL_PERFECT_REFLECTOR) {
            *dir = reflect3(sc->wo, sc->normal);
            *atten = ldc(pick->reflectance);
            event = 1;
            prob = 1.f;
        } else if (pick->type == YAR_MATERIAL_PERFECT_REFRACTOR) {
            const float eta = !sc->flipped ? 1.f / pick->index_of_refraction : pick->index_of_refraction;
            event = refract3(sc->wo, sc->normal, eta, dir) ? 1 : 2;
            *kind = eta;
            prob = 1.f;
        }
        if (has1 && has2) prob *= pick == m1 ? amount : 1.f - amount;
        else prob = has1 ? 1.f - amount : amount;
        *bsdf_prob = 1.f - prob;
        return event;
    }
    const float u = *u_ptr;
    if (sc->material_type != YAR_MATERIAL_PERFECT_REFLECTOR && sc->material_type != YAR_MATERIAL_PERFECT_REFRACTOR &&
        sc->material_type != YAR_MATERIAL_GLASS)
        return 0;
    if (sc->material_type == YAR_MATERIAL_GLASS && m->u_roughness > 0.f) return 0;
    *bsdf_prob = 0.f;
    if (sc->material_type == YAR_MATERIAL_PERFECT_REFLECTOR) {
        *dir = reflect3(sc->wo, sc->normal);
        *atten = ldc(m->reflectance);
        return 1;
    }
    const int enter = !sc->flipped;
    if (sc->material_type == YAR_MATERIAL_PERFECT_REFRACTOR) {
        const float eta = enter ? 1.f / m->index_of_refraction : m->index_of_refraction;
        *kind = eta;
        /* Total internal reflection leaves the reference's direction at its
         * zero default (an ASSERT in debug builds); the zero-length ray finds
         * nothing and the path ends.  Reported here as 2: no delta ray. */
        if (!refract3(sc->wo, sc->normal, eta, dir)) {
            *dir = mk3(0, 0, 0);
            return 2;
        }
        return 1;
    }
    const float eta_t_over_i = enter ? m->index_of_refraction : 1.f / m->index_of_refraction;
    const float cos_i = dot3(sc->normal, sc->wo);
    const float fresnel = dielectric_fresnel(cos_i, eta_t_over_i);
    if (u < fresnel) {
        *dir = reflect3(sc->wo, sc->normal);
        *atten = m->reflectance_texture ? texture_reflectance(s, sc, m) : ldc(m->reflectance);
    } else {
        const float eta = 1.f / eta_t_over_i;
        *atten = mulcs(m->transmittance_texture ? texture_transmittance(s, sc, m) : ldc(m->transmittance), eta * eta);
        refract3(sc->wo, sc->normal, eta, dir);
        *kind = eta;
    }
    return 1;
}

/* get_emitted_radiance, src/ref/direct_lighting.cpp:386-413: rectangular lights
 * emit on both sides, triangle-mesh lights only on the side their normal faces. */
static int emitted_radiance(const yar_flat_scene* s, const shading_ctx* sc, col* le) {
    if (sc->light_type == YAR_LIGHT_DIFFUSE_RECTANGULAR) {
        *le = ldc(s->rect_lights[sc->light_index].emitted_radiance);
        return 1;
    }
    if (sc->light_type == YAR_LIGHT_DIFFUSE_SPHERE) {
        *le = ldc(s->sphere_lights[sc->light_index].emitted_radiance);
        return 1;
    }
    if (sc->light_type == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH && !sc->flipped) {
        *le = ldc(s->mesh_lights[sc->light_index].emitted_radiance);
        return 1;
    }
    return 0;
}

/* trace_path, src/ref/path_tracing.cpp:11-133 */
static int trace_path(const yar_flat_scene* s, const mesh_light_sampler* mesh_samplers, const env_sampler* env,
                      v3 ro, v3 rd, const v3 differential_dirs[2], sampler_view* sv, col* radiance) {
    const yar_render_config* cfg = &s->config;
    const int total_lights = (int)(s->delta_light_count + s->rect_light_count + s->sphere_light_count +
                                   s->mesh_light_count + (env->e ? 1 : 0) + s->other_light_count);
    col le;
    col coeff = mkc(1, 1, 1), L = mkc(0, 0, 0);
    int bounce = 0;
    int traced_by_delta_bounce = 0;
    hit_state h;
    shading_ctx sc;
    int hit = 0;
    for (;;) {
        if (!traced_by_delta_bounce) {
            hit = trace_closest(s, ro, rd, &h);
            if (hit < 0) return YAR_ERR_CAPACITY;
            if (hit) init_shading(s, rd, h.object, h.prim, h.b, &sc);
            /* the camera ray's differential rays (trace_ray at bounce 0, path_tracing.cpp:25) */
            if (hit && bounce == 0) uv_derivatives(&sc, ro, differential_dirs[0], ro, differential_dirs[1]);
            if (bounce == 0) {
                if (hit && emitted_radiance(s, &sc, &le)) L = addc(L, mulc(coeff, le));
                else if (!hit && env->e) L = addc(L, mulc(coeff, env_radiance(env, rd, 1)));
                if (cfg->max_light_bounces == 0) break;
            }
            if (!hit || sc.light_type != YAR_LIGHT_NULL) break;
        }
        traced_by_delta_bounce = 0;

        float u_scatter = next1d(sv);
        float u_light_index = next1d(sv);
        float u_scatter_next = next1d(sv);
        float ul0, ul1, ub0, ub1, un0, un1;
        next2d(sv, &ul0, &ul1);
        next2d(sv, &ub0, &ub1);
        next2d(sv, &un0, &un1);

        if (sc.material_type == YAR_MATERIAL_NULL) return YAR_ERR_UNSUPPORTED;
        /* Shading_Context::initialize_scattering (src/ref/shading_context.cpp:174-186) */
        v3 ddir;
        col datten;
        float bsdf_prob = 1.f; /* 1 - delta_layer_selection_probability */
        float delta_kind;
        apply_material_bump(s, &sc);
        const int delta = delta_scattering(s, &sc, &u_scatter, &ddir, &datten, &bsdf_prob, &delta_kind);
        if (delta == 2) break; /* perfect refractor at total internal reflection */
        bsdf_t f, f_sub[2];
        if (!delta || bsdf_prob != 0.f) {
            int rc = make_bsdf(s, &sc, &f, f_sub);
            if (rc != YAR_OK) return rc;
            /* estimate_direct_lighting_from_single_sample, src/ref/direct_lighting.cpp:522-578 */
            int light_index = (int)(u_light_index * (float)total_lights);
            /* point, spot, directional, rectangular, sphere, triangle-mesh, then the environment light */
            const int rect_first = (int)s->delta_light_count, sphere_first = rect_first + (int)s->rect_light_count;
            const int mesh_first = sphere_first + (int)s->sphere_light_count;
            const int env_first = mesh_first + (int)s->mesh_light_count;
            col one = light_index < rect_first ? direct_delta(s, &sc, &f, &s->delta_lights[light_index])
                      : light_index < sphere_first
                          ? direct_rect(s, &sc, &f, light_index - rect_first, ul0, ul1, ub0, ub1, u_scatter)
                      : light_index < mesh_first
                          ? direct_sphere(s, &sc, &f, light_index - sphere_first, ul0, ul1, ub0, ub1, u_scatter)
                      : light_index < env_first
                          ? direct_mesh(s, &sc, &f, &mesh_samplers[light_index - mesh_first], light_index - mesh_first,
                                        ul0, ul1, ub0, ub1, u_scatter)
                          : direct_env(s, &sc, &f, env, ul0, ul1, ub0, ub1, u_scatter);
            col direct = mulcs(one, (float)total_lights);
            L = addc(L, mulc(coeff, direct));
        }
        if (!delta) {
            bounce++;
            if (bounce == cfg->max_light_bounces) break;
            v3 wi = mk3(0, 0, 0);
            float pdf;
            col fv = bsdf_sample(&f, un0, un1, u_scatter_next, sc.wo, &wi, &pdf);
            if (blackc(fv)) break;
            coeff = mulc(coeff, mulcs(fv, fabsf(dot3(sc.normal, wi)) / (pdf * bsdf_prob)));
            ro = origin_for_direction(&sc, wi);
            rd = wi;
        } else {
            /* the delta ray is traced at once; light it reaches counts (path_tracing.cpp:76-107);
             * reflected and transmitted delta rays carry differential rays while the vertex
             * has dxdy derivatives, for max_differential_ray_specular_bounces bounces
             * (delta_scattering.cpp:283-322) */
            v3 diff[4];
            const int has_diff = delta_kind >= 0.f && sc.has_dxdy && bounce < MAX_DIFFERENTIAL_RAY_SPECULAR_BOUNCES;
            if (has_diff) specular_differentials(&sc, ddir, delta_kind, diff);
            ro = origin_for_direction(&sc, ddir);
            rd = ddir;
            hit = trace_closest(s, ro, rd, &h);
            if (hit < 0) return YAR_ERR_CAPACITY;
            if (hit) init_shading(s, rd, h.object, h.prim, h.b, &sc);
            if (hit && has_diff) uv_derivatives(&sc, diff[0], diff[1], diff[2], diff[3]);
            coeff = mulc(coeff, datten);
            if (hit && emitted_radiance(s, &sc, &le)) L = addc(L, mulc(coeff, le));
            else if (!hit && env->e) L = addc(L, mulc(coeff, env_radiance(env, rd, 1)));
            bounce++;
            if (bounce == cfg->max_light_bounces) break;
            if (!hit || sc.light_type != YAR_LIGHT_NULL) break;
            traced_by_delta_bounce = 1;
        }
        if (bounce >= cfg->russian_roulette_bounce_count_threshold) {
            float u_term = next1d(sv);
            float max_coeff = fmaxf_std(coeff.r, fmaxf_std(coeff.g, coeff.b));
            if (max_coeff < cfg->russian_roulette_threshold) {
                float p_term = fmaxf_std(0.05f, 1.f - max_coeff);
                if (u_term < p_term) break;
                coeff = mulcs(coeff, 1.f / (1.f - p_term));
            }
        }
    }
    *radiance = L;
    return YAR_OK;
}

/* ---------------- render_scene with the reference's tiles, merge order and variance */
#define TILE 64 /* src/ref/film.cpp:5 */

typedef struct film_px { float r, g, b, w; } film_px;

/* The direct-lighting algorithm's sample arrays of one pixel sample: per
 * rectangular light, then per sphere light, k x k 2D light samples, k x k 2D
 * BSDF samples and k x k 1D scattering samples
 * (src/ref/reference_renderer.cpp:101-128). */
typedef struct direct_arrays {
    const float* light2d[2];  /* [0] rectangular lights, [1] sphere lights: per light, k*k float2 */
    const float* bsdf2d[2];
    const float* scatter1d[2];
    const int* k[2];          /* array side per light */
    const size_t* offset[2];  /* per light, its first element in the arrays above */
} direct_arrays;

/* estimate_direct_lighting, src/ref/direct_lighting.cpp:415-520 (the delta ray's
 * hit adds its emission only, so only the camera hit reads derivatives) */
static int trace_direct(const yar_flat_scene* s, const env_sampler* env, v3 ro, v3 rd, const v3 differential_dirs[2],
                        const direct_arrays* da, oracle_pcg32* rng, col* radiance) {
    hit_state h;
    int hit = trace_closest(s, ro, rd, &h);
    if (hit < 0) return YAR_ERR_CAPACITY;
    if (!hit) {
        *radiance = env->e ? env_radiance(env, rd, 1) : mkc(0, 0, 0);
        return YAR_OK;
    }
    shading_ctx sc;
    init_shading(s, rd, h.object, h.prim, h.b, &sc);
    uv_derivatives(&sc, ro, differential_dirs[0], ro, differential_dirs[1]);
    float u_scatter = oracle_pcg32_float(rng); /* past the (empty) 1D budget */
    col L = mkc(0, 0, 0), le;
    v3 ddir;
    col datten;
    float bsdf_prob = 1.f;
    int delta = 0;
    if (sc.light_type == YAR_LIGHT_NULL) apply_material_bump(s, &sc);
    float delta_kind;
    if (sc.material_type != YAR_MATERIAL_NULL)
        delta = delta_scattering(s, &sc, &u_scatter, &ddir, &datten, &bsdf_prob, &delta_kind);
    if (sc.light_type != YAR_LIGHT_NULL) {
        if (emitted_radiance(s, &sc, &le)) L = le;
    } else if (sc.material_type != YAR_MATERIAL_NULL && (!delta || bsdf_prob != 0.f)) {
        bsdf_t f, f_sub[2];
        int rc = make_bsdf(s, &sc, &f, f_sub);
        if (rc != YAR_OK) return rc;
        for (uint32_t i = 0; i < s->delta_light_count; i++) /* point lights */
            if (s->delta_lights[i].type == YAR_LIGHT_POINT) L = addc(L, direct_delta(s, &sc, &f, &s->delta_lights[i]));
        for (uint32_t i = 0; i < s->delta_light_count; i++) /* directional lights */
            if (s->delta_lights[i].type == YAR_LIGHT_DIRECTIONAL)
                L = addc(L, direct_delta(s, &sc, &f, &s->delta_lights[i]));
        for (int kind = 0; kind < 2; kind++) {
            const uint32_t n = kind == 0 ? s->rect_light_count : s->sphere_light_count;
            for (uint32_t i = 0; i < n; i++) {
                const int k = da->k[kind][i], count = k * k;
                const size_t o = da->offset[kind][i];
                col L2 = mkc(0, 0, 0);
                for (int j = 0; j < count; j++) {
                    const float* ul = da->light2d[kind] + 2 * (o + j);
                    const float* ub = da->bsdf2d[kind] + 2 * (o + j);
                    const float us = da->scatter1d[kind][o + j];
                    L2 = addc(L2, kind == 0 ? direct_rect(s, &sc, &f, (int)i, ul[0], ul[1], ub[0], ub[1], us)
                                            : direct_sphere(s, &sc, &f, (int)i, ul[0], ul[1], ub[0], ub[1], us));
                }
                L = addc(L, mulcs(L2, 1.f / (float)count)); /* ColorRGB::operator/= multiplies by 1/v */
            }
        }
        if (env->e) {
            col L2 = mkc(0, 0, 0);
            for (int j = 0; j < env->e->sample_count; j++) {
                float ul0 = oracle_pcg32_float(rng), ul1 = oracle_pcg32_float(rng);
                float ub0 = oracle_pcg32_float(rng), ub1 = oracle_pcg32_float(rng);
                float us = oracle_pcg32_float(rng);
                L2 = addc(L2, direct_env(s, &sc, &f, env, ul0, ul1, ub0, ub1, us));
            }
            L = addc(L, mulcs(L2, 1.f / (float)env->e->sample_count));
        }
    }
    if (delta == 1) {
        v3 o = origin_for_direction(&sc, ddir);
        hit = trace_closest(s, o, ddir, &h);
        if (hit < 0) return YAR_ERR_CAPACITY;
        col emitted = mkc(0, 0, 0);
        if (hit) {
            init_shading(s, ddir, h.object, h.prim, h.b, &sc);
            if (emitted_radiance(s, &sc, &le)) emitted = le;
        } else if (env->e) {
            emitted = env_radiance(env, ddir, 1);
        }
        L = addc(L, mulc(datten, emitted));
    }
    *radiance = L;
    return YAR_OK;
}

typedef struct render_job {
    const yar_flat_scene* s;
    int x0, y0, x1, y1;         /* render region */
    int sx0, sy0, sx1, sy1;     /* sample region */
    int tiles_x, tiles_y;
    int row_begin, row_end;     /* rows of the render region that must be exact */
    film_px** tile_pixels;      /* per tile: pixel bounds size */
    int* tile_bounds;           /* per tile: px0, py0, px1, py1 */
    double* tile_variance;
    int next_tile;
    mesh_light_sampler* mesh_samplers;
    env_sampler env;
    pthread_mutex_t lock;
    int status;
} render_job;

static void tile_bounds(const render_job* J, int t, int* sb, int* pb) {
    int tx = t % J->tiles_x, ty = t / J->tiles_x;
    const float radius = J->s->config.pixel_filter_radius;
    sb[0] = J->sx0 + tx * TILE;
    sb[1] = J->sy0 + ty * TILE;
    sb[2] = sb[0] + TILE < J->sx1 ? sb[0] + TILE : J->sx1;
    sb[3] = sb[1] + TILE < J->sy1 ? sb[1] + TILE : J->sy1;
    int a = (int)ceilf((float)sb[0] - radius - 0.5f), b = (int)ceilf((float)sb[1] - radius - 0.5f);
    int c = (int)floorf((float)sb[2] + radius - 0.5f) + 1, d = (int)floorf((float)sb[3] + radius - 0.5f) + 1;
    pb[0] = a > J->x0 ? a : J->x0;
    pb[1] = b > J->y0 ? b : J->y0;
    pb[2] = c < J->x1 ? c : J->x1;
    pb[3] = d < J->y1 ? d : J->y1;
}

static int render_tile(render_job* J, int t) {
    const yar_flat_scene* s = J->s;
    const yar_render_config* cfg = &s->config;
    int sb[4], pb[4];
    tile_bounds(J, t, sb, pb);
    memcpy(&J->tile_bounds[4 * t], pb, sizeof(pb));
    const int pw = pb[2] - pb[0], ph = pb[3] - pb[1];
    film_px* px = (film_px*)calloc((size_t)(pw > 0 ? pw : 1) * (ph > 0 ? ph : 1), sizeof(film_px));
    if (!px) return YAR_ERR_NOMEM;
    J->tile_pixels[t] = px;
    const int nx = cfg->x_pixel_sample_count, ny = cfg->y_pixel_sample_count, spp = nx * ny;
    const int direct = cfg->rendering_algorithm == 0;
    const int maxb = cfg->max_light_bounces < 10 ? cfg->max_light_bounces : 10;
    const int n1d = direct ? 0 : maxb * 4, n2d = direct ? 0 : maxb * 3; /* src/ref/reference_renderer.cpp:87-99 */
    /* direct lighting: k x k sample arrays per rectangular and per sphere light */
    int* dk[2] = {NULL, NULL};
    size_t* doff[2] = {NULL, NULL};
    size_t dper[2] = {0, 0}; /* array elements per pixel sample */
    float* dbuf[2][3] = {{NULL, NULL, NULL}, {NULL, NULL, NULL}};
    if (direct) {
        for (int kind = 0; kind < 2; kind++) {
            const uint32_t n = kind == 0 ? s->rect_light_count : s->sphere_light_count;
            dk[kind] = (int*)calloc(n + 1, sizeof(int));
            doff[kind] = (size_t*)calloc(n + 1, sizeof(size_t));
            for (uint32_t i = 0; i < n; i++) {
                const int sc = kind == 0 ? s->rect_lights[i].sample_count : s->sphere_lights[i].sample_count;
                dk[kind][i] = (int)ceil(sqrt((double)sc));
                doff[kind][i] = dper[kind];
                dper[kind] += (size_t)dk[kind][i] * dk[kind][i];
            }
            for (int b = 0; b < 3; b++)
                dbuf[kind][b] = (float*)malloc(sizeof(float) * (b < 2 ? 2 : 1) * (dper[kind] * spp + 1));
        }
    }
    float* image = (float*)malloc(sizeof(float) * 2 * spp);
    float* s1d = (float*)malloc(sizeof(float) * ((size_t)spp * n1d + 1));
    float* s2d = (float*)malloc(sizeof(float) * (2 * (size_t)spp * n2d + 1));
    const float radius = cfg->pixel_filter_radius;
    const int support = (int)ceilf(radius + 0.5f);  /* sample rows that reach a requested row */
    double var_acc = 0.0;
    int rc = YAR_OK;
    for (int y = sb[1]; y < sb[3] && rc == YAR_OK; y++) {
        if (y < J->row_begin - support || y >= J->row_end + support) continue;  /* outside the rows requested */
        for (int x = sb[0]; x < sb[2] && rc == YAR_OK; x++) {
            uint32_t stream = ((uint32_t)x & 0xffffu) | ((uint32_t)y << 16);
            stream += (uint32_t)cfg->rng_seed_offset;
            oracle_pcg32 rng;
            oracle_pcg32_seed(&rng, 0, stream);
            /* next_pixel with the live rng so draws beyond the budget continue its stream */
            {
                const float dx = 1.f / (float)nx, dy = 1.f / (float)ny;
                float* o = image;
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++) {
                        float a = ((float)i + oracle_pcg32_float(&rng)) * dx;
                        *o++ = a < ONE_MINUS_EPSILON ? a : ONE_MINUS_EPSILON;
                        float b = ((float)j + oracle_pcg32_float(&rng)) * dy;
                        *o++ = b < ONE_MINUS_EPSILON ? b : ONE_MINUS_EPSILON;
                    }
                float tmp[2 * 4096];
                if (spp > 4096) { rc = YAR_ERR_UNSUPPORTED; break; }
                for (int i = 0; i < n1d; i++) {
                    stratified_1d(&rng, spp, tmp);
                    shuffle(tmp, spp, 1, &rng);
                    for (int k = 0; k < spp; k++) s1d[k * n1d + i] = tmp[k];
                }
                for (int i = 0; i < n2d; i++) {
                    stratified_2d(&rng, nx, ny, tmp);
                    shuffle(tmp, spp, 2, &rng);
                    for (int k = 0; k < spp; k++) {
                        s2d[2 * (k * n2d + i)] = tmp[2 * k];
                        s2d[2 * (k * n2d + i) + 1] = tmp[2 * k + 1];
                    }
                }
                /* Stratified_Pixel_Sampler::next_pixel's array samples (src/ref/pixel_sampling.cpp:88-141):
                 * the 2D arrays in registration order (per light: light, BSDF), then the 1D arrays */
                for (int pass = 0; pass < 2 && direct && rc == YAR_OK; pass++) {
                    for (int kind = 0; kind < 2; kind++) {
                        const uint32_t n = kind == 0 ? s->rect_light_count : s->sphere_light_count;
                        for (uint32_t li = 0; li < n; li++) {
                            const int k = dk[kind][li], count = k * k;
                            float* grids = (float*)malloc(sizeof(float) * 2 * (size_t)count * spp);
                            for (int which = 0; which < (pass == 0 ? 2 : 1); which++) {
                                for (int g = 0; g < count; g++) {
                                    float* grid = grids + (pass == 0 ? 2 : 1) * (size_t)g * spp;
                                    if (pass == 0) stratified_2d(&rng, nx, ny, grid);
                                    else stratified_1d(&rng, spp, grid);
                                    shuffle(grid, spp, pass == 0 ? 2 : 1, &rng);
                                }
                                float* out = dbuf[kind][pass == 0 ? which : 2];
                                const float dxa = pass == 0 ? 1.f / (float)k : 1.f / (float)count;
                                for (int i = 0; i < spp; i++)
                                    for (int g = 0; g < count; g++) {
                                        const size_t e = (size_t)i * dper[kind] + doff[kind][li] + g;
                                        if (pass == 0) {
                                            const float* u = grids + 2 * ((size_t)g * spp + i);
                                            const int gx = g % k, gy = g / k;
                                            float sx = ((float)gx + u[0]) * dxa, sy = ((float)gy + u[1]) * dxa;
                                            out[2 * e] = sx < ONE_MINUS_EPSILON ? sx : ONE_MINUS_EPSILON;
                                            out[2 * e + 1] = sy < ONE_MINUS_EPSILON ? sy : ONE_MINUS_EPSILON;
                                        } else {
                                            float v = ((float)g + grids[(size_t)g * spp + i]) * dxa;
                                            out[e] = v < ONE_MINUS_EPSILON ? v : ONE_MINUS_EPSILON;
                                        }
                                    }
                            }
                            free(grids);
                        }
                    }
                }
            }
            double lsum = 0.0, lsq = 0.0;
            for (int k = 0; k < spp; k++) {
                float fx = (float)x + image[2 * k], fy = (float)y + image[2 * k + 1];
                v3 o, d;
                camera_ray(&s->camera, fx, fy, &o, &d);
                sampler_view sv = {s1d + (size_t)k * n1d, s2d + 2 * (size_t)k * n2d, n1d, n2d, 0, 0, &rng};
                col radiance;
                /* differential rays one pixel over, scaled to the sample's footprint
                 * (src/ref/reference_renderer.cpp:367-378) */
                v3 dd[2], ox;
                camera_ray(&s->camera, fx + 1.f, fy, &ox, &dd[0]);
                camera_ray(&s->camera, fx, fy + 1.f, &ox, &dd[1]);
                const float dscale = 1.f / sqrtf((float)spp);
                for (int q = 0; q < 2; q++) {
                    dd[q] = add3(d, mul3s(sub3(dd[q], d), dscale));
                    dd[q] = div3s(dd[q], len3(dd[q]));
                }
                if (direct) {
                    direct_arrays da;
                    for (int kind = 0; kind < 2; kind++) {
                        da.light2d[kind] = dbuf[kind][0] + 2 * (size_t)k * dper[kind];
                        da.bsdf2d[kind] = dbuf[kind][1] + 2 * (size_t)k * dper[kind];
                        da.scatter1d[kind] = dbuf[kind][2] + (size_t)k * dper[kind];
                        da.k[kind] = dk[kind];
                        da.offset[kind] = doff[kind];
                    }
                    rc = trace_direct(s, &J->env, o, d, dd, &da, &rng, &radiance);
                } else {
                    rc = trace_path(s, J->mesh_samplers, &J->env, o, d, dd, &sv, &radiance);
                }
                if (rc != YAR_OK) break;
                float limit = cfg->max_rgb_component_value_of_film_sample;
                float mc = fmaxf_std(radiance.r, fmaxf_std(radiance.g, radiance.b));
                if (mc > limit) radiance = mulcs(radiance, limit / mc);
                if (cfg->film_radiance_scale != 1.f) radiance = mulcs(radiance, cfg->film_radiance_scale);
                /* Film_Tile::add_sample, src/ref/film.cpp:27-50 */
                int rx0 = (int)ceilf(fx - radius - 0.5f), ry0 = (int)ceilf(fy - radius - 0.5f);
                int rx1 = (int)floorf(fx + radius - 0.5f) + 1, ry1 = (int)floorf(fy + radius - 0.5f) + 1;
                if (rx0 < pb[0]) rx0 = pb[0];
                if (ry0 < pb[1]) ry0 = pb[1];
                if (rx1 > pb[2]) rx1 = pb[2];
                if (ry1 > pb[3]) ry1 = pb[3];
                for (int yy = ry0; yy < ry1; yy++)
                    for (int xx = rx0; xx < rx1; xx++) {
                        film_px* p = &px[(yy - pb[1]) * pw + (xx - pb[0])];
                        const float w = film_filter_weight(cfg, fx - ((float)xx + 0.5f), fy - ((float)yy + 0.5f));
                        p->r += w * radiance.r;
                        p->g += w * radiance.g;
                        p->b += w * radiance.b;
                        p->w += w;
                    }
                float lum = 0.2126729f * radiance.r + 0.7151522f * radiance.g + 0.0721750f * radiance.b;
                lsum += lum;
                lsq += lum * lum;
            }
            if (spp > 1) {
                double pv = (lsq - lsum * lsum / spp) / (spp * (spp - 1));
                var_acc += pv > 0.0 ? pv : 0.0;
            }
        }
    }
    free(image);
    free(s1d);
    free(s2d);
    for (int kind = 0; kind < 2; kind++) {
        free(dk[kind]);
        free(doff[kind]);
        for (int b = 0; b < 3; b++) free(dbuf[kind][b]);
    }
    J->tile_variance[t] = var_acc;
    return rc;
}

static void* render_worker(void* arg) {
    render_job* J = (render_job*)arg;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int t = J->next_tile++;
        int stop = J->status != YAR_OK;
        pthread_mutex_unlock(&J->lock);
        if (stop || t >= J->tiles_x * J->tiles_y) break;
        int rc = render_tile(J, t);
        if (rc != YAR_OK) {
            pthread_mutex_lock(&J->lock);
            J->status = rc;
            pthread_mutex_unlock(&J->lock);
        }
    }
    return NULL;
}

int oracle_render_trig(const yar_flat_scene* s, float* rgb, double* variance, int32_t row_begin, int32_t row_end,
                       int32_t thread_count, int32_t correctly_rounded_trig) {
    g_correctly_rounded_trig = correctly_rounded_trig != 0;
    return oracle_render(s, rgb, variance, row_begin, row_end, thread_count);
}

int oracle_render(const yar_flat_scene* s, float* rgb, double* variance, int32_t row_begin, int32_t row_end,
                  int32_t thread_count) {
    const yar_render_config* cfg = &s->config;
    if ((cfg->rendering_algorithm != 0 && cfg->rendering_algorithm != 1) || cfg->pixel_filter_type < 0 ||
        cfg->pixel_filter_type > 2)
        return YAR_ERR_UNSUPPORTED;
    for (uint32_t i = 0; i < s->material_count; i++) {
        uint32_t t = s->materials[i].type;
        if (t != YAR_MATERIAL_DIFFUSE && t != YAR_MATERIAL_METAL && t != YAR_MATERIAL_GLASS &&
            t != YAR_MATERIAL_PLASTIC && t != YAR_MATERIAL_COATED_DIFFUSE && t != YAR_MATERIAL_PERFECT_REFLECTOR &&
            t != YAR_MATERIAL_PERFECT_REFRACTOR && t != YAR_MATERIAL_DIFFUSE_TRANSMISSION &&
            t != YAR_MATERIAL_PBRT3_TRANSLUCENT && t != YAR_MATERIAL_PBRT3_UBER && t != YAR_MATERIAL_MIX &&
            t != YAR_MATERIAL_PBRT3_FOURIER)
            return YAR_ERR_UNSUPPORTED;
        if (t == YAR_MATERIAL_PBRT3_FOURIER) {
            /* the tables the reference's evaluation accepts: one or three channels,
             * reflection only (eta 1), increasing nodes ending at or above 1 (so
             * lower_bound finds every clamped cosine), series inside the coefficients */
            const uint32_t ti = s->materials[i].fourier_table;
            if (ti == 0 || ti > s->fourier_count) return YAR_ERR_INVALID;
            const yar_fourier_desc* ft = &s->fourier_tables[ti - 1];
            const uint64_t pairs = (uint64_t)ft->node_count * ft->node_count;
            if (ft->node_count == 0 || ft->nodes + ft->node_count > s->fourier_float_count ||
                ft->coeffs + ft->coeff_count > s->fourier_float_count || ft->series + 2 * pairs > s->fourier_uint_count)
                return YAR_ERR_INVALID;
            if ((ft->channel_count != 1 && ft->channel_count != 3) || ft->eta != 1.f) return YAR_ERR_UNSUPPORTED;
            const float* nodes = s->fourier_floats + ft->nodes;
            for (uint32_t k = 1; k < ft->node_count; k++)
                if (!(nodes[k - 1] <= nodes[k])) return YAR_ERR_INVALID;
            if (!(nodes[ft->node_count - 1] >= 1.f)) return YAR_ERR_UNSUPPORTED;
            for (uint64_t k = 0; k < pairs; k++) {
                const uint64_t off = s->fourier_uints[ft->series + 2 * k], cnt = s->fourier_uints[ft->series + 2 * k + 1];
                if (off + cnt * ft->channel_count > ft->coeff_count) return YAR_ERR_INVALID;
            }
        }
    }
    if (s->other_light_count) return YAR_ERR_UNSUPPORTED;
    /* image textures: the reflectance of diffuse, plastic, coated diffuse, glass
     * and diffuse transmission, the transmittance of glass and diffuse
     * transmission, and bump maps, with camera-ray differentials and the
     * specular differential rays of delta bounces.  A constant bump height
     * needs no differentials. */
    for (uint32_t i = 0; i < s->material_count; i++) {
        const yar_material_desc* m = &s->materials[i];
        if (m->other_textured_parameters) return YAR_ERR_UNSUPPORTED;
        const int reflectance_slot = m->type == YAR_MATERIAL_DIFFUSE || m->type == YAR_MATERIAL_PLASTIC ||
                                     m->type == YAR_MATERIAL_COATED_DIFFUSE || m->type == YAR_MATERIAL_GLASS ||
                                     m->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION;
        const int transmittance_slot = m->type == YAR_MATERIAL_GLASS || m->type == YAR_MATERIAL_DIFFUSE_TRANSMISSION;
        if ((m->reflectance_texture && !reflectance_slot) || (m->transmittance_texture && !transmittance_slot) ||
            m->bump > 2 || (m->bump && m->type == YAR_MATERIAL_MIX))
            return YAR_ERR_UNSUPPORTED;
        const uint32_t used[3] = {m->reflectance_texture, m->transmittance_texture, m->bump == 2 ? m->bump_texture : 0u};
        for (int k = 0; k < 3; k++) {
            if (!used[k]) continue;
            if (used[k] > s->texture_count) return YAR_ERR_INVALID;
            const yar_texture_desc* t = &s->textures[used[k] - 1];
            if (t->mip_count == 0 || t->first_mip + t->mip_count > s->texture_mip_count) return YAR_ERR_INVALID;
        }
        if (m->bump == 2 && !used[2]) return YAR_ERR_INVALID;
    }
    init_ewa_weights();
    for (uint32_t i = 0; i < s->material_count; i++) {
        const yar_material_desc* m = &s->materials[i];
        if (m->type == YAR_MATERIAL_MIX) {
            /* sub-materials: pure delta, or BSDF materials without a delta event; not both delta */
            int delta_subs = 0;
            for (int k = 0; k < 2; k++) {
                const int32_t si = m->mix_materials[k];
                if (si < 0 || (uint32_t)si >= s->material_count) return YAR_ERR_INVALID;
                const yar_material_desc* sm = &s->materials[si];
                if (sm->type == YAR_MATERIAL_MIX || sm->type == YAR_MATERIAL_PBRT3_UBER ||
                    (sm->type == YAR_MATERIAL_GLASS && !(sm->u_roughness > 0.f)) || sm->bump ||
                    sm->type == YAR_MATERIAL_PBRT3_FOURIER)
                    return YAR_ERR_UNSUPPORTED;
                delta_subs += is_pure_delta(sm->type);
            }
            if (delta_subs == 2) return YAR_ERR_UNSUPPORTED;
            continue;
        }
        if (m->type != YAR_MATERIAL_PBRT3_UBER) continue;
        if (m->component_count < 1 || m->component_count > 5) return YAR_ERR_UNSUPPORTED;
        for (uint32_t k = 0; k < m->component_count; k++)
            if (m->components[k] > YAR_UBER_OPACITY || m->components[k] == YAR_UBER_DELTA_TRANSMISSION)
                return YAR_ERR_UNSUPPORTED;
    }
    for (uint32_t i = 0; i < s->delta_light_count; i++) {
        uint32_t t = s->delta_lights[i].type;
        if (t > YAR_LIGHT_DIRECTIONAL || (i > 0 && t < s->delta_lights[i - 1].type)) return YAR_ERR_INVALID;
    }
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s;
    J.x0 = cfg->render_region[0];
    J.y0 = cfg->render_region[1];
    J.x1 = cfg->render_region[2];
    J.y1 = cfg->render_region[3];
    const float radius = cfg->pixel_filter_radius;
    J.sx0 = (int)floorf((float)J.x0 + 0.5f - radius);
    J.sy0 = (int)floorf((float)J.y0 + 0.5f - radius);
    J.sx1 = (int)ceilf((float)(J.x1 - 1) + 0.5f + radius);
    J.sy1 = (int)ceilf((float)(J.y1 - 1) + 0.5f + radius);
    J.tiles_x = (J.sx1 - J.sx0 + TILE - 1) / TILE;
    J.tiles_y = (J.sy1 - J.sy0 + TILE - 1) / TILE;
    J.row_begin = row_begin + J.y0;
    J.row_end = row_end + J.y0;
    const int nt = J.tiles_x * J.tiles_y;
    J.tile_pixels = (film_px**)calloc(nt, sizeof(film_px*));
    J.tile_bounds = (int*)calloc(4 * (size_t)nt, sizeof(int));
    J.tile_variance = (double*)calloc(nt, sizeof(double));
    int ms_rc = build_mesh_samplers(s, &J.mesh_samplers);
    if (ms_rc == YAR_OK) {
        ms_rc = build_env_sampler(s, &J.env);
        if (ms_rc != YAR_OK) free_mesh_samplers(J.mesh_samplers, s->mesh_light_count);
    }
    if (ms_rc != YAR_OK) {
        free(J.tile_pixels);
        free(J.tile_bounds);
        free(J.tile_variance);
        return ms_rc;
    }
    pthread_mutex_init(&J.lock, NULL);
    J.status = YAR_OK;
    int nthreads = thread_count > 0 ? thread_count : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, render_worker, &J);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
    int rc = J.status;
    if (rc == YAR_OK) {
        /* merge tiles in index order, then resolve (src/ref/film.cpp:88-120) */
        const int W = J.x1 - J.x0, H = J.y1 - J.y0;
        film_px* film = (film_px*)calloc((size_t)W * H, sizeof(film_px));
        for (int t = 0; t < nt; t++) {
            const int* pb = &J.tile_bounds[4 * t];
            const int pw = pb[2] - pb[0];
            for (int y = pb[1]; y < pb[3]; y++)
                for (int x = pb[0]; x < pb[2]; x++) {
                    film_px* f = &film[(y - J.y0) * W + (x - J.x0)];
                    const film_px* p = &J.tile_pixels[t][(y - pb[1]) * pw + (x - pb[0])];
                    f->r += p->r;
                    f->g += p->g;
                    f->b += p->b;
                    f->w += p->w;
                }
        }
        for (int i = 0; i < W * H; i++) {
            col c = mkc(0, 0, 0);
            if (film[i].w != 0.f) c = mulcs(mkc(film[i].r, film[i].g, film[i].b), 1.f / film[i].w);
            rgb[3 * i + 0] = fmaxf_std(0.f, c.r);
            rgb[3 * i + 1] = fmaxf_std(0.f, c.g);
            rgb[3 * i + 2] = fmaxf_std(0.f, c.b);
        }
        free(film);
        const int spp = cfg->x_pixel_sample_count * cfg->y_pixel_sample_count;
        if (variance && spp > 1) {
            double acc = 0.0;
            int64_t count = 0;
            for (int t = 0; t < nt; t++) {
                int sb[4], pb[4];
                acc += J.tile_variance[t];
                tile_bounds(&J, t, sb, pb);
                count += (int64_t)(sb[2] - sb[0]) * (sb[3] - sb[1]);
            }
            *variance = acc / (double)count;
        }
    }
    for (int t = 0; t < nt; t++) free(J.tile_pixels[t]);
    free(J.tile_pixels);
    free(J.tile_bounds);
    free(J.tile_variance);
    free_mesh_samplers(J.mesh_samplers, s->mesh_light_count);
    free_env_sampler(&J.env);
    pthread_mutex_destroy(&J.lock);
    return rc;
}
