// device_scene.cuh - HBM layout of an uploaded scene and the two-level kd-tree
// traversal used by the extend (closest-hit) and shadow (any-hit) kernels.
//
// Layout (all arrays 16-byte aligned, read with 8/16-byte vector loads):
//   scene_nodes  uint2[]   scene kd-tree over objects, KdNode words unchanged
//   mesh_nodes   uint2[]   all mesh kd-trees concatenated; a mesh's child
//                          indices are local, so the traversal adds the
//                          mesh's node_offset (one IADD per fetch)
//   objects      float4[6] per object: rows of world_to_object (3),
//                          mesh bounds min (.w = node_offset bits),
//                          mesh bounds max (.w = triangle_offset bits),
//                          {mesh index, visibility, -, -} as int bits
//   tris         float4[3] per triangle: the three vertices gathered from
//                          the index buffer (48 B, the same bytes as 12 B of
//                          indices + 36 B of positions but no dependent load);
//                          v0.w != 0 marks a degenerate triangle, which the
//                          reference rejects after the test (kdtree.cpp:27-29)
//
// Arithmetic follows the reference operation by operation (the translation
// unit is compiled with -fmad=false and IEEE division), so hit triangle ids,
// t and barycentrics are bit-identical to KdTree::intersect.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace yar {

constexpr int kMaxTraversalDepth = 40;  // src/ref/kdtree.cpp:10

struct Device_Scene {
    const uint2* scene_nodes = nullptr;
    const uint2* mesh_nodes = nullptr;
    const float4* objects = nullptr;
    const float4* tris = nullptr;
    float scene_bounds[6] = {0, 0, 0, 0, 0, 0};
    uint32_t object_count = 0;
};

struct Hit {
    float t;
    uint32_t prim;
    uint32_t object;
    float b0, b1, b2;
};

__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }

// Bounding_Box::intersect_by_ray_without_NaNs, src/lib/bounding_box.h:63-85
__device__ __forceinline__ bool clip_ray(const float mn[3], const float mx[3], const float o[3], const float d[3],
                                         float& t_min, float& t_max) {
    float t0 = 0.f, t1 = __int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (d[i] != 0.f) {
            const float inv = 1.f / d[i];
            float s0 = (mn[i] - o[i]) * inv;
            float s1 = (mx[i] - o[i]) * inv;
            if (inv < 0.f) { const float tmp = s0; s0 = s1; s1 = tmp; }
            t0 = s0 > t0 ? s0 : t0;
            t1 = s1 < t1 ? s1 : t1;
            if (t0 > t1) return false;
        } else if (o[i] < mn[i] || o[i] > mx[i]) {
            return false;
        }
    }
    t_min = t0;
    t_max = t1;
    return true;
}

// intersect_triangle_watertight, src/ref/intersection.cpp:53-113.
// Returns +inf when there is no intersection.
__device__ __forceinline__ float watertight(const float o[3], const float d[3], int kx, int ky, int kz, float sx,
                                            float sy, float sz, const float4 v0, const float4 v1, const float4 v2,
                                            float& b0, float& b1, float& b2) {
    const float p0[3] = {v0.x, v0.y, v0.z};
    const float p1[3] = {v1.x, v1.y, v1.z};
    const float p2[3] = {v2.x, v2.y, v2.z};
    const float p0x = p0[kx] - o[kx], p0y = p0[ky] - o[ky], p0z = p0[kz] - o[kz];
    const float p1x = p1[kx] - o[kx], p1y = p1[ky] - o[ky], p1z = p1[kz] - o[kz];
    const float p2x = p2[kx] - o[kx], p2y = p2[ky] - o[ky], p2z = p2[kz] - o[kz];
    const float x0 = p0x + sx * p0z;
    const float y0 = p0y + sy * p0z;
    const float x1 = p1x + sx * p1z;
    const float y1 = p1y + sy * p1z;
    const float x2 = p2x + sx * p2z;
    const float y2 = p2y + sy * p2z;
    float e0 = x1 * y2 - y1 * x2;
    float e1 = x2 * y0 - y2 * x0;
    float e2 = x0 * y1 - y0 * x1;
    if (e0 == 0.f || e1 == 0.f || e2 == 0.f) {
        e0 = (float)((double)x1 * (double)y2 - (double)y1 * (double)x2);
        e1 = (float)((double)x2 * (double)y0 - (double)y2 * (double)x0);
        e2 = (float)((double)x0 * (double)y1 - (double)y0 * (double)x1);
    }
    const float inf = __int_as_float(0x7f800000);
    if ((e0 < 0.f || e1 < 0.f || e2 < 0.f) && (e0 > 0.f || e1 > 0.f || e2 > 0.f)) return inf;
    const float det = e0 + e1 + e2;
    if (det == 0.f) return inf;
    const float z0 = sz * p0z;
    const float z1 = sz * p1z;
    const float z2 = sz * p2z;
    const float t_scaled = e0 * z0 + e1 * z1 + e2 * z2;
    if ((__float_as_uint(det) ^ __float_as_uint(t_scaled)) >> 31) return inf;
    const float inv_det = 1.f / det;
    const float t = inv_det * t_scaled;
    b0 = e0 * inv_det;
    b1 = e1 * inv_det;
    b2 = e2 * inv_det;
    return t;
}

struct Stack_Entry {
    uint32_t node;
    float t_max;
};

// One descent step, src/ref/kdtree.cpp:254-298 (closest) and :361-406 (any).
// Returns false on stack overflow.
__device__ __forceinline__ bool descend(uint2 n, uint32_t& node, const float o[3], const float d[3],
                                        const float inv[3], float& t_min, float& t_max, Stack_Entry* stack,
                                        int& sp) {
    const int axis = (int)(n.x & 3u);
    const float dist = u2f(n.y) - o[axis];
    const uint32_t below_child = node + 1;
    const uint32_t above_child = n.x >> 2;
    if (dist != 0.f) {
        const bool below_first = dist > 0.f;
        const uint32_t first_child = below_first ? below_child : above_child;
        const uint32_t second_child = below_first ? above_child : below_child;
        const float t_split = dist * inv[axis];
        if (t_split > t_max || t_split < 0.f) {
            node = first_child;
        } else if (t_split < t_min) {
            node = second_child;
        } else {
            if (sp >= kMaxTraversalDepth) return false;
            stack[sp].node = second_child;
            stack[sp].t_max = t_max;
            sp++;
            node = first_child;
            t_max = t_split;
        }
    } else {
        node = (d[axis] > 0.f) ? above_child : below_child;
    }
    return true;
}

struct Object_Record {
    float m[12];
    float bmin[3];
    float bmax[3];
    uint32_t node_offset;
    uint32_t tri_offset;
    int32_t visibility;
};

__device__ __forceinline__ Object_Record load_object(const float4* objects, uint32_t index) {
    const float4* p = objects + 6 * (size_t)index;
    const float4 r0 = __ldg(p + 0), r1 = __ldg(p + 1), r2 = __ldg(p + 2);
    const float4 lo = __ldg(p + 3), hi = __ldg(p + 4), info = __ldg(p + 5);
    Object_Record r;
    r.m[0] = r0.x; r.m[1] = r0.y; r.m[2] = r0.z; r.m[3] = r0.w;
    r.m[4] = r1.x; r.m[5] = r1.y; r.m[6] = r1.z; r.m[7] = r1.w;
    r.m[8] = r2.x; r.m[9] = r2.y; r.m[10] = r2.z; r.m[11] = r2.w;
    r.bmin[0] = lo.x; r.bmin[1] = lo.y; r.bmin[2] = lo.z;
    r.bmax[0] = hi.x; r.bmax[1] = hi.y; r.bmax[2] = hi.z;
    r.node_offset = __float_as_uint(lo.w);
    r.tri_offset = __float_as_uint(hi.w);
    r.visibility = __float_as_int(info.y);
    return r;
}

// transform_ray, src/lib/matrix.cpp:368-389: ((a*x + b*y) + c*z) + w
__device__ __forceinline__ void transform_ray(const float m[12], const float o[3], const float d[3], float oo[3],
                                              float od[3]) {
#pragma unroll
    for (int r = 0; r < 3; r++) {
        oo[r] = m[4 * r + 0] * o[0] + m[4 * r + 1] * o[1] + m[4 * r + 2] * o[2] + m[4 * r + 3];
        od[r] = m[4 * r + 0] * d[0] + m[4 * r + 1] * d[1] + m[4 * r + 2] * d[2];
    }
}

// KdTree::intersect (closest) or intersect_any (ANY) over one mesh tree with
// the triangle leaf callbacks (src/ref/kdtree.cpp:12-79, :219-439).
// Closest: updates hit, returns 1 if hit.t decreased, 0 otherwise.
// Any: returns 1 when an occluder in [0, ray_tmax) was found.
// Returns -1 on traversal-stack overflow.
template <bool ANY>
__device__ __forceinline__ int mesh_traverse(const Device_Scene& s, const Object_Record& obj, const float o[3],
                                             const float d[3], float ray_tmax, Hit& hit) {
    float t_min, t_max;
    if (!clip_ray(obj.bmin, obj.bmax, o, d, t_min, t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    // watertight-test setup depends only on the ray (src/ref/intersection.cpp:55-62)
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    const int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    const int kx = (kz == 2 ? 0 : kz + 1);
    const int ky = (kz == 0 ? 2 : kz - 1);
    const float sx = -d[kx] / d[kz];
    const float sy = -d[ky] / d[kz];
    const float sz = 1.f / d[kz];

    const bool test_triangles = ANY ? (obj.visibility == 0) : (obj.visibility != 2);
    const uint2* nodes = s.mesh_nodes + obj.node_offset;
    Stack_Entry stack[kMaxTraversalDepth];
    int sp = 0;
    uint32_t node = 0;
    const float entry_t = hit.t;
    while ((ANY ? ray_tmax : hit.t) > t_min) {
        const uint2 n = __ldg(nodes + node);
        if ((n.x & 3u) != 3u) {
            if (!descend(n, node, o, d, inv, t_min, t_max, stack, sp)) return -1;
        } else {
            const uint32_t count = n.x >> 2;
            if (test_triangles && count) {
                const uint32_t* idx = reinterpret_cast<const uint32_t*>(nodes + node) + 1;
                for (uint32_t i = 0; i < count; i++) {
                    const uint32_t prim = (i == 0) ? n.y : __ldg(idx + i);
                    const float4* tp = s.tris + 3 * ((size_t)obj.tri_offset + prim);
                    const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
                    float b0, b1, b2;
                    const float t = watertight(o, d, kx, ky, kz, sx, sy, sz, v0, v1, v2, b0, b1, b2);
                    if (ANY) {
                        // `t >= ray_tmax` rejects; a NaN t does not (src/ref/kdtree.cpp:60-62)
                        if (!(t >= ray_tmax) && v0.w == 0.f) return 1;
                    } else if (t < hit.t && v0.w == 0.f) {
                        hit.t = t;
                        hit.prim = prim;
                        hit.b0 = b0;
                        hit.b1 = b1;
                        hit.b2 = b2;
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
    return ANY ? 0 : (hit.t < entry_t ? 1 : 0);
}

// Scene-level traversal with intersect_scene_geometry_data /
// intersect_any_scene_geometry_data (src/ref/kdtree.cpp:81-109).
// Closest: returns 1 on hit (hit filled), 0 on miss.  Any: 1 if occluded.
// Returns -1 on stack overflow.
template <bool ANY>
__device__ __forceinline__ int scene_traverse(const Device_Scene& s, const float o[3], const float d[3],
                                              float ray_tmax, Hit& hit) {
    hit.t = ray_tmax;
    hit.prim = 0xffffffffu;
    hit.object = 0xffffffffu;
    hit.b0 = hit.b1 = hit.b2 = 0.f;
    float t_min, t_max;
    const float mn[3] = {s.scene_bounds[0], s.scene_bounds[1], s.scene_bounds[2]};
    const float mx[3] = {s.scene_bounds[3], s.scene_bounds[4], s.scene_bounds[5]};
    if (!clip_ray(mn, mx, o, d, t_min, t_max)) return 0;
    const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
    Stack_Entry stack[kMaxTraversalDepth];
    int sp = 0;
    uint32_t node = 0;
    while ((ANY ? ray_tmax : hit.t) > t_min) {
        const uint2 n = __ldg(s.scene_nodes + node);
        if ((n.x & 3u) != 3u) {
            if (!descend(n, node, o, d, inv, t_min, t_max, stack, sp)) return -1;
        } else {
            const uint32_t count = n.x >> 2;
            const uint32_t* idx = reinterpret_cast<const uint32_t*>(s.scene_nodes + node) + 1;
            for (uint32_t i = 0; i < count; i++) {
                const uint32_t object_index = (i == 0) ? n.y : __ldg(idx + i);
                const Object_Record obj = load_object(s.objects, object_index);
                float oo[3], od[3];
                transform_ray(obj.m, o, d, oo, od);
                const int r = mesh_traverse<ANY>(s, obj, oo, od, ray_tmax, hit);
                if (r < 0) return -1;
                if (ANY) {
                    if (r) return 1;
                } else if (r) {
                    hit.object = object_index;
                }
            }
            if (sp == 0) break;
            --sp;
            node = stack[sp].node;
            t_min = t_max;
            t_max = stack[sp].t_max;
        }
    }
    return ANY ? 0 : (hit.t < ray_tmax ? 1 : 0);
}

} // namespace yar
