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
// Traversal structure (GB300-first): the reference recurses scene tree ->
// object -> mesh tree with a separate loop per level.  On a SIMT machine that
// nesting serialises a warp whose lanes sit at different levels, so here one
// loop drives a small state machine per lane: DESCEND (fetch the current
// level's node, descend through interior nodes), SCENE_LEAF (enter the next
// object of a scene leaf: transform the ray, clip it to the mesh bounds),
// MESH_LEAF (test the next triangle of a mesh leaf).  Scene and mesh levels
// share the descend code and one traversal stack (mesh entries sit above the
// scene entries).  Lanes reconverge at the top of every iteration.
//
// Visit order, termination tests and every float operation follow the
// reference (src/ref/kdtree.cpp:12-109, :219-439) step by step: the
// translation unit is compiled with -fmad=false and IEEE division, and small
// per-axis values are selected with conditional moves rather than indexed
// (indexing register arrays would put them in local memory).  Hit triangle
// ids, t and barycentrics are therefore bit-identical to KdTree::intersect.
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
    // alpha test: per-triangle shading records (uvs in the .w / last lanes),
    // texels and mip records of the scene's image textures
    const float4* shading = nullptr;
    const float4* texels = nullptr;
    const uint4* texture_mips = nullptr;
    float scene_bounds[6] = {0, 0, 0, 0, 0, 0};
    uint32_t object_count = 0;
};

struct Hit {
    float t;
    uint32_t prim;
    uint32_t object;
    float b0, b1, b2;
};

__device__ __forceinline__ float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

// Bounding_Box::intersect_by_ray_without_NaNs, src/lib/bounding_box.h:63-85
__device__ __forceinline__ bool clip_axis(float mn, float mx, float o, float d, float& t0, float& t1) {
    if (d != 0.f) {
        const float inv = 1.f / d;
        float s0 = (mn - o) * inv;
        float s1 = (mx - o) * inv;
        if (inv < 0.f) { const float tmp = s0; s0 = s1; s1 = tmp; }
        t0 = s0 > t0 ? s0 : t0;
        t1 = s1 < t1 ? s1 : t1;
        return !(t0 > t1);
    }
    return !(o < mn || o > mx);
}

// The same with 1/d already computed (the value clip_axis divides out).
__device__ __forceinline__ bool clip_axis_inv(float mn, float mx, float o, float d, float inv, float& t0, float& t1) {
    if (d != 0.f) {
        float s0 = (mn - o) * inv;
        float s1 = (mx - o) * inv;
        if (inv < 0.f) { const float tmp = s0; s0 = s1; s1 = tmp; }
        t0 = s0 > t0 ? s0 : t0;
        t1 = s1 < t1 ? s1 : t1;
        return !(t0 > t1);
    }
    return !(o < mn || o > mx);
}

__device__ __forceinline__ bool clip_ray_inv(float3 mn, float3 mx, float3 o, float3 d, float3 inv, float& t_min,
                                             float& t_max) {
    float t0 = 0.f, t1 = __int_as_float(0x7f800000);
    if (!clip_axis_inv(mn.x, mx.x, o.x, d.x, inv.x, t0, t1)) return false;
    if (!clip_axis_inv(mn.y, mx.y, o.y, d.y, inv.y, t0, t1)) return false;
    if (!clip_axis_inv(mn.z, mx.z, o.z, d.z, inv.z, t0, t1)) return false;
    t_min = t0;
    t_max = t1;
    return true;
}

__device__ __forceinline__ bool clip_ray(float3 mn, float3 mx, float3 o, float3 d, float& t_min, float& t_max) {
    float t0 = 0.f, t1 = __int_as_float(0x7f800000);
    if (!clip_axis(mn.x, mx.x, o.x, d.x, t0, t1)) return false;
    if (!clip_axis(mn.y, mx.y, o.y, d.y, t0, t1)) return false;
    if (!clip_axis(mn.z, mx.z, o.z, d.z, t0, t1)) return false;
    t_min = t0;
    t_max = t1;
    return true;
}

// Per-ray setup of the watertight test (src/ref/intersection.cpp:55-62).
struct Watertight_Ray {
    int kx, ky, kz;
    float sx, sy, sz;
};

// inv = 1/d per axis (the same IEEE division the setup's 1/dz is).
__device__ __forceinline__ Watertight_Ray watertight_setup(float3 d, float3 inv) {
    Watertight_Ray w;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    w.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);  // Vector3::max_dimension
    w.kx = (w.kz == 2 ? 0 : w.kz + 1);
    w.ky = (w.kz == 0 ? 2 : w.kz - 1);
    const float dx = sel3(d.x, d.y, d.z, w.kx), dy = sel3(d.x, d.y, d.z, w.ky), dz = sel3(d.x, d.y, d.z, w.kz);
    w.sx = -dx / dz;
    w.sy = -dy / dz;
    w.sz = sel3(inv.x, inv.y, inv.z, w.kz);
    return w;
}

// intersect_triangle_watertight, src/ref/intersection.cpp:64-113.
// Returns +inf when there is no intersection.
__device__ __forceinline__ float watertight(float3 o, const Watertight_Ray& w, float4 v0, float4 v1, float4 v2,
                                            float& b0, float& b1, float& b2) {
    const float ox = sel3(o.x, o.y, o.z, w.kx), oy = sel3(o.x, o.y, o.z, w.ky), oz = sel3(o.x, o.y, o.z, w.kz);
    const float p0x = sel3(v0.x, v0.y, v0.z, w.kx) - ox, p0y = sel3(v0.x, v0.y, v0.z, w.ky) - oy,
                p0z = sel3(v0.x, v0.y, v0.z, w.kz) - oz;
    const float p1x = sel3(v1.x, v1.y, v1.z, w.kx) - ox, p1y = sel3(v1.x, v1.y, v1.z, w.ky) - oy,
                p1z = sel3(v1.x, v1.y, v1.z, w.kz) - oz;
    const float p2x = sel3(v2.x, v2.y, v2.z, w.kx) - ox, p2y = sel3(v2.x, v2.y, v2.z, w.ky) - oy,
                p2z = sel3(v2.x, v2.y, v2.z, w.kz) - oz;
    const float x0 = p0x + w.sx * p0z;
    const float y0 = p0y + w.sy * p0z;
    const float x1 = p1x + w.sx * p1z;
    const float y1 = p1y + w.sy * p1z;
    const float x2 = p2x + w.sx * p2z;
    const float y2 = p2y + w.sy * p2z;
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
    const float z0 = w.sz * p0z;
    const float z1 = w.sz * p1z;
    const float z2 = w.sz * p2z;
    const float t_scaled = e0 * z0 + e1 * z1 + e2 * z2;
    if ((__float_as_uint(det) ^ __float_as_uint(t_scaled)) >> 31) return inf;
    const float inv_det = 1.f / det;
    const float t = inv_det * t_scaled;
    b0 = e0 * inv_det;
    b1 = e1 * inv_det;
    b2 = e2 * inv_det;
    return t;
}

// The alpha test of both leaf callbacks (src/ref/kdtree.cpp:31-38, :69-77):
// the hit's uv, Triangle_Mesh::get_uv (barycentric_interpolate, src/lib/math.h:
// 146-153: b.x uv0 + b.y uv1 + b.z uv2), the alpha texture's mip 0 sampled by
// Image_Texture::sample_bilinear with repeat wrapping (image_texture.cpp:441-476);
// true when its red channel is 0 (the triangle is skipped).
__device__ __forceinline__ float alpha_texel_r(const Device_Scene& s, uint4 mip, int x, int y) {  // get_texel_repeat
    const int w = (int)mip.x, h = (int)mip.y;
    if (x >= 0) x &= w - 1;
    else { x %= w; x += (x >> 31) & w; }
    if (y >= 0) y &= h - 1;
    else { y %= h; y += (y >> 31) & h; }
    return __ldg(&s.texels[mip.z + (size_t)y * (size_t)w + (size_t)x].x);
}
static __device__ __noinline__ bool alpha_rejects(const Device_Scene& s, uint32_t object, uint32_t global_tri, float b0, float b1,
                                           float b2) {
    const uint32_t mip_index = __float_as_uint(__ldg(s.objects + 6 * (size_t)object + 5).z);
    const float4* sh = s.shading + 4 * (size_t)global_tri;
    const float4 s0 = __ldg(sh), s1 = __ldg(sh + 1), s2 = __ldg(sh + 2), s3 = __ldg(sh + 3);
    const float u = b0 * s0.w + b1 * s2.w + b2 * s3.y;
    const float v = b0 * s1.w + b1 * s3.x + b2 * s3.z;
    const uint4 mip = __ldg(s.texture_mips + mip_index);
    const float x = u * (float)mip.x - 0.5f, y = v * (float)mip.y - 0.5f;
    const float x_floor = floorf(x), y_floor = floorf(y);
    const float wx = x - x_floor, wy = y - y_floor;
    const int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    const float r = ((alpha_texel_r(s, mip, x0, y0) * ((1 - wy) * (1 - wx)) +
                      alpha_texel_r(s, mip, x1, y0) * ((1 - wy) * wx)) +
                     alpha_texel_r(s, mip, x0, y1) * (wy * (1 - wx))) +
                    alpha_texel_r(s, mip, x1, y1) * (wy * wx);
    return r == 0.f;
}

// transform_ray, src/lib/matrix.cpp:368-389: ((a*x + b*y) + c*z) + w
__device__ __forceinline__ void transform_ray(float4 r0, float4 r1, float4 r2, float3 o, float3 d, float3& oo,
                                              float3& od) {
    oo.x = r0.x * o.x + r0.y * o.y + r0.z * o.z + r0.w;
    oo.y = r1.x * o.x + r1.y * o.y + r1.z * o.z + r1.w;
    oo.z = r2.x * o.x + r2.y * o.y + r2.z * o.z + r2.w;
    od.x = r0.x * d.x + r0.y * d.y + r0.z * d.z;
    od.y = r1.x * d.x + r1.y * d.y + r1.z * d.z;
    od.z = r2.x * d.x + r2.y * d.y + r2.z * d.z;
}

enum : int { kDescend = 0, kSceneLeaf = 1, kMeshLeaf = 2, kDone = 3 };

// Traversal stack: 2 * kMaxTraversalDepth node entries (scene level below,
// mesh level above) plus the two entries that save the scene level while a
// mesh is traversed.
constexpr int kStackEntries = 2 * kMaxTraversalDepth + 2;

// Two-level closest-hit (ANY = false) or any-hit (ANY = true) traversal of one
// ray as a resumable state machine: begin() sets up a ray, step() performs one
// unit of work (a descent through interior nodes down to a leaf, one scene-leaf
// object entry, or one triangle test) and returns false once the ray is
// finished.  status() afterwards: closest 1 = hit / 0 = miss; any 1 =
// occluded / 0 = not; -1 = traversal-stack overflow.
//
// The state is kept small so that it stays in registers: the world ray is not
// held while a mesh is traversed (it is reloaded from the ray record when the
// mesh is left, and 1/d recomputed with the same IEEE division); the scene
// level's interval and leaf cursor go onto the traversal stack when an object
// is entered; mode, level, the triangle-test flag, the watertight axis
// permutation and the status share one word; a leaf's primitive count is
// re-read from its node (an L1 hit) instead of being held.
template <bool ANY>
struct Traversal {
    float3 co, cinv;       // ray origin and 1/direction of the current level (world ray at scene level)
    float ray_tmax;        // (read by any hit only)
    uint32_t ray;          // index of the ray record
    uint32_t node;         // current node; while a leaf is processed, the leaf
    float t_min, t_max;
    int sp, mesh_sp_base;
    uint32_t mesh_offset;  // node offset of the current mesh in mesh_nodes
    uint32_t tri_offset;   // triangle offset of the current mesh
    uint32_t leaf_i;       // next primitive of the current leaf
    uint32_t cur_object;
    uint32_t flags;        // bits 0-1 mode, 2 in mesh, 3 test triangles, 4-9 kx ky kz, 10-11 status + 1,
                           // 12-14 direction component > 0 (x, y, z) of the current level's ray,
                           // 15 the current mesh has an alpha texture
    float sx, sy, sz;      // watertight setup of the mesh ray (src/ref/intersection.cpp:55-62)
    Hit hit;

    __device__ __forceinline__ int mode() const { return (int)(flags & 3u); }
    __device__ __forceinline__ void set_mode(int m) { flags = (flags & ~3u) | (uint32_t)m; }
    __device__ __forceinline__ bool in_mesh() const { return (flags >> 2) & 1u; }
    __device__ __forceinline__ int status() const { return (int)((flags >> 10) & 3u) - 1; }

    // the direction itself is not held: its per-axis signs steer descents
    // through split planes the origin lies on, and the world direction is
    // reloaded from the ray record where an object is entered
    static __device__ __forceinline__ uint32_t positive_bits(float x, float y, float z) {
        return (x > 0.f ? 1u << 12 : 0u) | (y > 0.f ? 1u << 13 : 0u) | (z > 0.f ? 1u << 14 : 0u);
    }
    static constexpr uint32_t kSignBits = 7u << 12;
    __device__ __forceinline__ int closest_status() const { return hit.prim != 0xffffffffu ? 1 : 0; }

    __device__ __forceinline__ void finish(int st) { flags = (flags & ~(3u | (3u << 10))) | (uint32_t)kDone | ((uint32_t)(st + 1) << 10); }

    template <class STACK>
    __device__ __forceinline__ void leave_mesh(const Device_Scene& s, const float4* rays, STACK& stack) {
        sp = mesh_sp_base;
        const uint2 cursor = stack.pop(sp - 1);
        const uint2 interval = stack.pop(sp - 2);
        sp -= 2;
        node = cursor.x;
        leaf_i = cursor.y;
        t_min = __uint_as_float(interval.x);
        t_max = __uint_as_float(interval.y);
        const float4 r0 = __ldg(rays + 2 * (size_t)ray), r1 = __ldg(rays + 2 * (size_t)ray + 1);
        co = make_float3(r0.x, r0.y, r0.z);
        cinv = make_float3(1.f / r1.x, 1.f / r1.y, 1.f / r1.z);
        flags = (flags & ~(3u | 4u | kSignBits)) | (uint32_t)kSceneLeaf | positive_bits(r1.x, r1.y, r1.z);
    }

    __device__ __forceinline__ void begin(const Device_Scene& s, uint32_t ray_index, float3 ro, float3 rd, float tmax) {
        ray = ray_index;
        ray_tmax = tmax;
        hit.t = tmax;
        hit.prim = 0xffffffffu;
        hit.object = 0xffffffffu;
        hit.b0 = hit.b1 = hit.b2 = 0.f;
        sp = 0;
        mesh_sp_base = 0;
        node = 0;
        flags = (uint32_t)kDescend | (1u << 10);  // status 0
        const float3 inv = make_float3(1.f / rd.x, 1.f / rd.y, 1.f / rd.z);
        if (!clip_ray_inv(make_float3(s.scene_bounds[0], s.scene_bounds[1], s.scene_bounds[2]),
                          make_float3(s.scene_bounds[3], s.scene_bounds[4], s.scene_bounds[5]), ro, rd, inv, t_min,
                          t_max)) {
            finish(0);
            return;
        }
        co = ro;
        cinv = inv;
        flags |= positive_bits(rd.x, rd.y, rd.z);
    }

    // The current level's leaf is done: pop the level's next node, or end the
    // level (leave the mesh; finish the ray at the scene level).
    template <class STACK>
    __device__ __forceinline__ void leaf_done(const Device_Scene& s, const float4* rays, STACK& stack) {
        if (in_mesh()) {
            if (sp == mesh_sp_base) {
                leave_mesh(s, rays, stack);
                return;
            }
        } else if (sp == 0) {
            finish(ANY ? 0 : closest_status());
            return;
        }
        --sp;
        const uint2 e = stack.pop(sp);
        node = e.x;
        t_min = t_max;
        t_max = __uint_as_float(e.y);
        set_mode(kDescend);
    }

    // DESCEND: up to MAXD node fetches of the current level.  A leaf with
    // primitives to process switches the mode; an empty leaf (or a mesh leaf
    // whose triangles this ray kind skips) is done at once, as the reference's
    // leaf callback returns without work, and the descent goes on from the
    // popped node.  `stack` holds kStackEntries entries (Local_Stack or
    // Split_Stack; kept out of this struct so the scalar state can live in
    // registers).
    template <int MAXD, class STACK>
    __device__ __forceinline__ void step_descend(const Device_Scene& s, const float4* rays, STACK& stack) {
        for (int steps = 0; steps < MAXD; steps++) {
            const uint2* nodes = in_mesh() ? s.mesh_nodes + mesh_offset : s.scene_nodes;
            const float limit = ANY ? ray_tmax : hit.t;
            if (!(limit > t_min)) {  // the level's loop condition failed
                if (in_mesh()) {
                    leave_mesh(s, rays, stack);
                } else {
                    finish(ANY ? 0 : closest_status());
                }
                return;
            }
            const uint2 n = __ldg(nodes + node);
            if ((n.x & 3u) == 3u) {
                const bool skip = in_mesh() && !((flags >> 3) & 1u);
                if ((n.x >> 2) == 0u || skip) {
                    leaf_done(s, rays, stack);
                    if (mode() != kDescend) return;
                    continue;
                }
                leaf_i = 0;
                set_mode(in_mesh() ? kMeshLeaf : kSceneLeaf);
                return;
            }
            const int axis = (int)(n.x & 3u);
            const float dist = __uint_as_float(n.y) - sel3(co.x, co.y, co.z, axis);
            const uint32_t below_child = node + 1;
            const uint32_t above_child = n.x >> 2;
            if (dist != 0.f) {
                const bool below_first = dist > 0.f;
                const uint32_t first_child = below_first ? below_child : above_child;
                const uint32_t second_child = below_first ? above_child : below_child;
                const float t_split = dist * sel3(cinv.x, cinv.y, cinv.z, axis);
                if (t_split > t_max || t_split < 0.f) {
                    node = first_child;
                } else if (t_split < t_min) {
                    node = second_child;
                } else {
                    if (sp >= kStackEntries) {
                        finish(-1);
                        return;
                    }
                    stack.push(sp, second_child, t_max);
                    sp++;
                    node = first_child;
                    t_max = t_split;
                }
            } else {
                node = ((flags >> (12 + axis)) & 1u) ? above_child : below_child;
            }
        }
    }

    // MESH_LEAF: one triangle test of the current mesh leaf; after the leaf's
    // last triangle the leaf is done in the same step.
    template <class STACK>
    __device__ __forceinline__ void step_mesh_leaf(const Device_Scene& s, const float4* rays, STACK& stack) {
        const uint2* nodes = s.mesh_nodes + mesh_offset;
        const uint2 leaf = __ldg(nodes + node);
        const uint32_t count = leaf.x >> 2;
        if (leaf_i < count) {
            const uint32_t prim =
                (leaf_i == 0) ? leaf.y : __ldg(reinterpret_cast<const uint32_t*>(nodes + node) + 1 + leaf_i);
            leaf_i++;
            const float4* tp = s.tris + 3 * ((size_t)tri_offset + prim);
            const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
            Watertight_Ray wr;
            wr.kx = (int)((flags >> 4) & 3u);
            wr.ky = (int)((flags >> 6) & 3u);
            wr.kz = (int)((flags >> 8) & 3u);
            wr.sx = sx;
            wr.sy = sy;
            wr.sz = sz;
            float b0, b1, b2;
            const float t = watertight(co, wr, v0, v1, v2, b0, b1, b2);
            if (ANY) {
                // `t >= ray_tmax` rejects; a NaN t does not (src/ref/kdtree.cpp:60-62)
                if (!(t >= ray_tmax) && v0.w == 0.f &&
                    !(((flags >> 15) & 1u) && alpha_rejects(s, cur_object, tri_offset + prim, b0, b1, b2))) {
                    finish(1);
                    return;
                }
            } else if (t < hit.t && v0.w == 0.f &&
                       !(((flags >> 15) & 1u) && alpha_rejects(s, cur_object, tri_offset + prim, b0, b1, b2))) {
                // the object of the closest hit is the one whose mesh produced it
                // (src/ref/kdtree.cpp:81-95 sets it after the mesh improved the hit)
                hit.t = t;
                hit.prim = prim;
                hit.object = cur_object;
                hit.b0 = b0;
                hit.b1 = b1;
                hit.b2 = b2;
            }
            if (leaf_i < count) return;
        }
        leaf_done(s, rays, stack);
    }

    // SCENE_LEAF: one object of the current scene leaf (transform the ray into
    // the object's space and clip it to the mesh bounds; when it overlaps,
    // save the scene level on the stack and descend the mesh tree), or, with
    // every object done, the end of the leaf.
    template <class STACK>
    __device__ __forceinline__ void step_scene_leaf(const Device_Scene& s, const float4* rays, STACK& stack) {
        const uint2 leaf = __ldg(s.scene_nodes + node);
        const uint32_t count = leaf.x >> 2;
        if (leaf_i < count) {
            const uint32_t obj =
                (leaf_i == 0) ? leaf.y : __ldg(reinterpret_cast<const uint32_t*>(s.scene_nodes + node) + 1 + leaf_i);
            leaf_i++;
            const float4* p = s.objects + 6 * (size_t)obj;
            const float4 r0 = __ldg(p + 0), r1 = __ldg(p + 1), r2 = __ldg(p + 2);
            const float4 lo = __ldg(p + 3), hi = __ldg(p + 4), info = __ldg(p + 5);
            const float4 wd = __ldg(rays + 2 * (size_t)ray + 1);  // the world direction
            float3 oo, od;
            transform_ray(r0, r1, r2, co, make_float3(wd.x, wd.y, wd.z), oo, od);
            float mt_min, mt_max;
            const float3 oinv = make_float3(1.f / od.x, 1.f / od.y, 1.f / od.z);
            if (clip_ray_inv(make_float3(lo.x, lo.y, lo.z), make_float3(hi.x, hi.y, hi.z), oo, od, oinv, mt_min, mt_max)) {
                if (sp + 2 > kStackEntries) {
                    finish(-1);
                    return;
                }
                stack.push(sp, __float_as_uint(t_min), t_max);  // the scene level's interval
                stack.push(sp + 1, node, __uint_as_float(leaf_i));  // and its leaf cursor
                sp += 2;
                mesh_sp_base = sp;
                cur_object = obj;
                co = oo;
                cinv = oinv;
                mesh_offset = __float_as_uint(lo.w);
                tri_offset = __float_as_uint(hi.w);
                const int visibility = __float_as_int(info.y);
                const bool test_triangles = ANY ? (visibility == 0) : (visibility != 2);
                const Watertight_Ray wr = watertight_setup(od, oinv);
                sx = wr.sx;
                sy = wr.sy;
                sz = wr.sz;
                flags = (flags & (3u << 10)) | (uint32_t)kDescend | 4u | (test_triangles ? 8u : 0u) |
                        ((uint32_t)wr.kx << 4) | ((uint32_t)wr.ky << 6) | ((uint32_t)wr.kz << 8) |
                        positive_bits(od.x, od.y, od.z) | (__float_as_int(info.z) >= 0 ? 1u << 15 : 0u);
                node = 0;
                t_min = mt_min;
                t_max = mt_max;
            }
            return;
        }
        leaf_done(s, rays, stack);
    }

    // One unit of work in the current mode; false once the ray is finished.
    // A descent stops at a leaf or after MAXD node fetches.
    template <int MAXD, class STACK>
    __device__ __forceinline__ bool step(const Device_Scene& s, const float4* rays, STACK& stack) {
        const int m = mode();
        if (m == kDescend) step_descend<MAXD>(s, rays, stack);
        else if (m == kMeshLeaf) step_mesh_leaf(s, rays, stack);
        else if (m == kSceneLeaf) step_scene_leaf(s, rays, stack);
        return mode() != kDone;
    }
};

// Traversal stack in local memory (L1-cached).
struct Local_Stack {
    uint2 e[kStackEntries];
    __device__ __forceinline__ void push(int sp, uint32_t node, float t_max) {
        e[sp] = make_uint2(node, __float_as_uint(t_max));
    }
    __device__ __forceinline__ uint2 pop(int sp) const { return e[sp]; }
};

// Traversal stack whose first SHORT entries live in shared memory, laid out
// entry-major ([entry][thread], conflict-free for a warp), with the rarely
// used deeper entries in local memory.
template <int SHORT, int BLOCK>
struct Split_Stack {
    uint2* smem;  // this thread's column: base + threadIdx.x
    uint2 deep[kStackEntries - SHORT];
    __device__ __forceinline__ void push(int sp, uint32_t node, float t_max) {
        const uint2 v = make_uint2(node, __float_as_uint(t_max));
        if (sp < SHORT) smem[sp * BLOCK] = v;
        else deep[sp - SHORT] = v;
    }
    __device__ __forceinline__ uint2 pop(int sp) const { return sp < SHORT ? smem[sp * BLOCK] : deep[sp - SHORT]; }
};

} // namespace yar
