// wavefront.cuh - the wavefront path tracer's kernels and their host-side
// launch helpers, shared by the reference-order render (render.cu) and the
// guided render (guided.cu).  Everything here has internal linkage: each
// translation unit that includes it gets its own copies.
//
// Kernels, one wavefront step each:
//   sample tables / camera   per (pixel, dimension) row and per path: the
//              pixel's pcg stream, its stratified + shuffled sample tables
//              (Stratified_Pixel_Sampler::next_pixel, src/ref/pixel_sampling.cpp:54-141)
//              and one camera ray per sample (Camera::generate_ray, src/ref/camera.cpp:16-31)
//   extend     closest hit for the path rays (shared traversal, cast.cu)
//   shade      per path vertex: emission, shading context, BSDF, the light
//              sample (shadow ray), the MIS BSDF sample (probe ray), the
//              continuation ray and Russian roulette
//              (trace_path, src/ref/path_tracing.cpp:11-133;
//               direct_lighting_from_rectangular_light, direct_lighting.cpp:109-194)
//   shadow     any hit for the shadow queue
//   probe      closest hit for the MIS probe queue
//   connect    adds the vertex's direct light in the reference's order
//   film       clamp/scale, luminance variance, tile-ordered film merge and
//              resolve (src/ref/film.cpp, reference_renderer.cpp:388-409, :565-581)
//
// Paths of a chunk of pixels live in structure-of-arrays state indexed by
// slot = pixel_in_chunk * spp + sample.  Ray queues are compacted with one
// warp-aggregated atomic per warp.  Queue order is not deterministic, the
// results are: every path and every film pixel is computed in the
// reference's order.
#pragma once

#include "context.hpp"
#include "shade.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

namespace yar {

namespace {

constexpr int kBlock = 128;
constexpr int kTile = 64;                           // src/ref/film.cpp:5
constexpr uint64_t kChunkSampleBudget = 16u << 20;  // paths in flight per chunk

// Path flags above the bounce and dimension counters of Path_State::info.
// kDeltaArrival: the path's extend ray left a delta vertex (mirror, perfect
// refractor, smooth glass) and its hit is shaded as the reference's delta
// branch does; kDeltaFinal: that delta vertex used the last bounce.
// What the MIS probe of a vertex must hit: pend_probe2.z
enum : uint32_t { kProbeRectLight = 0, kProbeMeshLight = 1, kProbeSphereLight = 2, kProbeEnvLight = 3 };

enum : uint32_t {
    kPendShadow = 1u << 24,
    kPendProbe = 1u << 25,
    kPendDirect = 1u << 26,
    kDeltaArrival = 1u << 27,
    kDeltaFinal = 1u << 28,
    kDeferred = 1u << 29,  // exact tail: the path's next extend ray waits in Path_State::deferred
    kDiffRays = 1u << 30   // the delta ray carries specular differential rays (Path_State::diff)
};

// Raytracer_Config::max_differential_ray_specular_bounces (src/lib/raytracer_config.h:33);
// no scene format sets it.
constexpr int kMaxDifferentialRaySpecularBounces = 4;

struct Rect_Light_Dev {
    float4 r0, r1, r2;  // light_to_world rows
    float4 le;          // emitted radiance rgb, size.x
    float4 sz;          // size.y, then (probe culling, set when the light's own triangles lie on its
                        // rectangle) 1 / |x axis|^2, 1 / |y axis|^2, 0 = off
};

// Whether the MIS probe from o along d can reach rectangular light L: false
// only when the ray's crossing of the light's plane lies behind o or outside
// the rectangle widened by 10%, by 2e-3 of its larger side and by 2e-3 of that
// side per unit of 1/cos (the light's triangles lie within 1e-3 of its larger
// side of the rectangle, in the plane and across it, checked on upload, so such
// a ray cannot hit them and the probe would add nothing).
__device__ __forceinline__ bool probe_may_reach(const Rect_Light_Dev& L, V3 o, V3 d, float lndw) {
    const float4 r0 = __ldg(&L.r0), r1 = __ldg(&L.r1), r2 = __ldg(&L.r2), sz = __ldg(&L.sz);
    if (sz.w == 0.f) return true;
    const V3 c = v3(r0.w, r1.w, r2.w), n = v3(r0.z, r1.z, r2.z);
    const float den = dot(d, n);
    if (!(fabsf(den) > 0.f)) return true;
    const float t = dot(c - o, n) / den;
    if (t < 0.f) return false;
    const V3 q = (o + mul(d, t)) - c;
    const float sx = __ldg(&L.le).w, sy = sz.x;
    const float big = fmaxf(sx, sy);
    const float slack = 2e-3f * big + 2e-3f * big / lndw;
    const float a = dot(q, v3(r0.x, r1.x, r2.x)) * sz.y, b = dot(q, v3(r0.y, r1.y, r2.y)) * sz.z;
    return fabsf(a) <= 0.55f * sx + slack && fabsf(b) <= 0.55f * sy + slack;
}

// Point, spot and directional lights (direct_lighting.cpp:26-107):
//   a = position xyz, type bits | b = direction xyz, cos(cone angle)
//   c = intensity (irradiance) rgb, cos(max(0, cone angle - penumbra angle))
// The cosines are computed on the host, as the reference computes them per use.
struct Delta_Light_Dev {
    float4 a, b, c;
};

// Triangle-mesh lights (Diffuse_Triangle_Mesh_Light_Sampler, light_sampling.cpp:126-184):
//   le = emitted radiance rgb, mesh area
//   info = first triangle of the mesh in the scene's triangle arrays, triangle
//          count, offset of its CDF in Scene_Dev::mesh_cdf, -
struct Mesh_Light_Dev {
    float4 le;
    uint4 info;
};

// Sphere lights (Diffuse_Sphere_Light): a = center xyz, radius; le = emitted rgb.
struct Sphere_Light_Dev {
    float4 a, le;
};

struct Render_Params {
    yar_camera_desc camera;
    int32_t sx0, sy0, sw, sh;    // sample region
    int32_t rx0, ry0, rw, rh;    // render region
    int32_t tiles_x, tiles_y;
    int32_t nx, ny, spp, n1d, n2d;
    int32_t max_bounces, rr_bounce_threshold;
    float rr_threshold;
    float filter_radius;
    int32_t filter_type;    // Raytracer_Config::Pixel_Filter_Type: 0 box, 1 gaussian, 2 triangle
    float filter_alpha;     // gaussian falloff
    float filter_zero;      // gaussian: exp(-alpha r^2), the weight at the radius (computed on the host)
    float film_scale, max_component;
    int32_t total_lights, delta_lights, rect_lights, sphere_lights, mesh_lights, env_lights;  // selection order
    int32_t full_shading;  // the scene needs shade_kernel<*, true>
    int32_t arrays_2d_first;  // direct lighting: the 2D rows (array grids) come before the 1D rows in the stream
    uint32_t seed_offset;
    uint32_t stream_hi;  // upper 32 bits of the pixel streams' sequence (0 = the reference's streams)
    // Draws past the sampler budget: 0 = one pcg stream per sample; 1 = exact
    // tail, first phase (a path that might draw past the budget at its next
    // vertex is deferred); 2 = exact tail, waves (draws are counted per path).
    int32_t exact_tail;
    int32_t textured;  // some material has an image texture or a bump map
    int32_t spec_diffs;  // image textures with delta materials: delta rays carry differential rays
};

struct Path_State {
    float4* coeff;
    float4* L;
    uint32_t* info;        // bounce | i1d << 8 | i2d << 16 | pending flags
    uint4* rng;            // pcg state for dimensions beyond the sampler budget
    float4* pend_light;    // unoccluded light-sample contribution
    float4* pend_probe0;   // Le * f, bsdf pdf
    float4* pend_probe1;   // probe origin, dot(light_n, -wi)
    float4* pend_probe2;   // dot(n, wi), light index bits
    float4* pend_coeff;    // path throughput at the vertex
    uint8_t* occluded;
    float4* probe_hit4;    // t, b0, b1, b2
    uint2* probe_hit2;     // prim, object
    uint32_t* rec;         // guided training: this bounce's record index (0xffffffff = none)
    uint32_t* rng_draws;   // exact tail: pcg draws this path took past the budget
    float4* deferred;      // exact tail: the deferred extend ray, 2 float4 per slot
    const float2* image_samples;  // image-plane samples of the render (textured scenes' ray differentials)
    uint32_t chunk_first;         // the chunk's first pixel
    float4* diff;  // specular differential rays of the slot's delta ray: dx origin, dx direction, dy origin,
                   // dy direction packed in 3 float4 (Render_Params::spec_diffs)
};

// Learned-proposal hooks of the shade kernel (guided render only).
// Training records, kGuideRecordF4 float4 each:
//   0 {pos, n.x}  1 {n.yz, wo.xy}  2 {wo.z, dir}  3 {f cos / p (luminance), slot bits, -, -}
//   4 {path throughput after the continuation}  5 {path radiance after this vertex's direct light}
constexpr int kGuideRecordF4 = 6;
struct Guide_Shade {
    const float* lobes = nullptr;    // per extend-queue position (null: BSDF continuation only)
    const float4* queries = nullptr; // per extend-queue position: 3 float4 of the network input
    float alpha = 0.f;               // probability of drawing the continuation from the mixture
    float4* records = nullptr;       // null: no training records
    uint32_t* record_count = nullptr;
    uint32_t record_capacity = 0;
};

// Mixture of von Mises-Fisher lobes {mean xyz, kappa, weight} x 8.
__device__ __forceinline__ float vmf_norm(float kappa) {
    // kappa / (2 pi (1 - exp(-2 kappa)))
    return kappa / (6.283185307f * -expm1f(-2.f * kappa));
}
__device__ __forceinline__ float mixture_pdf(const float* lob, V3 w) {
    float q = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float c = lob[5 * k] * w.x + lob[5 * k + 1] * w.y + lob[5 * k + 2] * w.z;
        const float kap = lob[5 * k + 3];
        q += lob[5 * k + 4] * vmf_norm(kap) * __expf(kap * (c - 1.f));
    }
    return q;
}
// Lobe by its weight (u0), then the vMF direction (u1, u2) by inversion of
// its cosine distribution (Jakob, "Numerically stable sampling of the von
// Mises-Fisher distribution on S^2", 2012).
__device__ __forceinline__ V3 mixture_sample(const float* lob, float u0, float u1, float u2) {
    int k = 0;
    float acc = lob[4];
    while (k < 7 && u0 >= acc) {
        k++;
        acc += lob[5 * k + 4];
    }
    const V3 mu = v3(lob[5 * k], lob[5 * k + 1], lob[5 * k + 2]);
    const float kap = lob[5 * k + 3];
    const float cz = fminf(1.f, fmaxf(-1.f, 1.f + log1pf(u1 * expm1f(-2.f * kap)) / kap));
    const float s = sqrtf(fmaxf(0.f, 1.f - cz * cz));
    float sp, cp;
    sincospif(2.f * u2, &sp, &cp);
    const V3 t = coordinate_axis(mu);
    const V3 b = cross(mu, t);
    return mul(t, s * cp) + mul(b, s * sp) + mul(mu, cz);
}

struct Queues {
    float4* ext_rays[2];
    uint32_t* ext_slot[2];
    float4* ext_hit4;
    uint2* ext_hit2;
    float4* shd_rays;
    uint32_t* shd_slot;
    float4* prb_rays;
    uint32_t* prb_slot;
    uint32_t* counters;  // [0] next ext, [1] shadow, [2] probe, [3] error, [4..6] ray hand-out
    const uint32_t* ext_count = nullptr;  // device count of the extend queue (graph-captured renders)
    const uint32_t* order = nullptr;      // the shade kernel's visiting order of the extend queue, or none
};

struct Scene_Dev {
    Device_Scene ds;
    const float4* shading;        // 4 float4 per triangle
    const float4* obj_render;     // 7 float4 per object
    const Material_Dev* materials;
    const Rect_Light_Dev* lights;
    const Delta_Light_Dev* delta_lights;
    const Mesh_Light_Dev* mesh_lights;
    const float* mesh_cdf;
    const Sphere_Light_Dev* sphere_lights;
    // environment light (env_map null: none)
    const float4* env_map;
    const float* env_marginal;
    const float* env_cdfs;
    float4 env_l2w[3], env_w2l[3];
    float4 env_scale;  // rgb, -
    int32_t env_nx, env_ny;
    const float4* texels;        // image textures (rgb)
    const uint4* texture_mips;   // width, height, texel offset
    const uint2* textures;       // first mip, mip count
    const float* ewa_weights;    // 256
};

// The device view of an uploaded scene.
inline Scene_Dev scene_dev(const Device_Scene& ds, const Render_Scene& R) {
    Scene_Dev S{};
    S.ds = ds;
    S.shading = reinterpret_cast<const float4*>(R.shading.ptr);
    S.obj_render = reinterpret_cast<const float4*>(R.object_info.ptr);
    S.materials = reinterpret_cast<const Material_Dev*>(R.materials.ptr);
    S.lights = reinterpret_cast<const Rect_Light_Dev*>(R.rect_lights.ptr);
    S.delta_lights = reinterpret_cast<const Delta_Light_Dev*>(R.delta_lights.ptr);
    S.mesh_lights = reinterpret_cast<const Mesh_Light_Dev*>(R.mesh_lights.ptr);
    S.mesh_cdf = reinterpret_cast<const float*>(R.mesh_cdf.ptr);
    S.sphere_lights = reinterpret_cast<const Sphere_Light_Dev*>(R.sphere_lights.ptr);
    S.env_map = R.has_environment ? reinterpret_cast<const float4*>(R.env_map.ptr) : nullptr;
    S.env_marginal = reinterpret_cast<const float*>(R.env_marginal.ptr);
    S.env_cdfs = reinterpret_cast<const float*>(R.env_cdfs.ptr);
    const yar_environment_desc& e = R.environment;
    for (int r = 0; r < 3; r++) {
        S.env_l2w[r] = make_float4(e.light_to_world[4 * r], e.light_to_world[4 * r + 1], e.light_to_world[4 * r + 2],
                                   e.light_to_world[4 * r + 3]);
        S.env_w2l[r] = make_float4(e.world_to_light[4 * r], e.world_to_light[4 * r + 1], e.world_to_light[4 * r + 2],
                                   e.world_to_light[4 * r + 3]);
    }
    S.env_scale = make_float4(e.scale[0], e.scale[1], e.scale[2], 0.f);
    S.env_nx = (int32_t)e.width;
    S.env_ny = (int32_t)e.height;
    S.texels = reinterpret_cast<const float4*>(R.texels.ptr);
    S.texture_mips = reinterpret_cast<const uint4*>(R.texture_mips.ptr);
    S.textures = reinterpret_cast<const uint2*>(R.textures.ptr);
    S.ewa_weights = reinterpret_cast<const float*>(R.ewa_weights.ptr);
    return S;
}

// Warp-aggregated queue append: one atomic per warp and predicate value.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, pred);
    if (!pred) return 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ float one_minus_eps_min(float v) {
    const float ome = __uint_as_float(0x3f7fffffu);  // 0x1.fffffep-1, src/lib/math.h:14
    return v < ome ? v : ome;
}

// ---------------------------------------------------------------- generate
// Stratified_Pixel_Sampler::next_pixel (src/ref/sampling.cpp:98-133) draws,
// from the pixel's pcg stream and in this order: the image samples (2 draws
// per sample), then per 1D dimension spp stratified values and spp - 1
// shuffle draws, then per 2D dimension 2 spp values and spp - 1 shuffle draws.
// The bounded draw of the shuffle takes exactly one number
// (RNG::get_bounded_uint_fast_and_biased, src/lib/random.h:58-62), so every
// dimension starts at a fixed offset of the stream.  Each (pixel, dimension)
// is built by its own thread from a jump-ahead of the stream to that offset
// (Brown, "Random number generation with arbitrary strides", 1994: the LCG
// s' = a s + c advanced n steps is A_n s + C_n c, both computable in
// O(log n)), instead of one thread walking the pixel's stream sequentially.
//
// Sample tables, per pixel of the chunk, dimension-major:
//   s1d[(lp * n1d + dim) * spp + sample],  s2d[(lp * n2d + dim) * spp + sample]
// A thread's column is shuffled in shared memory ([sample][thread], so the
// random indices of a warp's lanes never share a bank) and stored as a
// contiguous row; the lanes of a warp own adjacent rows.

// Advance the pcg stream by n draws.
// The affine map of n LCG steps: state_n = mult * state + plus * inc.
__device__ __forceinline__ void pcg_jump(uint32_t n, uint64_t& acc_mult, uint64_t& acc_plus) {
    uint64_t cur_mult = 6364136223846793005ULL, cur_plus = 1u;  // increment factored out
    acc_mult = 1u;
    acc_plus = 0u;
    while (n) {
        if (n & 1u) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        n >>= 1;
    }
}
__device__ __forceinline__ void pcg_advance(Pcg& r, uint32_t n) {
    uint64_t acc_mult, acc_plus;
    pcg_jump(n, acc_mult, acc_plus);
    r.state = acc_mult * r.state + acc_plus * r.inc;
}

// SplitMix64's output function (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", 2014): a bijective 64-bit mix.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The pcg stream of a pixel: the reference's (initstate 0, sequence = the
// pixel's stream id) when stream_hi is 0; otherwise (independent passes of
// the guided render) sequence and initial state are mixed from the stream id
// and the pass, so that passes share no low-order state bits.
__device__ __forceinline__ Pcg pixel_pcg(const Render_Params& p, uint32_t stream) {
    if (p.stream_hi == 0) return pcg_seed(0, stream);
    const uint64_t key = (uint64_t)stream | ((uint64_t)p.stream_hi << 32);
    return pcg_seed(mix64(key ^ 0x6A09E667F3BCC909ull), mix64(key));
}

__device__ __forceinline__ uint32_t pixel_stream(const Render_Params& p, uint32_t pix, int& x, int& y) {
    x = p.sx0 + (int)(pix % (uint32_t)p.sw);
    y = p.sy0 + (int)(pix / (uint32_t)p.sw);
    uint32_t stream = ((uint32_t)x & 0xffffu) | ((uint32_t)y << 16);
    return stream + p.seed_offset;
}

// One thread per (pixel, table row): row 0 the image samples, rows
// 1..n1d the 1D dimensions, then the 2D dimensions.  Shared memory: spp float2
// per thread.  Stores are float4 when the row length allows.
__global__ void sample_tables_kernel(Render_Params p, uint32_t chunk_first, uint32_t chunk_pixels,
                                     float* __restrict__ s1d, float* __restrict__ s2d,
                                     float2* __restrict__ image_samples) {
    extern __shared__ float2 gen_smem[];
    const uint32_t rows = 1u + (uint32_t)p.n1d + (uint32_t)p.n2d;
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (uint64_t)chunk_pixels * rows) return;
    // row-major over the pixels: a warp builds the same row (the same kind,
    // jump-ahead distance and loop lengths) for 32 pixels
    const uint32_t lp = (uint32_t)(g % chunk_pixels);
    const uint32_t row = (uint32_t)(g / chunk_pixels);
    int x, y;
    Pcg rng = pixel_pcg(p, pixel_stream(p, chunk_first + lp, x, y));
    const int spp = p.spp;
    const uint32_t n1d = (uint32_t)p.n1d;
    float2* sm = gen_smem + threadIdx.x;
    const int stride = (int)blockDim.x;
    const float dx = 1.f / (float)p.nx, dy = 1.f / (float)p.ny;
    if (row == 0) {  // image samples: stratified, not shuffled
        float2* img = image_samples + ((size_t)chunk_first + lp) * spp;
        for (int j = 0; j < p.ny; j++)
            for (int i = 0; i < p.nx; i++) {
                const float a = one_minus_eps_min(((float)i + pcg_float(rng)) * dx);
                const float b = one_minus_eps_min(((float)j + pcg_float(rng)) * dy);
                img[j * p.nx + i] = make_float2(a, b);
            }
        return;
    }
    if (row <= n1d) {
        const uint32_t dim = row - 1u;
        pcg_advance(rng, (uint32_t)(2 * spp) + (p.arrays_2d_first ? (uint32_t)p.n2d * (uint32_t)(3 * spp - 1) : 0u) +
                             dim * (uint32_t)(2 * spp - 1));
        const float d = 1.f / (float)spp;
        for (int k = 0; k < spp; k++) sm[k * stride].x = one_minus_eps_min(((float)k + pcg_float(rng)) * d);
        for (int m = spp; m > 1; m--) {  // shuffle, src/lib/math.h:138-145
            const uint32_t r = pcg_bounded_fast(rng, (uint32_t)m);
            const float t = sm[(m - 1) * stride].x;
            sm[(m - 1) * stride].x = sm[r * stride].x;
            sm[r * stride].x = t;
        }
        float* out = s1d + ((size_t)lp * n1d + dim) * spp;
        if ((spp & 3) == 0) {
            float4* o4 = reinterpret_cast<float4*>(out);
            for (int k = 0; k < spp; k += 4)
                o4[k >> 2] = make_float4(sm[k * stride].x, sm[(k + 1) * stride].x, sm[(k + 2) * stride].x,
                                         sm[(k + 3) * stride].x);
        } else {
            for (int k = 0; k < spp; k++) out[k] = sm[k * stride].x;
        }
        return;
    }
    const uint32_t dim = row - 1u - n1d;
    pcg_advance(rng, (uint32_t)(2 * spp) + (p.arrays_2d_first ? 0u : n1d * (uint32_t)(2 * spp - 1)) +
                         dim * (uint32_t)(3 * spp - 1));
    for (int j = 0; j < p.ny; j++)
        for (int i = 0; i < p.nx; i++) {
            const float a = one_minus_eps_min(((float)i + pcg_float(rng)) * dx);
            const float b = one_minus_eps_min(((float)j + pcg_float(rng)) * dy);
            sm[(j * p.nx + i) * stride] = make_float2(a, b);
        }
    for (int m = spp; m > 1; m--) {
        const uint32_t r = pcg_bounded_fast(rng, (uint32_t)m);
        const float2 t = sm[(m - 1) * stride];
        sm[(m - 1) * stride] = sm[r * stride];
        sm[r * stride] = t;
    }
    float2* out = reinterpret_cast<float2*>(s2d) + ((size_t)lp * (uint32_t)p.n2d + dim) * spp;
    if ((spp & 1) == 0) {
        float4* o4 = reinterpret_cast<float4*>(out);
        for (int k = 0; k < spp; k += 2) {
            const float2 a = sm[k * stride], b = sm[(k + 1) * stride];
            o4[k >> 1] = make_float4(a.x, a.y, b.x, b.y);
        }
    } else {
        for (int k = 0; k < spp; k++) out[k] = sm[k * stride];
    }
}

// Camera::generate_ray (src/ref/camera.cpp:16-31) through film position (fx, fy).
__device__ __forceinline__ void camera_ray(const yar_camera_desc& c, float fx, float fy, V3& o, V3& d) {
    const float4 m0 = make_float4(c.camera_to_world[0], c.camera_to_world[1], c.camera_to_world[2], c.camera_to_world[3]);
    const float4 m1 = make_float4(c.camera_to_world[4], c.camera_to_world[5], c.camera_to_world[6], c.camera_to_world[7]);
    const float4 m2 = make_float4(c.camera_to_world[8], c.camera_to_world[9], c.camera_to_world[10], c.camera_to_world[11]);
    const float u = 2.f * (fx / c.image_extent[0]) - 1.f;
    const float v = 2.f * (fy / c.image_extent[1]) - 1.f;
    const float right = u * c.horz_half_dist;
    const float up = -v * c.vert_half_dist;
    V3 dir = v3(right, c.z_is_up ? 1.f : up, c.z_is_up ? up : -1.f);
    dir = divs(dir, len(dir));
    o = xform_point(m0, m1, m2, v3(0.f, 0.f, 0.f));
    d = xform_vector(m0, m1, m2, dir);
}

// One thread per path of the chunk: camera ray (Camera::generate_ray,
// src/ref/camera.cpp) through the path's image sample, path initialisation.
__global__ void __launch_bounds__(kBlock)
camera_kernel(Render_Params p, uint32_t chunk_first, uint32_t chunk_paths, const float2* __restrict__ image_samples,
              Path_State ps, Queues q) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= chunk_paths) return;
    const int spp = p.spp;
    const uint32_t lp = slot / (uint32_t)spp;
    const uint32_t k = slot - lp * (uint32_t)spp;
    int x, y;
    const uint32_t stream = pixel_stream(p, chunk_first + lp, x, y);
    const float2 s = image_samples[((size_t)chunk_first + lp) * spp + k];
    V3 o, d;
    camera_ray(p.camera, (float)x + s.x, (float)y + s.y, o, d);
    q.ext_rays[0][2 * (size_t)slot] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
    q.ext_rays[0][2 * (size_t)slot + 1] = make_float4(d.x, d.y, d.z, 0.f);
    q.ext_slot[0][slot] = slot;
    ps.coeff[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
    ps.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    ps.info[slot] = 0u;
    // dimensions beyond the sampler budget: an independent pcg stream per sample
    const uint64_t seq2 = ((uint64_t)stream << 20) ^ 0x2545F4914F6CDD1Dull;
    const Pcg r2 = pcg_seed((uint64_t)k + 1u,
                            p.stream_hi ? mix64(seq2 + (uint64_t)p.stream_hi * 0x9E3779B97F4A7C15ull) : seq2);
    ps.rng[slot] = make_uint4((uint32_t)r2.state, (uint32_t)(r2.state >> 32), (uint32_t)r2.inc,
                              (uint32_t)(r2.inc >> 32));
    if (p.exact_tail) ps.rng_draws[slot] = 0u;
}

// ---------------------------------------------------------------- extend / probe / shadow
// The three ray queues of a bounce are traced by the cast kernels (cast.cu).
// Extend hits are written at the queue position (shade reads the queue in
// order); shadow and probe results at the path slot.  Hand-out counters are
// counters[4..6], the error word counters[3].
//
// The traversal kernel is chosen per ray kind and per bounce (camera rays,
// the first bounces and the deep, sparse, incoherent ones favour different
// kernels): the first kRenderTuneQueues queues of at least kRenderTuneMinRays
// rays of a bounce bucket after a scene upload are traced by every kernel and
// timed, and the kernel of the least summed time is kept (a queue's results
// are the same whichever ran last).  A bucket timed on fewer queues by the
// end of the first render takes its best so far.  The deep bucket covers
// bounces 4 and later, whose queues shrink: one queue alone picked a kernel
// that was 8% slower on C3 in one of four scene uploads.  The MIS probe queue
// uses the extend queue's choice.  A context option can fix the kernel.
constexpr uint32_t kRenderTuneMinRays = 1u << 16;
constexpr int kRenderTuneQueues = 3;

inline void fix_render_bucket(yar_gpu_ctx* ctx, int kind, int bucket) {
    const float* ms = ctx->render_tune_ms[kind][bucket];
    int best = 0;
    for (int k = 1; k < kCastKernelCount; k++)
        if (ms[k] < ms[best]) best = k;
    ctx->render_kernel[kind][bucket] = best;
}

// Times every kernel on this queue (its results stay in place) and adds the
// times to the bucket's sums; fixes the bucket after kRenderTuneQueues queues.
inline cudaError_t tune_render_bucket(yar_gpu_ctx* ctx, const Cast_Args& a, int kind, int bucket, cudaStream_t st) {
    static_assert(kCastKernelCount == 4, "tuning sums per kernel");
    float ms[kCastKernelCount];
    const bool first = ctx->render_tune_queues[kind][bucket] == 0;
    cudaError_t e = time_cast_kernels(ctx->ds, a, kind == 1, st, ctx->ev_start, ctx->ev_stop, 1, first, ms);
    if (e != cudaSuccess) return e;
    for (int k = 0; k < kCastKernelCount; k++) ctx->render_tune_ms[kind][bucket][k] += ms[k];
    if (++ctx->render_tune_queues[kind][bucket] >= kRenderTuneQueues) fix_render_bucket(ctx, kind, bucket);
    return cudaSuccess;
}

// After the first render: buckets timed on fewer queues take their best so far.
inline void finish_render_tuning(yar_gpu_ctx* ctx) {
    for (int kind = 0; kind < 2; kind++)
        for (int b = 0; b < yar_gpu_ctx::kBounceBuckets; b++)
            if (ctx->render_kernel[kind][b] < 0 && ctx->render_tune_queues[kind][b] > 0) fix_render_bucket(ctx, kind, b);
}

inline int bounce_bucket(int bounce) { return bounce < yar_gpu_ctx::kBounceBuckets ? bounce : yar_gpu_ctx::kBounceBuckets - 1; }

// The kernel a bounce runs with: its own choice, else the choice of the
// nearest earlier bounce (queues too short to time follow the bounce before
// them), else the persistent 64-register kernel.
inline int render_choice(const yar_gpu_ctx* ctx, int kind, int bounce) {
    for (int b = bounce_bucket(bounce); b >= 0; b--)
        if (ctx->render_kernel[kind][b] >= 0) return ctx->render_kernel[kind][b];
    return kCastPersistent64;
}

cudaError_t trace_extend(yar_gpu_ctx* ctx, const Queues& q, int cur, uint32_t count, int bounce, cudaStream_t st) {
    Cast_Args a;
    a.rays = q.ext_rays[cur];
    a.n = count;
    a.next_ray = q.counters + 4;
    a.err = reinterpret_cast<int*>(q.counters + 3);
    a.hit4 = q.ext_hit4;
    a.hit2 = q.ext_hit2;
    const int b = bounce_bucket(bounce);
    if (ctx->render_kernel[0][b] < 0 && count >= kRenderTuneMinRays) return tune_render_bucket(ctx, a, 0, b, st);
    return launch_extend(ctx->ds, a, render_choice(ctx, 0, bounce), st);
}

cudaError_t trace_light_queues(yar_gpu_ctx* ctx, const Queues& q, const Path_State& ps, uint32_t count, int bounce,
                               cudaStream_t st) {
    Cast_Args sh;
    sh.rays = q.shd_rays;
    sh.count = q.counters + 1;
    sh.n_max = count;
    sh.perm = q.shd_slot;
    sh.next_ray = q.counters + 5;
    sh.err = reinterpret_cast<int*>(q.counters + 3);
    sh.occluded = ps.occluded;
    const int b = bounce_bucket(bounce);
    cudaError_t e = (ctx->render_kernel[1][b] < 0 && count >= kRenderTuneMinRays)
                        ? tune_render_bucket(ctx, sh, 1, b, st)
                        : launch_shadow(ctx->ds, sh, render_choice(ctx, 1, bounce), st);
    if (e != cudaSuccess) return e;
    Cast_Args pr;
    pr.rays = q.prb_rays;
    pr.count = q.counters + 2;
    pr.n_max = count;
    pr.perm = q.prb_slot;
    pr.next_ray = q.counters + 6;
    pr.err = reinterpret_cast<int*>(q.counters + 3);
    pr.hit4 = ps.probe_hit4;
    pr.hit2 = ps.probe_hit2;
    return launch_extend(ctx->ds, pr, render_choice(ctx, 0, bounce), st);
}

// ---------------------------------------------------------------- shading context
// Shading_Context::initialize_local_geometry + init_from_triangle_mesh_intersection
// (src/ref/shading_context.cpp:65-172, :188-240), constant materials, no bump.
__device__ __forceinline__ void init_shading(const Scene_Dev& S, V3 ray_d, uint32_t object, uint32_t prim, float b0,
                                             float b1, float b2, Shading& sc, int4& info) {
    const float4* orec = S.ds.objects + 6 * (size_t)object;
    const uint32_t tri_offset = __float_as_uint(__ldg(orec + 4).w);
    const float4* rrec = S.obj_render + 7 * (size_t)object;
    const float4 w0 = __ldg(rrec + 0), w1 = __ldg(rrec + 1), w2 = __ldg(rrec + 2);
    const float4 n0 = __ldg(rrec + 3), n1 = __ldg(rrec + 4), n2 = __ldg(rrec + 5);
    const float4 inf4 = __ldg(rrec + 6);
    info = make_int4(__float_as_int(inf4.x), __float_as_int(inf4.y), __float_as_int(inf4.z), __float_as_int(inf4.w));
    const size_t g = (size_t)tri_offset + prim;
    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1), q2 = __ldg(S.ds.tris + 3 * g + 2);
    const V3 p0 = v3(q0.x, q0.y, q0.z), p1 = v3(q1.x, q1.y, q1.z), p2 = v3(q2.x, q2.y, q2.z);
    const float4 h0 = __ldg(S.shading + 4 * g), h1 = __ldg(S.shading + 4 * g + 1);
    const float4 h2 = __ldg(S.shading + 4 * g + 2), h3 = __ldg(S.shading + 4 * g + 3);
    const uint32_t flags = __float_as_uint(h3.w);

    sc.wo = -normalized(ray_d);
    V3 position = bary(p0, p1, p2, b0, b1, b2);
    V3 gn = normalized(cross(p1 - p0, p2 - p0));
    if (flags & 4u) gn = -gn;
    V3 normal = gn;
    if (flags & 1u) {
        const V3 in = bary(v3(h0.x, h0.y, h0.z), v3(h1.x, h1.y, h1.z), v3(h2.x, h2.y, h2.z), b0, b1, b2);
        if (len2(in) != 0.f) normal = normalized(in);
    }
    const bool has_uv = (flags & 2u) != 0;
    V3 dpdu = v3(0.f, 0.f, 0.f);
    if (has_uv) {
        // uvs: u0 = h0.w, v0 = h1.w, u1 = h2.w, v1 = h3.x, u2 = h3.y, v2 = h3.z
        const float a00 = h2.w - h0.w, a01 = h3.x - h1.w, a10 = h3.y - h0.w, a11 = h3.z - h1.w;
        const V3 bp0 = p1 - p0, bp1 = p2 - p0;
        const float det = a00 * a11 - a01 * a10;  // solve_linear_system_2x2, src/lib/math.cpp:8-16
        if (det != 0.f) {
            const float inv_det = 1.f / det;
            dpdu = mul(mul(bp0, a11) - mul(bp1, a01), inv_det);
        }
        if (fabsf(det) < 1e-9f) dpdu = coordinate_axis(gn);
    }
    position = xform_point(make_float4(w0.x, w0.y, w0.z, w0.w), w1, w2, position);
    normal = xform_vector(n0, n1, n2, normal);
    normal = divs(normal, len(normal));
    gn = xform_vector(n0, n1, n2, gn);
    gn = divs(gn, len(gn));
    dpdu = xform_vector(w0, w1, w2, dpdu);
    if (dot(normal, gn) == 0.f) gn = normal;
    if (dot(gn, sc.wo) < 0) gn = -gn;
    sc.flipped = false;
    if (dot(normal, gn) < 0) {
        normal = -normal;
        sc.flipped = true;
    }
    offset_axis(position.x, gn.x, sc.origin_pos.x, sc.origin_neg.x);
    offset_axis(position.y, gn.y, sc.origin_pos.y, sc.origin_neg.y);
    offset_axis(position.z, gn.z, sc.origin_pos.z, sc.origin_neg.z);
    normal = adjust_shading_normal(sc.wo, gn, normal);
    V3 dpdu_shading;
    if (!has_uv) {
        dpdu_shading = coordinate_axis(normal);
    } else if (fabsf(dot(normal, gn) - 1.f) < 1e-6f) {
        dpdu_shading = dpdu;
    } else {
        const V3 t = cross(dpdu, normal);
        dpdu_shading = mul(normalized(cross(normal, t)), len(dpdu));
    }
    sc.position = position;
    sc.ng = gn;
    sc.n = normal;
    sc.dpdu_shading = dpdu_shading;
}

// A path's view of its pixel's sample tables: dimension i of this sample is
// s1d[i * spp] (s1d already offset to the sample).
struct Dims {
    const float* s1d;
    const float2* s2d;
    int n1d, n2d, i1d, i2d, spp;
    Pcg rng;
    bool rng_used;
    uint32_t draws;  // pcg draws past the budget
};
__device__ __forceinline__ float next1d(Dims& d) {
    if (d.i1d < d.n1d) return d.s1d[(size_t)(d.i1d++) * d.spp];
    d.rng_used = true;
    d.draws += 1u;
    return pcg_float(d.rng);
}
__device__ __forceinline__ float2 next2d(Dims& d) {
    if (d.i2d < d.n2d) return d.s2d[(size_t)(d.i2d++) * d.spp];
    d.rng_used = true;
    d.draws += 2u;
    const float a = pcg_float(d.rng);
    const float b = pcg_float(d.rng);
    return make_float2(a, b);
}

// Whether the vertex a path reaches next may take a draw past the sampler
// budget: a vertex takes 3 1D and 3 2D dimensions, one more 1D for the
// Russian roulette after a delta arrival and one for the roulette after the
// continuation.
__device__ __forceinline__ bool tail_may_draw_past_budget(const Render_Params& p, uint32_t info) {
    const int bounce = (int)(info & 0xffu);
    const int i1d = (int)((info >> 8) & 0xffu), i2d = (int)((info >> 16) & 0xffu);
    const int n1 = 3 + ((info & kDeltaArrival) && bounce >= p.rr_bounce_threshold ? 1 : 0) +
                   (bounce + 1 >= p.rr_bounce_threshold ? 1 : 0);
    return i1d + n1 > p.n1d || i2d + 3 > p.n2d;
}

// ---------------------------------------------------------------- triangle-mesh lights
// The light's normal at barycentrics b of global triangle g: the interpolated
// vertex normal (not normalised) or the geometric normal
// (Triangle_Mesh::get_normal / get_geometric_normal, src/lib/triangle_mesh.h:61-77).
__device__ __forceinline__ V3 mesh_light_normal(const Scene_Dev& S, size_t g, float b0, float b1, float b2) {
    const float4 h0 = __ldg(S.shading + 4 * g), h1 = __ldg(S.shading + 4 * g + 1);
    const float4 h2 = __ldg(S.shading + 4 * g + 2), h3 = __ldg(S.shading + 4 * g + 3);
    const uint32_t flags = __float_as_uint(h3.w);
    if (flags & 1u) return bary(v3(h0.x, h0.y, h0.z), v3(h1.x, h1.y, h1.z), v3(h2.x, h2.y, h2.z), b0, b1, b2);
    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1), q2 = __ldg(S.ds.tris + 3 * g + 2);
    const V3 p0 = v3(q0.x, q0.y, q0.z);
    const V3 gn = normalized(cross(v3(q1.x, q1.y, q1.z) - p0, v3(q2.x, q2.y, q2.z) - p0));
    return (flags & 4u) ? -gn : gn;
}

// Diffuse_Triangle_Mesh_Light_Sampler::sample (light_sampling.cpp:126-161): a
// triangle by sample_from_CDF over the area CDF (sampling.cpp:98-147), the
// remapped first sample and the second one give uniform barycentrics
// (uniform_sample_triangle_baricentrics, sampling.cpp:69-77).  pdf is per solid
// angle from shading_pos, 0 on the light's back side.
__device__ __forceinline__ V3 mesh_light_sample(const Scene_Dev& S, uint4 info, float mesh_area, float u0, float u1,
                                                V3 shading_pos, float& pdf) {
    const float* cdf = S.mesh_cdf + info.z;
    const uint32_t n = info.y;
    uint32_t lo = 0, hi = n;  // std::lower_bound
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) < u0) lo = mid + 1;
        else hi = mid;
    }
    const uint32_t k = lo < n ? lo : n - 1;
    const float cdf_a = k == 0 ? 0.f : __ldg(cdf + k - 1), cdf_b = __ldg(cdf + k);
    const float fraction = (u0 - cdf_a) / (cdf_b - cdf_a);
    const float x = one_minus_eps_min(((float)k + fraction) * (1.f / (float)n));
    const float remapped = one_minus_eps_min(fraction);
    uint32_t tri = (uint32_t)(x * (float)n);
    if (tri > n - 1) tri = n - 1;
    const float a = sqrtf(remapped);
    const float b0 = 1 - a, b1 = u1 * a;
    const float b2 = 1.f - b0 - b1;
    const size_t g = (size_t)info.x + tri;
    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1), q2 = __ldg(S.ds.tris + 3 * g + 2);
    const V3 light_p = bary(v3(q0.x, q0.y, q0.z), v3(q1.x, q1.y, q1.z), v3(q2.x, q2.y, q2.z), b0, b1, b2);
    const V3 light_n = mesh_light_normal(S, g, b0, b1, b2);
    const V3 lv = light_p - shading_pos;
    const float d2 = len2(lv);
    const V3 wi = divs(lv, sqrtf(d2));
    const float lndw = dot(light_n, -wi);
    pdf = lndw <= 0.f ? 0.f : d2 / (lndw * mesh_area);
    return light_p;
}

// ---------------------------------------------------------------- environment light
// Environment_Light_Sampler (light_sampling.cpp:11-71) and Distribution_2D
// (sampling.cpp:185-291) over the map's mip 0.  atan2 and acos are rounded
// correctly (evaluated in double), like the sines and cosines.
__device__ __forceinline__ Col env_texel(const Scene_Dev& S, int x, int y) {  // get_texel_clamp
    x = x < 0 ? 0 : (S.env_nx - 1 < x ? S.env_nx - 1 : x);
    y = y < 0 ? 0 : (S.env_ny - 1 < y ? S.env_ny - 1 : y);
    const float4 t = __ldg(S.env_map + (size_t)y * S.env_nx + x);
    return col(t.x, t.y, t.z);
}
__device__ __forceinline__ Col env_nearest(const Scene_Dev& S, float u, float v) {
    return env_texel(S, (int)(u * (float)S.env_nx), (int)(v * (float)S.env_ny));
}
__device__ __forceinline__ Col env_bilinear(const Scene_Dev& S, float u, float v) {
    const float x = u * (float)S.env_nx - 0.5f, y = v * (float)S.env_ny - 0.5f;
    const float x_floor = floorf(x), y_floor = floorf(y);
    const float wx = x - x_floor, wy = y - y_floor;
    const int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    return ((mul(env_texel(S, x0, y0), (1 - wy) * (1 - wx)) + mul(env_texel(S, x1, y0), (1 - wy) * wx)) +
            mul(env_texel(S, x0, y1), wy * (1 - wx))) +
           mul(env_texel(S, x1, y1), wy * wx);
}
__device__ __forceinline__ void env_uv(V3 d, float& u, float& v) {  // get_uv_from_direction
    const float pi2 = 6.2831853f;  // src/lib/math.h:10
    float phi = (float)atan2((double)d.y, (double)d.x);
    phi = phi < 0 ? phi + pi2 : phi;
    const float z = d.z < -1.f ? -1.f : (1.f < d.z ? 1.f : d.z);
    const float theta = (float)acos((double)z);
    const float a = phi * (1.f / pi2);
    u = a < 0.f ? 0.f : one_minus_eps_min(a);
    v = one_minus_eps_min(theta * (1.f / kPi));
}
__device__ __forceinline__ Col env_radiance(const Scene_Dev& S, V3 world_dir, bool filtered) {
    float u, v;
    env_uv(xform_vector(S.env_w2l[0], S.env_w2l[1], S.env_w2l[2], world_dir), u, v);
    const Col c = filtered ? env_bilinear(S, u, v) : env_nearest(S, u, v);
    return c * col(S.env_scale.x, S.env_scale.y, S.env_scale.z);
}
__device__ __forceinline__ float env_light_pdf(const Scene_Dev& S, V3 world_dir) {
    const V3 d = xform_vector(S.env_w2l[0], S.env_w2l[1], S.env_w2l[2], world_dir);
    float u, v;
    env_uv(d, u, v);
    const int x = (int)(u * (float)S.env_nx), y = (int)(v * (float)S.env_ny);
    const float pdf_y = (__ldg(S.env_marginal + y) - (y == 0 ? 0.f : __ldg(S.env_marginal + y - 1))) * (float)S.env_ny;
    const float* c = S.env_cdfs + (size_t)y * S.env_nx;
    const float pdf_x = (__ldg(c + x) - (x == 0 ? 0.f : __ldg(c + x - 1))) * (float)S.env_nx;
    const float sin_theta = sqrtf(max_std(0.f, 1.f - d.z * d.z));
    return (pdf_y * pdf_x) / (2 * kPi * kPi * sin_theta);
}
// sample_from_CDF (sampling.cpp:98-147): the sample, its pdf and interval
__device__ __forceinline__ float cdf_sample(const float* cdf, int n, float u, float& pdf, int& index) {
    int lo = 0, hi = n;  // std::lower_bound
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) < u) lo = mid + 1;
        else hi = mid;
    }
    const int k = lo < n ? lo : n - 1;
    const float a = k == 0 ? 0.f : __ldg(cdf + k - 1), b = __ldg(cdf + k);
    const float fraction = (u - a) / (b - a);
    pdf = (b - a) * (float)n;
    index = k;
    return one_minus_eps_min(((float)k + fraction) * (1.f / (float)n));
}
__device__ __forceinline__ Col env_light_sample(const Scene_Dev& S, float u0, float u1, V3& wi, float& pdf) {
    float pdf_y, pdf_x;
    int y, x;
    const float ky = cdf_sample(S.env_marginal, S.env_ny, u0, pdf_y, y);
    const float kx = cdf_sample(S.env_cdfs + (size_t)y * S.env_nx, S.env_nx, u1, pdf_x, x);
    const float phi = kx * 6.2831853f, theta = ky * kPi;
    const float sin_theta = sin_f(theta);
    pdf = (pdf_y * pdf_x) / (2 * kPi * kPi * sin_theta);
    wi = xform_vector(S.env_l2w[0], S.env_l2w[1], S.env_l2w[2],
                      v3(sin_theta * cos_f(phi), sin_theta * sin_f(phi), cos_f(theta)));
    return env_nearest(S, kx, ky) * col(S.env_scale.x, S.env_scale.y, S.env_scale.z);
}

// ---------------------------------------------------------------- image textures
// Image_Texture (src/ref/image_texture.cpp) over the reference's mip chain
// and evaluate_texture_parameter (src/ref/parameter_evaluation.cpp:10-31):
// EWA filtering with repeat wrapping.  log2 of the footprint and the filter
// weights are rounded correctly (double evaluation), like the sines and cosines.
__device__ __forceinline__ Col texel_repeat(const Scene_Dev& S, uint4 mip, int x, int y) {  // get_texel_repeat
    const int w = (int)mip.x, h = (int)mip.y;
    if (x >= 0) x &= w - 1;
    else { x %= w; x += (x >> 31) & w; }
    if (y >= 0) y &= h - 1;
    else { y %= h; y += (y >> 31) & h; }
    const float4 t = __ldg(S.texels + mip.z + (size_t)y * (size_t)w + (size_t)x);
    return col(t.x, t.y, t.z);
}
__device__ __forceinline__ Col texture_bilinear(const Scene_Dev& S, uint4 mip, float u, float v) {
    const float x = u * (float)mip.x - 0.5f, y = v * (float)mip.y - 0.5f;
    const float x_floor = floorf(x), y_floor = floorf(y);
    const float wx = x - x_floor, wy = y - y_floor;
    const int x0 = (int)x_floor, y0 = (int)y_floor, x1 = x0 + 1, y1 = y0 + 1;
    return ((mul(texel_repeat(S, mip, x0, y0), (1 - wy) * (1 - wx)) +
             mul(texel_repeat(S, mip, x1, y0), (1 - wy) * wx)) +
            mul(texel_repeat(S, mip, x0, y1), wy * (1 - wx))) +
           mul(texel_repeat(S, mip, x1, y1), wy * wx);
}
// Texels from lo to lo + span (span = hi - lo of integer-valued floats): 0 for
// an empty or NaN span, at most 513.
__device__ __forceinline__ int ewa_trip_count(float span) {
    return span >= 0.f ? (span < 512.f ? (int)span + 1 : 513) : 0;
}
// do_EWA (image_texture.cpp:501-578) on one mip
__device__ __noinline__ Col texture_ewa_level(const Scene_Dev& S, uint4 mip, float u, float v, float2 a1, float2 a2) {
    const float w = (float)mip.x, h = (float)mip.y;
    u = u * w - 0.5f;
    v = v * h - 0.5f;
    const float a1x = a1.x * w, a1y = a1.y * h, a2x = a2.x * w, a2y = a2.y * h;
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
    Col sum = col(0.f, 0.f, 0.f);
    float weight_sum = 0.f;
    // The reference steps float counters (y++) over the footprint and asserts
    // u_delta, v_delta < 256.  Integer trip counts visit the same integer-valued
    // x and y (exact below 2^24) and end even outside that domain, where a
    // float counter stops advancing; they are capped at the 513 texels per axis
    // that the assertion allows (upload also refuses uv ranges that reach 2^22).
    const int nx = ewa_trip_count(x1 - x0), ny = ewa_trip_count(y1 - y0);
    for (int iy = 0; iy < ny; iy++) {
        const float y = y0 + (float)iy;
        const float yy = y - v;
        for (int ix = 0; ix < nx; ix++) {
            const float x = x0 + (float)ix;
            const float xx = x - u;
            const float r2 = A * xx * xx + B * xx * yy + C * yy * yy;
            if (r2 < 1.f) {
                const float wt = __ldg(S.ewa_weights + (int)(r2 * 256));
                sum = sum + mul(texel_repeat(S, mip, (int)x, (int)y), wt);
                weight_sum += wt;
            }
        }
    }
    return mul(sum, 1.f / weight_sum);
}
// Image_Texture::sample_EWA (image_texture.cpp:580-615), max anisotropy 32
__device__ Col texture_ewa(const Scene_Dev& S, uint2 tex, float u, float v, float2 a1, float2 a2) {
    float l1 = a1.x * a1.x + a1.y * a1.y, l2 = a2.x * a2.x + a2.y * a2.y;
    if (l1 < l2) {
        const float2 t = a1;
        a1 = a2;
        a2 = t;
        const float tl = l1;
        l1 = l2;
        l2 = tl;
    }
    const float major_length = sqrtf(l1);
    float minor_length = sqrtf(l2);
    if (minor_length < 1e-6f) return texture_bilinear(S, __ldg(S.texture_mips + tex.x), u, v);
    if (minor_length * 32.f < major_length) {
        const float scale = major_length / (minor_length * 32.f);
        minor_length *= scale;
        a2.x *= scale;
        a2.y *= scale;
    }
    const float lod = max_std(0.f, (float)((int)tex.y - 1) + (float)log2((double)minor_length));
    const float lod_floor = truncf(lod);  // std::modf of a non-negative value
    const float frac = lod - lod_floor;
    const int level0 = (int)lod_floor;
    if (level0 >= (int)tex.y - 1) {
        const float4 c = __ldg(S.texels + __ldg(S.texture_mips + tex.x + tex.y - 1).z);
        return col(c.x, c.y, c.z);
    }
    const Col c0 = texture_ewa_level(S, __ldg(S.texture_mips + tex.x + level0), u, v, a1, a2);
    const Col c1 = texture_ewa_level(S, __ldg(S.texture_mips + tex.x + level0 + 1), u, v, a1, a2);
    return mul(c0, 1.f - frac) + mul(c1, frac);  // lerp, src/lib/math.h:82-85
}

// The hit's uv and world-space dpdu/dpdv (init_from_triangle_mesh_intersection,
// src/ref/shading_context.cpp:209-223); false without uvs.
__device__ bool texture_geometry(const Scene_Dev& S, uint32_t object, uint32_t prim, float b0, float b1, float b2,
                                 float2& uv, V3& dpdu, V3& dpdv) {
    const float4* orec = S.ds.objects + 6 * (size_t)object;
    const uint32_t tri_offset = __float_as_uint(__ldg(orec + 4).w);
    const size_t g = (size_t)tri_offset + prim;
    const float4 h0 = __ldg(S.shading + 4 * g), h1 = __ldg(S.shading + 4 * g + 1);
    const float4 h2 = __ldg(S.shading + 4 * g + 2), h3 = __ldg(S.shading + 4 * g + 3);
    const uint32_t flags = __float_as_uint(h3.w);
    if (!(flags & 2u)) return false;
    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1), q2 = __ldg(S.ds.tris + 3 * g + 2);
    const V3 p0 = v3(q0.x, q0.y, q0.z), p1 = v3(q1.x, q1.y, q1.z), p2 = v3(q2.x, q2.y, q2.z);
    V3 gn = normalized(cross(p1 - p0, p2 - p0));
    if (flags & 4u) gn = -gn;
    // uvs: u0 = h0.w, v0 = h1.w, u1 = h2.w, v1 = h3.x, u2 = h3.y, v2 = h3.z
    uv = make_float2(h0.w * b0 + h2.w * b1 + h3.y * b2, h1.w * b0 + h3.x * b1 + h3.z * b2);
    const float a00 = h2.w - h0.w, a01 = h3.x - h1.w, a10 = h3.y - h0.w, a11 = h3.z - h1.w;
    const V3 bp0 = p1 - p0, bp1 = p2 - p0;
    const float det = a00 * a11 - a01 * a10;
    dpdu = v3(0.f, 0.f, 0.f);
    dpdv = v3(0.f, 0.f, 0.f);
    if (det != 0.f) {
        const float inv_det = 1.f / det;
        dpdu = mul(mul(bp0, a11) - mul(bp1, a01), inv_det);
        dpdv = mul(mul(bp0, -a10) + mul(bp1, a00), inv_det);
    }
    if (fabsf(det) < 1e-9f) {
        dpdu = coordinate_axis(gn);
        dpdv = cross(gn, dpdu);
    }
    const float4* rrec = S.obj_render + 7 * (size_t)object;
    const float4 w0 = __ldg(rrec + 0), w1 = __ldg(rrec + 1), w2 = __ldg(rrec + 2);
    dpdu = xform_vector(w0, w1, w2, dpdu);
    dpdv = xform_vector(w0, w1, w2, dpdv);
    return true;
}

// Shading_Context::calculate_dxdy_derivatives + calculate_uv_derivates
// (shading_context.cpp:242-333): where the differential rays (ox, dx) and
// (oy, dy) cross the hit's plane, and the uv derivatives there.  False when
// the sanity check drops them (has_dxdy_derivatives false: all zero).
__device__ bool dxdy_derivatives(const Shading& sc, V3 ox, V3 dx, V3 oy, V3 dy, V3 dpdu, V3 dpdv, V3& dpdx, V3& dpdy,
                                 float2& duvdx, float2& duvdy) {
    const V3 gn = sc.ng;
    const float plane_d = -dot(gn, sc.position);
    dpdx = v3(0.f, 0.f, 0.f);
    dpdy = v3(0.f, 0.f, 0.f);
    auto plane_t = [&](V3 o, V3 d) {  // ray_plane_intersection, src/lib/math.cpp:27-31
        const float k = -dot(o, gn) - plane_d;
        return k == 0 ? 0.f : k / dot(d, gn);
    };
    const float tx = plane_t(ox, dx);
    if (fabsf(tx) != __int_as_float(0x7f800000)) dpdx = (ox + mul(dx, tx)) - sc.position;
    const float ty = plane_t(oy, dy);
    if (fabsf(ty) != __int_as_float(0x7f800000)) dpdy = (oy + mul(dy, ty)) - sc.position;
    const float ax = fabsf(gn.x), ay = fabsf(gn.y), az = fabsf(gn.z);
    const int dim0 = (ax > ay && ax > az) ? 1 : 0;
    const int dim1 = (ax > ay && ax > az) ? 2 : (ay > az ? 2 : 1);
    auto comp = [](V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); };
    const float a00 = comp(dpdu, dim0), a01 = comp(dpdv, dim0), a10 = comp(dpdu, dim1), a11 = comp(dpdv, dim1);
    const float det = a00 * a11 - a01 * a10;  // solve_linear_system_2x2, src/lib/math.cpp:8-16
    duvdx = make_float2(0.f, 0.f);
    duvdy = make_float2(0.f, 0.f);
    if (det != 0.f) {
        const float inv_det = 1.f / det;
        duvdx = make_float2((a11 * comp(dpdx, dim0) - a01 * comp(dpdx, dim1)) * inv_det,
                            (-a10 * comp(dpdx, dim0) + a00 * comp(dpdx, dim1)) * inv_det);
        duvdy = make_float2((a11 * comp(dpdy, dim0) - a01 * comp(dpdy, dim1)) * inv_det,
                            (-a10 * comp(dpdy, dim0) + a00 * comp(dpdy, dim1)) * inv_det);
    }
    if (fabsf(duvdx.x) > 1e9f || fabsf(duvdx.y) > 1e9f || fabsf(duvdy.x) > 1e9f || fabsf(duvdy.y) > 1e9f) {
        duvdx = make_float2(0.f, 0.f);
        duvdy = make_float2(0.f, 0.f);
        dpdx = v3(0.f, 0.f, 0.f);
        dpdy = v3(0.f, 0.f, 0.f);
        return false;
    }
    return true;
}

// The differential rays a hit's derivatives come from (trace_ray's
// differential_rays argument, src/ref/path_tracing.cpp:25, :86-87): at bounce
// 0 the camera ray's, one pixel over and scaled to the sample's footprint
// (src/ref/reference_renderer.cpp:367-378); where a delta ray arrives, the
// specular differential rays it carries (kDiffRays); else none.
__device__ __noinline__ bool incoming_differentials(const Render_Params& p, const Path_State& ps, uint32_t slot,
                                                   int bounce, uint32_t info, V3& ox, V3& dx, V3& oy, V3& dy) {
    if (bounce == 0) {
        const uint32_t lp = slot / (uint32_t)p.spp, k = slot - lp * (uint32_t)p.spp;
        int x, y;
        pixel_stream(p, ps.chunk_first + lp, x, y);
        const float2 fs = ps.image_samples[((size_t)ps.chunk_first + lp) * (uint32_t)p.spp + k];
        const float fx = (float)x + fs.x, fy = (float)y + fs.y;
        V3 d, o1;
        camera_ray(p.camera, fx, fy, ox, d);
        camera_ray(p.camera, fx + 1.f, fy, o1, dx);
        camera_ray(p.camera, fx, fy + 1.f, o1, dy);
        const float scale = 1.f / sqrtf((float)p.spp);
        dx = d + mul(dx - d, scale);
        dx = divs(dx, len(dx));
        dy = d + mul(dy - d, scale);
        dy = divs(dy, len(dy));
        oy = ox;
        return true;
    }
    if (!(info & kDiffRays)) return false;
    const float4 a = ps.diff[3 * (size_t)slot], b = ps.diff[3 * (size_t)slot + 1], c = ps.diff[3 * (size_t)slot + 2];
    ox = v3(a.x, a.y, a.z);
    dx = v3(a.w, b.x, b.y);
    oy = v3(b.z, b.w, c.x);
    dy = v3(c.y, c.z, c.w);
    return true;
}

// Where a hit looks its textures up: the shading context's uv, world-space
// dpdu/dpdv and uv derivatives (zero without uvs).
struct Tex_Site {
    float2 uv, duvdx, duvdy;
    V3 dpdu, dpdv;
    bool has_uv;
};

// The texture site of a hit (init_from_triangle_mesh_intersection and
// calculate_dxdy_derivatives): the uv derivatives come from the hit's
// incoming differential rays, if it has any.
__device__ __noinline__ void texture_site(const Render_Params& p, const Scene_Dev& S, const Path_State& ps,
                                          uint32_t slot, int bounce, uint32_t info, const Shading& sc, float4 h4,
                                          uint2 h2, Tex_Site& t) {
    float2 uv = make_float2(0.f, 0.f), duvdx = make_float2(0.f, 0.f), duvdy = make_float2(0.f, 0.f);
    V3 dpdu = v3(0.f, 0.f, 0.f), dpdv = v3(0.f, 0.f, 0.f);
    t.has_uv = texture_geometry(S, h2.y, h2.x, h4.y, h4.z, h4.w, uv, dpdu, dpdv);
    V3 ox, dx, oy, dy;
    if (t.has_uv && incoming_differentials(p, ps, slot, bounce, info, ox, dx, oy, dy)) {
        V3 dpdx, dpdy;
        dxdy_derivatives(sc, ox, dx, oy, dy, dpdu, dpdv, dpdx, dpdy, duvdx, duvdy);
    }
    t.uv = uv;
    t.duvdx = duvdx;
    t.duvdy = duvdy;
    t.dpdu = dpdu;
    t.dpdv = dpdv;
}

// evaluate_texture_parameter (parameter_evaluation.cpp:10-31): the uv and its
// derivatives scaled, then EWA with repeat wrapping.
__device__ __forceinline__ Col texture_lookup(const Scene_Dev& S, const Tex_Site& t, uint32_t texture, float2 scale,
                                              float u, float v) {
    return texture_ewa(S, __ldg(S.textures + texture - 1), u * scale.x, v * scale.y,
                       make_float2(t.duvdx.x * scale.x, t.duvdx.y * scale.y),
                       make_float2(t.duvdy.x * scale.x, t.duvdy.y * scale.y));
}

// The bump map's height at (u, v): the constant, or the luminance of the
// texture (evaluate_leaf_parameter_float, parameter_evaluation.cpp:46-55;
// ColorRGB::luminance, src/lib/color.h:74-76).
__device__ __forceinline__ float bump_height_at(const Scene_Dev& S, const Tex_Site& t, const Material_Dev& m, float u,
                                                float v) {
    if (m.bump == 1) return m.bump_height;
    const Col c = texture_lookup(S, t, m.bump_texture, m.bump_scale, u, v);
    return 0.2126729f * c.r + 0.7151522f * c.g + 0.0721750f * c.b;
}

// The normal's uv derivatives of a hit (init_from_triangle_mesh_intersection,
// src/ref/shading_context.cpp:225-238; to world space, scaled with the
// normal and flipped with it, :102-109, :128-133); zero without uvs.
__device__ __noinline__ void normal_derivatives(const Scene_Dev& S, uint32_t object, uint32_t prim, float b0,
                                                float b1, float b2, bool has_uv, bool flipped, V3& dndu_out,
                                                V3& dndv_out) {
    const float4* orec = S.ds.objects + 6 * (size_t)object;
    const uint32_t tri_offset = __float_as_uint(__ldg(orec + 4).w);
    const size_t g = (size_t)tri_offset + prim;
    const float4 h0 = __ldg(S.shading + 4 * g), h1 = __ldg(S.shading + 4 * g + 1);
    const float4 h2 = __ldg(S.shading + 4 * g + 2), h3 = __ldg(S.shading + 4 * g + 3);
    const uint32_t flags = __float_as_uint(h3.w);
    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1), q2 = __ldg(S.ds.tris + 3 * g + 2);
    const V3 p0 = v3(q0.x, q0.y, q0.z), p1 = v3(q1.x, q1.y, q1.z), p2 = v3(q2.x, q2.y, q2.z);
    // the object-space normal as init_shading interpolates it, for its length after the transform
    V3 normal = normalized(cross(p1 - p0, p2 - p0));
    if (flags & 4u) normal = -normal;
    const V3 vn0 = (flags & 1u) ? v3(h0.x, h0.y, h0.z) : v3(0.f, 0.f, 0.f);
    const V3 vn1 = (flags & 1u) ? v3(h1.x, h1.y, h1.z) : v3(0.f, 0.f, 0.f);
    const V3 vn2 = (flags & 1u) ? v3(h2.x, h2.y, h2.z) : v3(0.f, 0.f, 0.f);
    if (flags & 1u) {
        const V3 in = bary(vn0, vn1, vn2, b0, b1, b2);
        if (len2(in) != 0.f) normal = normalized(in);
    }
    V3 dndu = v3(0.f, 0.f, 0.f), dndv = v3(0.f, 0.f, 0.f);
    if (has_uv) {
        // uvs: u0 = h0.w, v0 = h1.w, u1 = h2.w, v1 = h3.x, u2 = h3.y, v2 = h3.z
        const float a00 = h2.w - h0.w, a01 = h3.x - h1.w, a10 = h3.y - h0.w, a11 = h3.z - h1.w;
        const V3 bn0 = vn1 - vn0, bn1 = vn2 - vn0;
        const float det = a00 * a11 - a01 * a10;  // solve_linear_system_2x2, src/lib/math.cpp:8-16
        if (det != 0.f) {
            const float inv_det = 1.f / det;
            dndu = mul(mul(bn0, a11) - mul(bn1, a01), inv_det);
            dndv = mul(mul(bn0, -a10) + mul(bn1, a00), inv_det);
        }
        if (fabsf(det) < 1e-9f) {  // pbrt's approximation
            const V3 dn = cross(bn1, bn0);
            if (len2(dn) == 0.f) {
                dndu = v3(0.f, 0.f, 0.f);
                dndv = v3(0.f, 0.f, 0.f);
            } else {
                dndu = coordinate_axis(dn);
                dndv = cross(dn, dndu);
            }
        }
    }
    const float4* rrec = S.obj_render + 7 * (size_t)object;
    const float4 n0 = __ldg(rrec + 3), n1 = __ldg(rrec + 4), n2 = __ldg(rrec + 5);
    const float inv_length = 1 / len(xform_vector(n0, n1, n2, normal));
    dndu = mul(xform_vector(n0, n1, n2, dndu), inv_length);
    dndv = mul(xform_vector(n0, n1, n2, dndv), inv_length);
    if (flipped) {
        dndu = -dndu;
        dndv = -dndv;
    }
    dndu_out = dndu;
    dndv_out = dndv;
}

// Shading_Context::apply_bump_map (src/ref/shading_context.cpp:419-462) with the
// geometry it reads: the normal's uv derivatives and the shading frame's second
// tangent (:150-167).  Heights at the uv and one footprint step along u and v
// perturb the tangents; the normal is rebuilt from them, turned into the
// geometric normal's hemisphere and adjusted.
__device__ __noinline__ void apply_bump(const Scene_Dev& S, const Material_Dev& m, const Tex_Site& t,
                                        uint32_t object, uint32_t prim, float b0, float b1, float b2, Shading& sc) {
    V3 dndu, dndv;
    normal_derivatives(S, object, prim, b0, b1, b2, t.has_uv, sc.flipped, dndu, dndv);
    // the shading frame's second tangent before the bump
    V3 dpdv_shading;
    if (!t.has_uv) {
        dpdv_shading = cross(sc.n, sc.dpdu_shading);
    } else if (fabsf(dot(sc.n, sc.ng) - 1.f) < 1e-6f) {
        dpdv_shading = t.dpdv;
    } else {
        const V3 tv = cross(t.dpdv, sc.n);
        dpdv_shading = mul(normalized(cross(sc.n, tv)), len(t.dpdv));
    }
    const float height = bump_height_at(S, t, m, t.uv.x, t.uv.y);
    float du = 0.5f * (fabsf(t.duvdx.x) + fabsf(t.duvdy.x));
    if (du == 0.f) du = 0.0005f;
    const float height_du = bump_height_at(S, t, m, t.uv.x + du, t.uv.y + 0.f);
    float dv = 0.5f * (fabsf(t.duvdx.y) + fabsf(t.duvdy.y));
    if (dv == 0.f) dv = 0.0005f;
    const float height_dv = bump_height_at(S, t, m, t.uv.x + 0.f, t.uv.y + dv);
    const V3 original_shading_normal = sc.flipped ? -sc.n : sc.n;
    const float du_scale = m.bump == 2 ? m.bump_scale.x : 1.f;
    const float dv_scale = m.bump == 2 ? m.bump_scale.y : 1.f;
    const V3 dpdu_b = (sc.dpdu_shading + mul(original_shading_normal, (height_du - height) / (du * du_scale))) +
                      mul(mul(dndu, du_scale), height);
    const V3 dpdv_b = (dpdv_shading + mul(original_shading_normal, (height_dv - height) / (dv * dv_scale))) +
                      mul(mul(dndv, dv_scale), height);
    V3 n = normalized(cross(dpdu_b, dpdv_b));
    if (dot(n, sc.ng) < 0) n = -n;
    sc.n = adjust_shading_normal(sc.wo, sc.ng, n);
    sc.dpdu_shading = dpdu_b;
}

// The textured reflectance and transmittance of a BSDF (the constructors'
// evaluate_rgb_parameter calls, src/ref/bsdf.cpp:89-103, :205-213, :268-276,
// :427-438): diffuse transmission scales and clamps them.
__device__ __noinline__ void textured_bsdf_params(const Scene_Dev& S, const Tex_Site& t, const Material_Dev& m,
                                                  Bsdf& f) {
    auto clamp_unit = [](Col c) {
        auto c1 = [](float v) { return v < 0.f ? 0.f : (1.f < v ? 1.f : v); };
        return col(c1(c.r), c1(c.g), c1(c.b));
    };
    if (m.texture) {
        const Col r = texture_lookup(S, t, m.texture, m.texture_scale, t.uv.x, t.uv.y);
        f.reflectance = m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION ? clamp_unit(m.extra * r) : r;
    }
    if (m.texture2) {
        const Col r = texture_lookup(S, t, m.texture2, m.texture2_scale, t.uv.x, t.uv.y);
        f.transmittance = m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION ? clamp_unit(m.extra * r) : r;
    }
}

// get_glass_info's textured Kr and Kt (src/ref/delta_scattering.cpp:53-97): the
// attenuation of a smooth-glass delta event of the given kind (0 reflection,
// else etaI_over_etaT of the transmission).
__device__ __noinline__ Col textured_glass_attenuation(const Scene_Dev& S, const Tex_Site& t, const Material_Dev& m,
                                                       float kind, Col atten) {
    if (kind == 0.f) return m.texture ? texture_lookup(S, t, m.texture, m.texture_scale, t.uv.x, t.uv.y) : atten;
    if (!m.texture2) return atten;
    return mul(texture_lookup(S, t, m.texture2, m.texture2_scale, t.uv.x, t.uv.y), kind * kind);
}

// Shading_Context::compute_differential_rays_for_specular_reflection (kind 0)
// and _for_specular_transmission (kind = etaI_over_etaT), src/ref/shading_context.cpp:357-403:
// the differential rays of a delta ray in direction dir from a vertex that
// has dxdy derivatives (check_for_delta_scattering_event,
// src/ref/delta_scattering.cpp:283-322), written to Path_State::diff for the
// ray's arrival.  False when the vertex has none: no incoming differential
// rays, no uvs, or derivatives dropped as implausible.
__device__ __noinline__ bool specular_differentials(const Render_Params& p, const Scene_Dev& S, const Path_State& ps,
                                                    uint32_t slot, int bounce, uint32_t info, const Shading& sc,
                                                    float4 h4, uint2 h2, V3 dir, float kind) {
    float2 uv;
    V3 dpdu, dpdv;
    if (!texture_geometry(S, h2.y, h2.x, h4.y, h4.z, h4.w, uv, dpdu, dpdv)) return false;
    V3 ox, dx, oy, dy;
    if (!incoming_differentials(p, ps, slot, bounce, info, ox, dx, oy, dy)) return false;
    V3 dpdx, dpdy;
    float2 duvdx, duvdy;
    if (!dxdy_derivatives(sc, ox, dx, oy, dy, dpdu, dpdv, dpdx, dpdy, duvdx, duvdy)) return false;
    V3 dndu, dndv;
    normal_derivatives(S, h2.y, h2.x, h4.y, h4.z, h4.w, true, sc.flipped, dndu, dndv);
    const V3 n = sc.n, wo = sc.wo;
    const V3 dwo_dx = -dx - wo, dwo_dy = -dy - wo;
    const V3 dndx = mul(dndu, duvdx.x) + mul(dndv, duvdx.y);
    const V3 dndy = mul(dndu, duvdy.x) + mul(dndv, duvdy.y);
    const float d_wo_dot_n_dx = dot(dwo_dx, n) + dot(wo, dndx);
    const float d_wo_dot_n_dy = dot(dwo_dy, n) + dot(wo, dndy);
    V3 dwi_dx, dwi_dy;
    if (kind == 0.f) {
        const float dot_wo_n = dot(wo, n);
        dwi_dx = mul(mul(n, d_wo_dot_n_dx) + mul(dndx, dot_wo_n), 2.f) - dwo_dx;
        dwi_dy = mul(mul(n, d_wo_dot_n_dy) + mul(dndy, dot_wo_n), 2.f) - dwo_dy;
    } else {
        const float cos_o = dot(wo, n);
        const float cos_t = -dot(dir, n);
        const float k1 = kind * kind * cos_o / cos_t;
        const float k2 = kind * cos_o - cos_t;
        const float d_cos_t_dx = k1 * d_wo_dot_n_dx, d_cos_t_dy = k1 * d_wo_dot_n_dy;
        dwi_dx = (mul(dwo_dx, -kind) + mul(dndx, k2)) + mul(n, kind * d_wo_dot_n_dx - d_cos_t_dx);
        dwi_dy = (mul(dwo_dy, -kind) + mul(dndy, k2)) + mul(n, kind * d_wo_dot_n_dy - d_cos_t_dy);
    }
    const V3 o_x = sc.position + dpdx, d_x = normalized(dir + dwi_dx);
    const V3 o_y = sc.position + dpdy, d_y = normalized(dir + dwi_dy);
    ps.diff[3 * (size_t)slot] = make_float4(o_x.x, o_x.y, o_x.z, d_x.x);
    ps.diff[3 * (size_t)slot + 1] = make_float4(d_x.y, d_x.z, o_y.x, o_y.y);
    ps.diff[3 * (size_t)slot + 2] = make_float4(o_y.z, d_y.x, d_y.y, d_y.z);
    return true;
}

// ---------------------------------------------------------------- sphere lights
// Diffuse_Sphere_Light_Sampler (light_sampling.cpp:76-123): the cone the
// sphere subtends from the shading point, sampled uniformly in solid angle.
struct Sphere_Sampler {
    V3 center, axes[3];
    float radius, d_center, cos_theta_max, cone_pdf;
};
__device__ __forceinline__ void sphere_sampler_init(Sphere_Sampler& ss, V3 center, float radius, V3 shading_pos) {
    ss.center = center;
    ss.radius = radius;
    V3 a2 = shading_pos - center;
    ss.d_center = len(a2);
    a2 = divs(a2, ss.d_center);
    ss.axes[0] = coordinate_axis(a2);  // coordinate_system_from_vector, src/lib/math.cpp:21-25
    ss.axes[1] = cross(a2, ss.axes[0]);
    ss.axes[2] = a2;
    const float sin_theta_max = radius / ss.d_center;
    ss.cos_theta_max = sqrtf(max_std(0.f, 1.f - sin_theta_max * sin_theta_max));
    ss.cone_pdf = 1.f / (2.f * kPi * (1.f - ss.cos_theta_max));
}
__device__ __forceinline__ V3 sphere_sampler_sample(const Sphere_Sampler& ss, float u0, float u1) {
    const float radius2 = ss.radius * ss.radius;
    const float d_center2 = ss.d_center * ss.d_center;
    const float cos_theta = (1.f - u0) + u0 * ss.cos_theta_max;
    const float phi = 2.f * kPi * u1;
    const float sin_theta2 = max_std(0.f, 1.f - cos_theta * cos_theta);
    const float d_sample = ss.d_center * cos_theta - sqrtf(max_std(0.f, radius2 - d_center2 * sin_theta2));
    const float cos_alpha = (d_center2 + radius2 - d_sample * d_sample) / (2.f * ss.d_center * ss.radius);
    const float sin_alpha = sqrtf(max_std(0.f, 1.f - cos_alpha * cos_alpha));
    const V3 dir = (mul(ss.axes[0], sin_alpha * cos_f(phi)) + mul(ss.axes[1], sin_alpha * sin_f(phi))) +
                   mul(ss.axes[2], cos_alpha);
    return mul(dir, ss.radius) + ss.center;
}

// ---------------------------------------------------------------- shade
// GUIDED adds the learned proposal to the continuation: with probability
// g.alpha the direction comes from the vertex's lobe mixture instead of the
// BSDF, and the throughput divides by the one-sample mixture pdf
// alpha q + (1 - alpha) p_bsdf, so the estimator stays unbiased; the light
// sample and the MIS probe are unchanged.  With g.records set, every
// continued vertex also leaves a training record.
// FULL: delta materials, the layered, translucent and mixed BSDFs, and every
// light kind but the quad light.  A scene without them runs the FULL = false
// instantiation, which has none of that code (launch_shade picks it from
// Render_Params::full_shading).
// Launch bounds: the plain instantiation (diffuse, metal, rough glass, quad
// lights: the C1, C3 and batch renders) at 4 blocks of 128 threads per SM
// (128 registers) spills nothing: the shadow, probe and next extend rays wait
// for the warp's appends in shared memory, and the path's radiance is read and
// written only where emission adds to it; its guided form spills 18 B.  The
// FULL instantiations keep 3 blocks (160-162 registers, no spills; at 4 the
// out-of-line BSDF routines, the fourier series among them, push the kernel
// to 36-60 B of spills).  The guided plain-material form at 3 blocks (152
// registers, no spills) rendered the guided room no faster than at 4 (38 B
// of spills).  Before those changes the plain kernel ran at 5
// blocks (96 registers, 202 B of spill stores), which measured 1.726 s on the
// C3 render against 1.732 s at 4 blocks and 1.764 s at 3.
template <bool GUIDED, bool FULL>
__global__ void __launch_bounds__(kBlock, FULL ? 3 : 4)
shade_kernel(Render_Params p, Scene_Dev S, int cur, uint32_t count, const float* __restrict__ s1d,
             const float2* __restrict__ s2d, Path_State ps, Queues q, Guide_Shade g) {
    // this thread's shadow, probe and next extend rays (origin + tmax,
    // direction) from where they are made until the warp's appends: in shared
    // memory, not in 24 registers live across the whole shading
    __shared__ float4 stash[6][kBlock];
    if (q.ext_count) count = *q.ext_count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t i = (q.order && k < count) ? q.order[k] : k;  // queue entry this thread shades
        bool want_shadow = false, want_probe = false, want_next = false;
        uint32_t slot = 0;
        if (k < count) {
            slot = q.ext_slot[cur][i];
            const float4 rb = q.ext_rays[cur][2 * (size_t)i + 1];
            const float4 h4 = q.ext_hit4[i];
            const uint2 h2 = q.ext_hit2[i];
            float4 coeff4 = ps.coeff[slot];
            uint32_t info = ps.info[slot];
            int bounce = (int)(info & 0xffu);
            const bool arrival = FULL && (info & kDeltaArrival) != 0;
            Col coeff = col(coeff4.x, coeff4.y, coeff4.z);
            const bool hit = h2.y != 0xffffffffu;
            Shading sc;
            int4 oinfo = make_int4(-1, -1, -1, -1);
            if (hit) init_shading(S, v3(rb.x, rb.y, rb.z), h2.y, h2.x, h4.y, h4.z, h4.w, sc, oinfo);
            const bool is_light = hit && (uint32_t)oinfo.z != 0xffffffffu;
            bool done = false;
            // Emission seen by a camera ray or by a delta ray (the delta vertex
            // already applied its attenuation and counted the bounce).
            // The path's radiance changes only here in this kernel (direct light
            // is added by the connect kernel): read and written back only then.
            if (bounce == 0 || arrival) {
                // get_emitted_radiance (direct_lighting.cpp:386-413): triangle-mesh
                // lights emit only on the side their normal faces
                bool emits = false;
                Col le = col(0.f, 0.f, 0.f);
                if (is_light && (uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_RECTANGULAR) {
                    const float4 e4 = __ldg(&S.lights[oinfo.w].le);
                    le = col(e4.x, e4.y, e4.z);
                    emits = true;
                } else if (FULL && is_light && (uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH && !sc.flipped) {
                    const float4 e4 = __ldg(&S.mesh_lights[oinfo.w].le);
                    le = col(e4.x, e4.y, e4.z);
                    emits = true;
                } else if (FULL && is_light && (uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_SPHERE) {
                    const float4 e4 = __ldg(&S.sphere_lights[oinfo.w].le);
                    le = col(e4.x, e4.y, e4.z);
                    emits = true;
                } else if (FULL && !hit && S.env_map) {  // a miss sees the environment, filtered
                    le = env_radiance(S, v3(rb.x, rb.y, rb.z), true);
                    emits = true;
                }
                if (emits) {
                    const float4 L4 = ps.L[slot];
                    const Col L = col(L4.x, L4.y, L4.z) + coeff * le;
                    ps.L[slot] = make_float4(L.r, L.g, L.b, 0.f);
                }
                if (arrival ? (info & kDeltaFinal) != 0 : p.max_bounces == 0) done = true;
            }
            if (!hit || is_light) done = true;
            Dims dm;
            dm.rng_used = false;
            dm.draws = 0u;
            if (!done) {
                {
                    const uint32_t lp = slot / (uint32_t)p.spp, k = slot - lp * (uint32_t)p.spp;
                    dm.s1d = s1d + (size_t)lp * p.n1d * p.spp + k;
                    dm.s2d = s2d + (size_t)lp * p.n2d * p.spp + k;
                    dm.spp = p.spp;
                }
                dm.n1d = p.n1d;
                dm.n2d = p.n2d;
                dm.i1d = (int)((info >> 8) & 0xffu);
                dm.i2d = (int)((info >> 16) & 0xffu);
                const uint4 rs = ps.rng[slot];
                dm.rng.state = (uint64_t)rs.x | ((uint64_t)rs.y << 32);
                dm.rng.inc = (uint64_t)rs.z | ((uint64_t)rs.w << 32);
                // The Russian roulette that ends the reference's delta iteration
                // (path_tracing.cpp:114-131) takes its draw before this vertex's.
                if (arrival && bounce >= p.rr_bounce_threshold) {
                    const float u_term = next1d(dm);
                    const float max_coeff = max_std(coeff.r, max_std(coeff.g, coeff.b));
                    if (max_coeff < p.rr_threshold) {
                        const float p_term = max_std(0.05f, 1.f - max_coeff);
                        if (u_term < p_term)
                            done = true;
                        else
                            coeff = mul(coeff, 1.f / (1.f - p_term));
                    }
                }
            }
            if (!done) {
                const float u_scatter = next1d(dm);
                const float u_light_index = next1d(dm);
                const float u_scatter_next = next1d(dm);
                const float2 ul = next2d(dm);
                const float2 ub = next2d(dm);
                const float2 un = next2d(dm);

                const Material_Dev& mat = S.materials[oinfo.y];
                // Image textures and bump maps read the hit's texture site; the bump
                // map changes the shading frame before the delta check and the BSDF
                // (check_for_delta_scattering_event applies it first,
                // src/ref/delta_scattering.cpp:252-257; create_bsdf again, which
                // gives the same frame).
                Tex_Site site;
                const bool textured = FULL && (mat.texture | mat.texture2 | mat.bump) != 0u;
                if (textured) {
                    texture_site(p, S, ps, slot, bounce, info, sc, h4, h2, site);
                    if (mat.bump) apply_bump(S, mat, site, h2.y, h2.x, h4.y, h4.z, h4.w, sc);
                }
                // Shading_Context::initialize_scattering (shading_context.cpp:174-186): a
                // delta event may be chosen (for the pbrt3 uber material per sample,
                // which remaps u_scatter); the BSDF exists unless every layer is delta.
                float u_sc = u_scatter;
                float bsdf_prob = 1.f;  // 1 - delta_layer_selection_probability
                V3 delta_wi = v3(0.f, 0.f, 0.f);
                Col delta_atten = col(1.f, 1.f, 1.f);
                float delta_kind = 0.f;
                int delta = 0;
                if (FULL && mat.delta != kDeltaNone) {
                    delta = delta_scattering(sc, mat, S.materials, u_sc, delta_wi, delta_atten, bsdf_prob, delta_kind);
                    if (textured && delta == 1 && mat.delta == kDeltaGlass && (mat.texture | mat.texture2) != 0u)
                        delta_atten = textured_glass_attenuation(S, site, mat, delta_kind, delta_atten);
                }
                Bsdf f;
                uint32_t pend = 0;
                if (delta == 0 || bsdf_prob != 0.f) {
                    make_bsdf(sc, mat, S.materials, f);
                    if (textured && (mat.texture | mat.texture2) != 0u) textured_bsdf_params(S, site, mat, f);
                    // estimate_direct_lighting_from_single_sample (direct_lighting.cpp:522-578):
                    // the light int(u * total_light_count), point, spot and directional lights
                    // first, then the rectangular lights (the reference asserts the index is
                    // below the total; the clamp only guards memory)
                    const int selected = min((int)(u_light_index * (float)p.total_lights), p.total_lights - 1);
                    pend = kPendDirect;
                    if (FULL && selected < p.delta_lights) {
                        // direct_lighting_from_point/spot/directional_light (direct_lighting.cpp:26-107):
                        // one shadow ray, no MIS
                        const Delta_Light_Dev& D = S.delta_lights[selected];
                        const float4 da = __ldg(&D.a), db = __ldg(&D.b), dc = __ldg(&D.c);
                        const uint32_t kind = __float_as_uint(da.w);
                        const V3 ldir = v3(db.x, db.y, db.z);
                        V3 wi, position;
                        float tmax = __int_as_float(0x7f800000), scale = 0.f;
                        bool lit = false;
                        if (kind == YAR_LIGHT_DIRECTIONAL) {
                            wi = ldir;
                            const float n_dot_l = dot(sc.n, wi);
                            position = origin_for_direction(sc, wi);
                            lit = n_dot_l > 0.f;
                            scale = n_dot_l;
                        } else {
                            const V3 lp = v3(da.x, da.y, da.z);
                            position = origin_for_point(sc, lp);
                            const V3 lv = lp - position;
                            const float dist = len(lv);
                            wi = divs(lv, dist);
                            tmax = dist * (1.f - 1e-5f);
                            if (kind == YAR_LIGHT_POINT) {
                                const float n_dot_l = dot(sc.n, wi);
                                lit = n_dot_l > 0.f;
                                scale = n_dot_l / (dist * dist);
                            } else {
                                const float cone_cos = db.w, penumbra_cos = dc.w;
                                const float wi_cos = dot(-wi, ldir);
                                if (!(wi_cos < cone_cos)) {
                                    float attenuation = 1.f;
                                    if (wi_cos < penumbra_cos) {
                                        const float k = (wi_cos - cone_cos) / (penumbra_cos - cone_cos);
                                        attenuation = (k * k) * (k * k);
                                    }
                                    const float ndw = dot(sc.n, wi);
                                    lit = (ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission);
                                    scale = attenuation * fabsf(ndw) / (dist * dist);
                                }
                            }
                        }
                        if (lit) {
                            const Col fv = bsdf_evaluate<FULL>(f, sc.wo, wi);
                            if (kind != YAR_LIGHT_SPOT || !black(fv)) {  // only the spot light skips a black BSDF
                                const Col c = mul(col(dc.x, dc.y, dc.z) * fv, scale);
                                ps.pend_light[slot] = make_float4(c.r, c.g, c.b, 0.f);
                                want_shadow = true;
                                stash[0][threadIdx.x] = make_float4(position.x, position.y, position.z, tmax);
                                stash[1][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                pend |= kPendShadow;
                            }
                        }
                    } else if (FULL && selected >= p.delta_lights + p.rect_lights &&
                               selected < p.delta_lights + p.rect_lights + p.sphere_lights) {
                        // direct_lighting_from_sphere_light (direct_lighting.cpp:196-260)
                        const int light_index = selected - p.delta_lights - p.rect_lights;
                        const Sphere_Light_Dev& SL = S.sphere_lights[light_index];
                        const float4 sa = __ldg(&SL.a), sle = __ldg(&SL.le);
                        const Col Le = col(sle.x, sle.y, sle.z);
                        Sphere_Sampler ss;
                        sphere_sampler_init(ss, v3(sa.x, sa.y, sa.z), sa.w, sc.position);
                        {   // light-sampling half of MIS
                            const V3 lp = sphere_sampler_sample(ss, ul.x, ul.y);
                            const V3 position = origin_for_point(sc, lp);
                            const V3 lv = lp - position;
                            const float dist = len(lv);
                            const V3 wi = divs(lv, dist);
                            const float ndw = dot(sc.n, wi);
                            if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
                                const Col fv = bsdf_evaluate<FULL>(f, sc.wo, wi);
                                if (!black(fv)) {
                                    const float bpdf = bsdf_pdf<FULL>(f, sc.wo, wi);
                                    const float w = mis_power(ss.cone_pdf, bpdf);
                                    const Col c = mul(Le * fv, w * fabsf(ndw) / ss.cone_pdf);
                                    ps.pend_light[slot] = make_float4(c.r, c.g, c.b, 0.f);
                                    want_shadow = true;
                                    stash[0][threadIdx.x] = make_float4(position.x, position.y, position.z, dist * (1.f - 1e-5f));
                                    stash[1][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                    pend |= kPendShadow;
                                }
                            }
                        }
                        {   // BSDF-sampling half of MIS: inside the light's cone, the probe must hit it
                            V3 wi = v3(0.f, 0.f, 0.f);
                            float bpdf = 0.f;
                            const Col fv = bsdf_sample<FULL>(f, ub.x, ub.y, u_sc, sc.wo, wi, bpdf);
                            if (!black(fv) && dot(-ss.axes[2], wi) >= ss.cos_theta_max) {
                                const V3 position = origin_for_direction(sc, wi);
                                const Col lef = Le * fv;
                                ps.pend_probe0[slot] = make_float4(lef.r, lef.g, lef.b, bpdf);
                                ps.pend_probe1[slot] = make_float4(wi.x, wi.y, wi.z, ss.cone_pdf);
                                ps.pend_probe2[slot] = make_float4(dot(sc.n, wi), __int_as_float(light_index),
                                                                   __uint_as_float(kProbeSphereLight), 0.f);
                                want_probe = true;
                                stash[2][threadIdx.x] = make_float4(position.x, position.y, position.z, __int_as_float(0x7f800000));
                                stash[3][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                pend |= kPendProbe;
                            }
                        }
                    } else if (FULL && selected >= p.total_lights - p.env_lights) {
                        // direct_lighting_from_environment_light (direct_lighting.cpp:324-384): the
                        // light sample is a shadow ray to infinity, the BSDF sample's probe must miss
                        {
                            V3 wi;
                            float light_pdf;
                            const Col Le = env_light_sample(S, ul.x, ul.y, wi, light_pdf);
                            const float ndw = dot(sc.n, wi);
                            if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
                                const Col fv = bsdf_evaluate<FULL>(f, sc.wo, wi);
                                if (!black(fv)) {
                                    const V3 position = origin_for_direction(sc, wi);
                                    const float bpdf = bsdf_pdf<FULL>(f, sc.wo, wi);
                                    const float w = mis_power(light_pdf, bpdf);
                                    const Col c = mul(Le * fv, w * fabsf(ndw) / light_pdf);
                                    ps.pend_light[slot] = make_float4(c.r, c.g, c.b, 0.f);
                                    want_shadow = true;
                                    stash[0][threadIdx.x] = make_float4(position.x, position.y, position.z, __int_as_float(0x7f800000));
                                    stash[1][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                    pend |= kPendShadow;
                                }
                            }
                        }
                        {
                            V3 wi = v3(0.f, 0.f, 0.f);
                            float bpdf = 0.f;
                            const Col fv = bsdf_sample<FULL>(f, ub.x, ub.y, u_sc, sc.wo, wi, bpdf);
                            if (!black(fv)) {
                                const Col Le = env_radiance(S, wi, false);
                                if (!black(Le)) {
                                    const V3 position = origin_for_direction(sc, wi);
                                    const Col lef = Le * fv;
                                    ps.pend_probe0[slot] = make_float4(lef.r, lef.g, lef.b, bpdf);
                                    ps.pend_probe1[slot] = make_float4(wi.x, wi.y, wi.z, env_light_pdf(S, wi));
                                    ps.pend_probe2[slot] = make_float4(dot(sc.n, wi), 0.f,
                                                                       __uint_as_float(kProbeEnvLight), 0.f);
                                    want_probe = true;
                                    stash[2][threadIdx.x] = make_float4(position.x, position.y, position.z, __int_as_float(0x7f800000));
                                    stash[3][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                    pend |= kPendProbe;
                                }
                            }
                        }
                    } else if (FULL && selected >= p.delta_lights + p.rect_lights + p.sphere_lights) {
                        // direct_lighting_from_triangle_mesh_light (direct_lighting.cpp:262-322)
                        const int light_index = selected - p.delta_lights - p.rect_lights - p.sphere_lights;
                        const Mesh_Light_Dev& M = S.mesh_lights[light_index];
                        const float4 mle = __ldg(&M.le);
                        const uint4 minfo = __ldg(&M.info);
                        const Col Le = col(mle.x, mle.y, mle.z);
                        {   // light-sampling half of MIS
                            float light_pdf;
                            const V3 lp = mesh_light_sample(S, minfo, mle.w, ul.x, ul.y, sc.position, light_pdf);
                            if (light_pdf != 0.f) {
                                const V3 position = origin_for_point(sc, lp);
                                const V3 lv = lp - position;
                                const float dist = len(lv);
                                const V3 wi = divs(lv, dist);
                                const float ndw = dot(sc.n, wi);
                                if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
                                    const Col fv = bsdf_evaluate<FULL>(f, sc.wo, wi);
                                    if (!black(fv)) {
                                        const float bpdf = bsdf_pdf<FULL>(f, sc.wo, wi);
                                        const float w = mis_power(light_pdf, bpdf);
                                        const Col c = mul(Le * fv, w * fabsf(ndw) / light_pdf);
                                        ps.pend_light[slot] = make_float4(c.r, c.g, c.b, 0.f);
                                        want_shadow = true;
                                        stash[0][threadIdx.x] = make_float4(position.x, position.y, position.z, dist * (1.f - 1e-5f));
                                        stash[1][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                        pend |= kPendShadow;
                                    }
                                }
                            }
                        }
                        {   // BSDF-sampling half of MIS: the probe ray must hit this light
                            V3 wi = v3(0.f, 0.f, 0.f);
                            float bpdf = 0.f;
                            const Col fv = bsdf_sample<FULL>(f, ub.x, ub.y, u_sc, sc.wo, wi, bpdf);
                            if (!black(fv)) {
                                const V3 position = origin_for_direction(sc, wi);
                                const Col lef = Le * fv;
                                ps.pend_probe0[slot] = make_float4(lef.r, lef.g, lef.b, bpdf);
                                ps.pend_probe1[slot] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                ps.pend_probe2[slot] = make_float4(dot(sc.n, wi), __int_as_float(light_index),
                                                                   __uint_as_float(kProbeMeshLight), 0.f);
                                want_probe = true;
                                stash[2][threadIdx.x] = make_float4(position.x, position.y, position.z, __int_as_float(0x7f800000));
                                stash[3][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                pend |= kPendProbe;
                            }
                        }
                    } else {
                        const int light_index = selected - p.delta_lights;
                        const Rect_Light_Dev& Ld = S.lights[light_index];
                        const float4 lr0 = __ldg(&Ld.r0), lr1 = __ldg(&Ld.r1), lr2 = __ldg(&Ld.r2);
                        const float4 lle = __ldg(&Ld.le), lsz = __ldg(&Ld.sz);
                        const V3 light_n = v3(lr0.z, lr1.z, lr2.z);
                        const Col Le = col(lle.x, lle.y, lle.z);
                        const float size_x = lle.w, size_y = lsz.x;
                        {   // light-sampling half of MIS
                            const V3 local = v3(size_x * (ul.x - 0.5f), size_y * (ul.y - 0.5f), 0.0f);
                            const V3 lp = xform_point(lr0, lr1, lr2, local);
                            const V3 position = origin_for_point(sc, lp);
                            const V3 lv = lp - position;
                            const float dist = len(lv);
                            const V3 wi = divs(lv, dist);
                            const float lndw = dot(light_n, -wi);
                            if (lndw > 1e-4f) {
                                const float ndw = dot(sc.n, wi);
                                const bool possible = (ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission);
                                if (possible) {
                                    const Col fv = bsdf_evaluate<FULL>(f, sc.wo, wi);
                                    if (!black(fv)) {
                                        const float light_pdf = (dist * dist) / (size_x * size_y * lndw);
                                        const float bpdf = bsdf_pdf<FULL>(f, sc.wo, wi);
                                        const float w = mis_power(light_pdf, bpdf);
                                        const Col c = mul(Le * fv, w * fabsf(ndw) / light_pdf);
                                        ps.pend_light[slot] = make_float4(c.r, c.g, c.b, 0.f);
                                        want_shadow = true;
                                        stash[0][threadIdx.x] = make_float4(position.x, position.y, position.z, dist * (1.f - 1e-5f));
                                        stash[1][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                        pend |= kPendShadow;
                                    }
                                }
                            }
                        }
                        {   // BSDF-sampling half of MIS: the probe ray must hit this light
                            V3 wi = v3(0.f, 0.f, 0.f);
                            float bpdf = 0.f;
                            const Col fv = bsdf_sample<FULL>(f, ub.x, ub.y, u_sc, sc.wo, wi, bpdf);
                            if (!black(fv)) {
                                const float lndw = dot(light_n, -wi);
                                const V3 position = origin_for_direction(sc, wi);
                                if (lndw > 1e-4f && probe_may_reach(Ld, position, wi, lndw)) {
                                    const Col lef = Le * fv;
                                    ps.pend_probe0[slot] = make_float4(lef.r, lef.g, lef.b, bpdf);
                                    ps.pend_probe1[slot] = make_float4(position.x, position.y, position.z, lndw);
                                    ps.pend_probe2[slot] = make_float4(dot(sc.n, wi), __int_as_float(light_index), 0.f, 0.f);
                                    want_probe = true;
                                    stash[2][threadIdx.x] = make_float4(position.x, position.y, position.z, __int_as_float(0x7f800000));
                                    stash[3][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                                    pend |= kPendProbe;
                                }
                            }
                        }
                    }
                    ps.pend_coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0.f);
                }
                if (delta != 0) {
                    // The delta branch of trace_path (path_tracing.cpp:76-112): the delta
                    // ray is the next extend ray, whose hit adds the light it reaches.
                    // A perfect refractor at total internal reflection ends the path.
                    // Reflected and transmitted delta rays carry differential rays for
                    // the first max_differential_ray_specular_bounces bounces.
                    uint32_t diff_flag = 0u;
                    if (FULL && p.spec_diffs && delta == 1 && delta_kind >= 0.f &&
                        bounce < kMaxDifferentialRaySpecularBounces &&
                        specular_differentials(p, S, ps, slot, bounce, info, sc, h4, h2, delta_wi, delta_kind))
                        diff_flag = kDiffRays;
                    bounce++;
                    if (delta == 1) {
                        coeff = coeff * delta_atten;
                        const V3 o = origin_for_direction(sc, delta_wi);
                        stash[4][threadIdx.x] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
                        stash[5][threadIdx.x] = make_float4(delta_wi.x, delta_wi.y, delta_wi.z, 0.f);
                        want_next = true;
                    }
                    if (GUIDED && g.records) ps.rec[slot] = 0xffffffffu;
                    info = (uint32_t)bounce | ((uint32_t)dm.i1d << 8) | ((uint32_t)dm.i2d << 16) | kDeltaArrival |
                           (bounce == p.max_bounces ? kDeltaFinal : 0u) | pend | diff_flag;
                } else {
                    bounce++;
                    bool cont = bounce != p.max_bounces;
                    float rec_value = 0.f;
                    V3 rec_dir = v3(0.f, 0.f, 0.f);
                    if (cont) {
                        V3 wi = v3(0.f, 0.f, 0.f);
                        float pdf = 0.f;
                        Col fv;
                        if (GUIDED && g.lobes) {
                            const float* lob = g.lobes + (size_t)i * kGuideLobeFloats;
                            const float u_sel = pcg_float(dm.rng);
                            dm.rng_used = true;
                            float pdf_b = 0.f;
                            if (u_sel < g.alpha) {
                                // the continuation's own stratified sample dimensions (the ones
                                // the BSDF branch takes): guided directions stay stratified
                                // over a pixel's samples
                                wi = mixture_sample(lob, u_scatter_next, un.x, un.y);
                                const float ndw = dot(sc.n, wi);
                                const bool possible = (ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission);
                                fv = possible ? bsdf_evaluate<FULL>(f, sc.wo, wi) : col(0.f, 0.f, 0.f);
                                pdf_b = possible ? bsdf_pdf<FULL>(f, sc.wo, wi) : 0.f;
                            } else {
                                fv = bsdf_sample<FULL>(f, un.x, un.y, u_scatter_next, sc.wo, wi, pdf_b);
                            }
                            pdf = g.alpha * mixture_pdf(lob, wi) + (1.f - g.alpha) * pdf_b;
                            if (!(pdf > 0.f)) fv = col(0.f, 0.f, 0.f);
                        } else {
                            fv = bsdf_sample<FULL>(f, un.x, un.y, u_scatter_next, sc.wo, wi, pdf);
                        }
                        if (black(fv)) {
                            cont = false;
                        } else {
                            if (GUIDED) {
                                rec_value = (0.2126729f * fv.r + 0.7151522f * fv.g + 0.0721750f * fv.b) *
                                            fabsf(dot(sc.n, wi)) / pdf;
                                rec_dir = wi;
                            }
                            coeff = coeff * mul(fv, fabsf(dot(sc.n, wi)) / (pdf * bsdf_prob));
                            const V3 o = origin_for_direction(sc, wi);
                            stash[4][threadIdx.x] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
                            stash[5][threadIdx.x] = make_float4(wi.x, wi.y, wi.z, 0.f);
                            if (bounce >= p.rr_bounce_threshold) {  // Russian roulette
                                const float u_term = next1d(dm);
                                const float max_coeff = max_std(coeff.r, max_std(coeff.g, coeff.b));
                                if (max_coeff < p.rr_threshold) {
                                    const float p_term = max_std(0.05f, 1.f - max_coeff);
                                    if (u_term < p_term) {
                                        cont = false;
                                    } else {
                                        coeff = mul(coeff, 1.f / (1.f - p_term));
                                    }
                                }
                            }
                        }
                    }
                    want_next = cont;
                    if (GUIDED && g.records) {
                        uint32_t r = 0xffffffffu;
                        if (cont) {
                            r = atomicAdd(g.record_count, 1u);
                            if (r < g.record_capacity) {
                                float4* rec = g.records + (size_t)r * kGuideRecordF4;
                                const float4* qr = g.queries + 3 * (size_t)i;
                                rec[0] = qr[0];
                                rec[1] = qr[1];
                                rec[2] = make_float4(qr[2].x, rec_dir.x, rec_dir.y, rec_dir.z);
                                rec[3] = make_float4(rec_value, __uint_as_float(slot), 0.f, 0.f);
                                rec[4] = make_float4(coeff.r, coeff.g, coeff.b, 0.f);
                            } else {
                                r = 0xffffffffu;
                            }
                        }
                        ps.rec[slot] = r;
                    }
                    info = (uint32_t)bounce | ((uint32_t)dm.i1d << 8) | ((uint32_t)dm.i2d << 16) | pend;
                }
            }
            // Saved also when the Russian roulette of a delta arrival ended the path.
            if (dm.rng_used) {
                ps.rng[slot] = make_uint4((uint32_t)dm.rng.state, (uint32_t)(dm.rng.state >> 32),
                                          (uint32_t)dm.rng.inc, (uint32_t)(dm.rng.inc >> 32));
                if (p.exact_tail) ps.rng_draws[slot] += dm.draws;
            }
            if (p.exact_tail == 1 && want_next && tail_may_draw_past_budget(p, info)) {
                ps.deferred[2 * (size_t)slot] = stash[4][threadIdx.x];
                ps.deferred[2 * (size_t)slot + 1] = stash[5][threadIdx.x];
                info |= kDeferred;
                want_next = false;
            }
            ps.coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0.f);
            ps.info[slot] = info;
        }
        const uint32_t is = warp_append(&q.counters[1], want_shadow);
        if (want_shadow) {
            q.shd_rays[2 * (size_t)is] = stash[0][threadIdx.x];
            q.shd_rays[2 * (size_t)is + 1] = stash[1][threadIdx.x];
            q.shd_slot[is] = slot;
        }
        const uint32_t ip = warp_append(&q.counters[2], want_probe);
        if (want_probe) {
            q.prb_rays[2 * (size_t)ip] = stash[2][threadIdx.x];
            q.prb_rays[2 * (size_t)ip + 1] = stash[3][threadIdx.x];
            q.prb_slot[ip] = slot;
        }
        const uint32_t in = warp_append(&q.counters[0], want_next);
        if (want_next) {
            q.ext_rays[cur ^ 1][2 * (size_t)in] = stash[4][threadIdx.x];
            q.ext_rays[cur ^ 1][2 * (size_t)in + 1] = stash[5][threadIdx.x];
            q.ext_slot[cur ^ 1][in] = slot;
        }
    }
}

template <bool GUIDED>
void launch_shade(const Render_Params& p, unsigned grid, cudaStream_t st, const Scene_Dev& S, int cur, uint32_t count,
                  const float* s1d, const float2* s2d, const Path_State& ps, const Queues& q, const Guide_Shade& g) {
    if (p.full_shading)
        shade_kernel<GUIDED, true><<<grid, kBlock, 0, st>>>(p, S, cur, count, s1d, s2d, ps, q, g);
    else
        shade_kernel<GUIDED, false><<<grid, kBlock, 0, st>>>(p, S, cur, count, s1d, s2d, ps, q, g);
}

// ---------------------------------------------------------------- connect
__global__ void __launch_bounds__(kBlock)
connect_kernel(Render_Params p, Scene_Dev S, const uint32_t* __restrict__ slots, uint32_t count, Path_State ps,
               float4* __restrict__ records, const uint32_t* __restrict__ count_dev = nullptr) {
    if (count_dev) count = *count_dev;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = slots[i];
        const uint32_t info = ps.info[slot];
        if (!(info & kPendDirect)) continue;
        Col direct = col(0.f, 0.f, 0.f);
        if ((info & kPendShadow) && !ps.occluded[slot]) {
            const float4 c = ps.pend_light[slot];
            direct = direct + col(c.x, c.y, c.z);
        }
        if (info & kPendProbe) {
            const uint2 h2 = ps.probe_hit2[slot];
            const float4 p2 = ps.pend_probe2[slot];
            const int light_index = __float_as_int(p2.y);
            const uint32_t kind = __float_as_uint(p2.z);
            if (kind == kProbeEnvLight && h2.y == 0xffffffffu) {
                const float4 p0 = ps.pend_probe0[slot], p1 = ps.pend_probe1[slot];
                const float w = mis_power(p0.w, p1.w);
                direct = direct + mul(col(p0.x, p0.y, p0.z), w * fabsf(p2.x) / p0.w);
            }
            if (kind != kProbeEnvLight && h2.y != 0xffffffffu) {
                const float4 inf4 = __ldg(S.obj_render + 7 * (size_t)h2.y + 6);
                const uint32_t hit_light = (uint32_t)__float_as_int(inf4.z);
                if (kind == kProbeSphereLight && hit_light == YAR_LIGHT_DIFFUSE_SPHERE &&
                    __float_as_int(inf4.w) == light_index) {
                    const float4 p0 = ps.pend_probe0[slot], p1 = ps.pend_probe1[slot];
                    const float w = mis_power(p0.w, p1.w);
                    direct = direct + mul(col(p0.x, p0.y, p0.z), w * fabsf(p2.x) / p0.w);
                } else if (kind == kProbeMeshLight && hit_light == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH &&
                    __float_as_int(inf4.w) == light_index) {
                    // Diffuse_Triangle_Mesh_Light_Sampler::pdf (light_sampling.cpp:163-184)
                    const float4 h4 = ps.probe_hit4[slot];
                    const Mesh_Light_Dev& M = S.mesh_lights[light_index];
                    const size_t g = (size_t)__ldg(&M.info).x + h2.x;
                    const float4 p0 = ps.pend_probe0[slot], p1 = ps.pend_probe1[slot];
                    const V3 light_n = mesh_light_normal(S, g, h4.y, h4.z, h4.w);
                    const float lndw = dot(light_n, -v3(p1.x, p1.y, p1.z));
                    const float light_pdf = lndw <= 0.f ? 0.f : (h4.x * h4.x) / (lndw * __ldg(&M.le).w);
                    const float w = mis_power(p0.w, light_pdf);
                    direct = direct + mul(col(p0.x, p0.y, p0.z), w * fabsf(p2.x) / p0.w);
                } else if (kind == kProbeRectLight && hit_light == YAR_LIGHT_DIFFUSE_RECTANGULAR &&
                           __float_as_int(inf4.w) == light_index) {
                    const float4 h4 = ps.probe_hit4[slot];
                    const uint32_t tri_offset = __float_as_uint(__ldg(S.ds.objects + 6 * (size_t)h2.y + 4).w);
                    const size_t g = (size_t)tri_offset + h2.x;
                    const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1),
                                 q2 = __ldg(S.ds.tris + 3 * g + 2);
                    // Triangle_Mesh::get_position: object-space barycentric interpolation
                    const V3 hp = bary(v3(q0.x, q0.y, q0.z), v3(q1.x, q1.y, q1.z), v3(q2.x, q2.y, q2.z), h4.y, h4.z, h4.w);
                    const float4 p0 = ps.pend_probe0[slot], p1 = ps.pend_probe1[slot];
                    const float d = len(hp - v3(p1.x, p1.y, p1.z));
                    const Rect_Light_Dev& Ld = S.lights[light_index];
                    const float size_x = __ldg(&Ld.le).w, size_y = __ldg(&Ld.sz).x;
                    const float light_pdf = (d * d) / (size_x * size_y * p1.w);
                    const float w = mis_power(p0.w, light_pdf);
                    const Col c = mul(col(p0.x, p0.y, p0.z), w * fabsf(p2.x) / p0.w);
                    direct = direct + c;
                }
            }
        }
        const float4 cv = ps.pend_coeff[slot];
        const Col scaled = mul(direct, (float)p.total_lights);
        const float4 L4 = ps.L[slot];
        const Col L = col(L4.x, L4.y, L4.z) + col(cv.x, cv.y, cv.z) * scaled;
        ps.L[slot] = make_float4(L.r, L.g, L.b, 0.f);
        ps.info[slot] = info & ~(kPendShadow | kPendProbe | kPendDirect);
        if (records) {
            const uint32_t r = ps.rec[slot];
            if (r != 0xffffffffu) records[(size_t)r * kGuideRecordF4 + 5] = make_float4(L.r, L.g, L.b, 0.f);
        }
    }
}

// ---------------------------------------------------------------- shading order
// The shade kernel visits the extend queue grouped by what the hit needs:
// misses and emitters, diffuse, metal, then every other material, so that a
// warp mostly runs one BSDF's code (the kernel's stalls are mostly
// instruction fetch, and mixed warps run every material's branch).  Each
// path's result does not depend on the order; the appends to the next
// queues, already in atomic order, only change places.
constexpr uint32_t kShadeClasses = 4;

__device__ __forceinline__ uint32_t shade_class(const Scene_Dev& S, uint2 h2) {
    if (h2.y == 0xffffffffu) return 0u;  // a miss
    const float4 inf4 = __ldg(S.obj_render + 7 * (size_t)h2.y + 6);
    if ((uint32_t)__float_as_int(inf4.z) != 0xffffffffu) return 0u;  // an emitter: emission only
    const uint32_t m = (uint32_t)__float_as_int(inf4.x);
    return m == YAR_MATERIAL_DIFFUSE ? 1u : (m == YAR_MATERIAL_METAL ? 2u : 3u);
}

// Lane's rank among the warp's lanes with the same key, and that group's
// leader lane (the lowest); every lane of the warp takes part.
__device__ __forceinline__ void key_group(uint32_t key, uint32_t& rank, int& leader, uint32_t& size) {
    const uint32_t group = __match_any_sync(0xffffffffu, key);
    const uint32_t lane = threadIdx.x & 31u;
    rank = __popc(group & ((1u << lane) - 1u));
    leader = __ffs(group) - 1;
    size = __popc(group);
}

// bins[0..3]: the queue's entries per class (bins zeroed by the caller).
__global__ void __launch_bounds__(kBlock)
shade_bin_kernel(Scene_Dev S, Queues q, uint32_t count, uint8_t* __restrict__ keys, uint32_t* __restrict__ bins) {
    if (q.ext_count) count = *q.ext_count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t key = i < count ? shade_class(S, q.ext_hit2[i]) : kShadeClasses;
        if (i < count) keys[i] = (uint8_t)key;
        uint32_t rank, size;
        int leader;
        key_group(key, rank, leader, size);
        if (i < count && rank == 0) atomicAdd(&bins[key], size);
    }
}

// order[]: the queue's entries class after class (bins[4..7] hand out the
// places within a class).
__global__ void __launch_bounds__(kBlock)
shade_order_kernel(Queues q, uint32_t count, const uint8_t* __restrict__ keys, uint32_t* __restrict__ bins,
                   uint32_t* __restrict__ order) {
    if (q.ext_count) count = *q.ext_count;
    uint32_t first[kShadeClasses];
    uint32_t acc = 0;
    for (uint32_t c = 0; c < kShadeClasses; c++) {
        first[c] = acc;
        acc += bins[c];
    }
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t key = i < count ? keys[i] : kShadeClasses;
        uint32_t rank, size;
        int leader;
        key_group(key, rank, leader, size);
        uint32_t at = 0;
        if (i < count && rank == 0) at = atomicAdd(&bins[kShadeClasses + key], size);
        at = __shfl_sync(0xffffffffu, at, leader);
        if (i < count) order[first[key] + at + rank] = i;
    }
}

// ---------------------------------------------------------------- extend-queue order
// The rays of a bounce can be traced grouped by direction octant and origin
// cell (an 8 x 8 x 8 grid over the scene box in Morton order): neighbours in
// the queue then walk much of the same kd-tree.  A counting sort: per-ray
// keys and a histogram, an exclusive scan, then a scatter of each ray and its
// path slot into the other extend buffer.  Results do not depend on the
// order (every per-ray quantity travels with the ray).
constexpr uint32_t kRayBins = 8u * 512u;

struct Ray_Grid {
    float lo[3], scale[3];  // cell = (origin - lo) * scale, 8 cells per axis
};

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__device__ __forceinline__ uint32_t ray_bin(const Ray_Grid& g, float4 a, float4 b) {
    const float o[3] = {a.x, a.y, a.z};
    uint32_t c[3];
    for (int k = 0; k < 3; k++) {
        const float f = (o[k] - g.lo[k]) * g.scale[k];
        c[k] = f >= 1.f ? (f < 7.f ? (uint32_t)f : 7u) : 0u;  // NaN and below the box: cell 0
    }
    const uint32_t oct = (b.x < 0.f ? 1u : 0u) | (b.y < 0.f ? 2u : 0u) | (b.z < 0.f ? 4u : 0u);
    return (oct << 9) | spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
}

__global__ void __launch_bounds__(256)
ray_hist_kernel(Ray_Grid g, const float4* __restrict__ rays, const uint32_t* __restrict__ count_dev, uint32_t count,
                uint16_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kRayBins];
    for (uint32_t j = threadIdx.x; j < kRayBins; j += blockDim.x) sh[j] = 0u;
    __syncthreads();
    if (count_dev) count = *count_dev;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t key = ray_bin(g, rays[2 * (size_t)i], rays[2 * (size_t)i + 1]);
        keys[i] = (uint16_t)key;
        atomicAdd(&sh[key], 1u);
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < kRayBins; j += blockDim.x)
        if (sh[j]) atomicAdd(&hist[j], sh[j]);
}

// hist[] becomes each bin's first place (exclusive prefix), one block of 1024 threads.
__global__ void __launch_bounds__(1024) ray_scan_kernel(uint32_t* __restrict__ hist) {
    constexpr uint32_t kPer = kRayBins / 1024u;
    __shared__ uint32_t part[1024];
    uint32_t v[kPer], sum = 0;
    for (uint32_t k = 0; k < kPer; k++) {
        v[k] = hist[threadIdx.x * kPer + k];
        sum += v[k];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024u; off <<= 1) {  // inclusive scan of the thread sums
        const uint32_t add = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += add;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t k = 0; k < kPer; k++) {
        hist[threadIdx.x * kPer + k] = run;
        run += v[k];
    }
}

__global__ void __launch_bounds__(kBlock)
ray_scatter_kernel(const float4* __restrict__ src_rays, const uint32_t* __restrict__ src_slot,
                   float4* __restrict__ dst_rays, uint32_t* __restrict__ dst_slot,
                   const uint16_t* __restrict__ keys, uint32_t* __restrict__ cursor,
                   const uint32_t* __restrict__ count_dev, uint32_t count) {
    if (count_dev) count = *count_dev;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < count;
        const uint32_t key = valid ? keys[i] : 0xffffffffu;
        uint32_t rank, size;
        int leader;
        key_group(key, rank, leader, size);
        uint32_t at = 0;
        if (valid && rank == 0) at = atomicAdd(&cursor[key], size);
        at = __shfl_sync(0xffffffffu, at, leader);
        if (valid) {
            const uint32_t pos = at + rank;
            dst_rays[2 * (size_t)pos] = src_rays[2 * (size_t)i];
            dst_rays[2 * (size_t)pos + 1] = src_rays[2 * (size_t)i + 1];
            dst_slot[pos] = src_slot[i];
        }
    }
}

// Device-driven bounces.  Queue counters: [0] next extend, [1] shadow, [2]
// probe, [3] error, [4..6] ray hand-out, [7] this bounce's extend count; rays:
// [0] closest, [1] any.  Turns the last bounce's appends into this bounce's
// extend count (first_paths for a chunk's first bounce) and adds the last
// bounce's rays.
__global__ void bounce_begin_kernel(uint32_t* counters, uint32_t first_paths, unsigned long long* rays) {
    const uint32_t prev_ext = counters[7], prev_shadow = counters[1], prev_probe = counters[2];
    rays[0] += prev_ext + prev_probe;
    rays[1] += prev_shadow;
    counters[7] = first_paths ? first_paths : counters[0];
    counters[0] = counters[1] = counters[2] = 0;
}

__global__ void __launch_bounds__(kBlock)
finish_chunk_kernel(uint32_t paths, uint64_t first_sample, const Path_State ps, float4* __restrict__ radiance) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < paths; i += gridDim.x * blockDim.x)
        radiance[first_sample + i] = ps.L[i];
}

// ---------------------------------------------------------------- exact tail
// The reference draws the dimensions past the sampler budget from the pixel's
// pcg stream, after the sample tables, in sample order: sample k starts where
// sample k-1 stopped (Stratified_Pixel_Sampler::get_next_1d/2d_sample,
// src/ref/pixel_sampling.cpp:159-173).  A path that may take such a draw at its next
// vertex is deferred (kDeferred, its extend ray kept per slot), and the
// deferred paths are finished in waves: wave j takes each pixel's j-th
// deferred sample, whose stream is the pixel's advanced by the table draws
// plus the draws of the pixel's earlier deferred samples.

// Per chunk pixel: the deferred samples' slots in sample order (list, spp
// entries per pixel), their count, and the stream position of the first.
// tail[0] = the largest count, tail[1] != 0 if a path drew past the budget
// before it was deferred.
__global__ void __launch_bounds__(kBlock)
tail_rank_kernel(Render_Params p, uint32_t chunk_pixels, Path_State ps, uint32_t* __restrict__ list,
                 uint32_t* __restrict__ deferred_count, uint32_t* __restrict__ stream_pos, uint32_t* __restrict__ tail) {
    const uint32_t spp = (uint32_t)p.spp;
    const uint32_t table_draws = 2u * spp + (uint32_t)p.n1d * (2u * spp - 1u) + (uint32_t)p.n2d * (3u * spp - 1u);
    for (uint32_t lp = blockIdx.x * blockDim.x + threadIdx.x; lp < chunk_pixels; lp += gridDim.x * blockDim.x) {
        uint32_t n = 0, stray = 0;
        for (uint32_t k = 0; k < spp; k++) {
            const uint32_t slot = lp * spp + k;
            if (ps.info[slot] & kDeferred) list[slot - k + n++] = slot;
            stray |= ps.rng_draws[slot];
        }
        deferred_count[lp] = n;
        stream_pos[lp] = table_draws;
        if (n) atomicMax(&tail[0], n);
        if (stray) atomicOr(&tail[1], 1u);
    }
}

// Wave `wave`: advances each pixel's stream position past its previous
// wave's draws and queues its next deferred sample as extend queue 0
// (count in counters[0]) with the pcg state at that position.
__global__ void __launch_bounds__(kBlock)
tail_wave_kernel(Render_Params p, uint32_t chunk_first, uint32_t chunk_pixels, uint32_t wave, Path_State ps, Queues q,
                 const uint32_t* __restrict__ list, const uint32_t* __restrict__ deferred_count,
                 uint32_t* __restrict__ stream_pos) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < chunk_pixels; base += gridDim.x * blockDim.x) {
        const uint32_t lp = base + threadIdx.x;
        bool take = false;
        uint32_t slot = 0;
        if (lp < chunk_pixels) {
            const uint32_t n = deferred_count[lp];
            const size_t row = (size_t)lp * (uint32_t)p.spp;
            uint32_t pos = stream_pos[lp];
            if (wave > 0 && wave <= n) {
                pos += ps.rng_draws[list[row + wave - 1]];
                stream_pos[lp] = pos;
            }
            if (wave < n) {
                take = true;
                slot = list[row + wave];
                int x, y;
                Pcg r = pixel_pcg(p, pixel_stream(p, chunk_first + lp, x, y));
                pcg_advance(r, pos);
                ps.rng[slot] = make_uint4((uint32_t)r.state, (uint32_t)(r.state >> 32), (uint32_t)r.inc,
                                          (uint32_t)(r.inc >> 32));
                ps.rng_draws[slot] = 0u;
            }
        }
        const uint32_t at = warp_append(&q.counters[0], take);
        if (take) {
            q.ext_rays[0][2 * (size_t)at] = ps.deferred[2 * (size_t)slot];
            q.ext_rays[0][2 * (size_t)at + 1] = ps.deferred[2 * (size_t)slot + 1];
            q.ext_slot[0][at] = slot;
        }
    }
}

// ---------------------------------------------------------------- film
// Per sample-region pixel: clamp/scale of each sample (reference_renderer.cpp:388-393)
// and the luminance variance of the pixel (:397-409).
__global__ void __launch_bounds__(kBlock)
samples_kernel(Render_Params p, float4* __restrict__ radiance, double* __restrict__ pixel_variance) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (uint32_t)(p.sw * p.sh)) return;
    double lsum = 0.0, lsq = 0.0;
    for (int k = 0; k < p.spp; k++) {
        float4 r = radiance[(size_t)pix * p.spp + k];
        const float mc = max_std(r.x, max_std(r.y, r.z));
        if (mc > p.max_component) {
            const float s = p.max_component / mc;
            r.x *= s; r.y *= s; r.z *= s;
        }
        if (p.film_scale != 1.f) {
            r.x *= p.film_scale; r.y *= p.film_scale; r.z *= p.film_scale;
        }
        radiance[(size_t)pix * p.spp + k] = r;
        const float lum = 0.2126729f * r.x + 0.7151522f * r.y + 0.0721750f * r.z;
        lsum += lum;
        lsq += lum * lum;
    }
    double v = 0.0;
    if (p.spp > 1) {
        const int n = p.spp;
        v = (lsq - lsum * lsum / n) / (n * (n - 1));
        v = v > 0.0 ? v : 0.0;
    }
    pixel_variance[pix] = v;
}

__device__ __forceinline__ void tile_sample_bounds(const Render_Params& p, int t, int& x0, int& y0, int& x1, int& y1) {
    const int tx = t % p.tiles_x, ty = t / p.tiles_x;
    x0 = p.sx0 + tx * kTile;
    y0 = p.sy0 + ty * kTile;
    x1 = min(x0 + kTile, p.sx0 + p.sw);
    y1 = min(y0 + kTile, p.sy0 + p.sh);
}

__device__ __forceinline__ void tile_pixel_bounds(const Render_Params& p, int t, int& x0, int& y0, int& x1, int& y1) {
    int sx0, sy0, sx1, sy1;
    tile_sample_bounds(p, t, sx0, sy0, sx1, sy1);
    const float r = p.filter_radius;
    x0 = max((int)ceilf((float)sx0 - r - 0.5f), p.rx0);
    y0 = max((int)ceilf((float)sy0 - r - 0.5f), p.ry0);
    x1 = min((int)floorf((float)sx1 + r - 0.5f) + 1, p.rx0 + p.rw);
    y1 = min((int)floorf((float)sy1 + r - 0.5f) + 1, p.ry0 + p.rh);
}

// Tile variance accumulators in the reference's pixel order (render_tile loops).
// One block per tile: the block stages the tile's pixel variances in shared
// memory with coalesced loads, then one thread adds them in the reference's
// sequential (y, x) order (double addition is not associative).
constexpr int kTileVarThreads = 256;
__global__ void __launch_bounds__(kTileVarThreads)
tile_variance_kernel(Render_Params p, const double* __restrict__ pixel_variance, double* __restrict__ tile_variance) {
    __shared__ double v[kTile * kTile];
    const int t = blockIdx.x;
    int x0, y0, x1, y1;
    tile_sample_bounds(p, t, x0, y0, x1, y1);
    const int w = x1 - x0, h = y1 - y0;
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        const int y = i / w, x = i - y * w;
        v[i] = pixel_variance[(size_t)(y0 + y - p.sy0) * p.sw + (x0 + x - p.sx0)];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int i = 0; i < w * h; i++) acc += v[i];
        tile_variance[t] = acc;
    }
}

// Mean pixel variance over the sample region (render_scene's
// variance_estimate, reference_renderer.cpp:565-581), from the per-tile
// sums, in tile order.
__global__ void variance_total_kernel(Render_Params p, const double* __restrict__ tile_variance,
                                      double* __restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double acc = 0.0;
    int64_t count = 0;
    for (int t = 0; t < p.tiles_x * p.tiles_y; t++) {
        acc += tile_variance[t];
        int x0, y0, x1, y1;
        tile_sample_bounds(p, t, x0, y0, x1, y1);
        count += (int64_t)(x1 - x0) * (y1 - y0);
    }
    *out = p.spp > 1 ? acc / (double)count : 0.0;
}

// Sample tables and camera rays of a chunk.  The table kernel's block is
// sized so that its spp float2 per thread fit in 96 KB of shared memory.
constexpr size_t kTablesSmemLimit = 96 * 1024;

// One-time kernel attribute (also called before a stream capture, so that
// no attribute change happens inside one).
cudaError_t generate_prepare() {
    // the table kernel's dynamic shared-memory limit, once per device
    static bool attr_set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        e = cudaFuncSetAttribute(sample_tables_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTablesSmemLimit);
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    return cudaSuccess;
}

cudaError_t launch_generate(const Render_Params& p, uint32_t first, uint32_t cp, float* s1d, float* s2d,
                            float2* image_samples, const Path_State& ps, const Queues& q, cudaStream_t st) {
    constexpr size_t kSmemLimit = kTablesSmemLimit;
    cudaError_t pe = generate_prepare();
    if (pe != cudaSuccess) return pe;
    // One thread per table row, its spp values shuffled in shared memory: above
    // 96 samples per pixel fewer threads fit a block.  (One warp per row, the
    // lanes drawing the values and lane 0 replaying the shuffle, measured
    // slower at 256-1024 samples per pixel: the shuffle's serial chain then
    // runs on one lane per warp instead of in lockstep across the threads.)
    const size_t per_thread = (size_t)p.spp * sizeof(float2);
    int threads = 128;
    while (threads > 1 && (size_t)threads * per_thread > kSmemLimit) threads /= 2;
    if ((size_t)threads * per_thread > kSmemLimit) return cudaErrorInvalidValue;
    const uint64_t rows = (uint64_t)cp * (1u + (uint32_t)p.n1d + (uint32_t)p.n2d);
    sample_tables_kernel<<<(uint32_t)((rows + threads - 1) / threads), threads, threads * per_thread, st>>>(
        p, first, cp, s1d, s2d, image_samples);
    const uint32_t paths = cp * (uint32_t)p.spp;
    camera_kernel<<<(paths + kBlock - 1) / kBlock, kBlock, 0, st>>>(p, first, paths, image_samples, ps, q);
    return cudaGetLastError();
}

// The film filter's weight at offset (x, y) = film position - pixel center
// (src/ref/film.cpp:123-142): box 1; gaussian max(0, exp(-alpha |p|^2) - exp(-alpha
// r^2)) with the exponential correctly rounded; triangle max(0, r - |x|) max(0, r - |y|).
__device__ __forceinline__ float film_filter_weight(const Render_Params& p, float x, float y) {
    if (p.filter_type == 1) {
        const float e = (float)exp((double)(-p.filter_alpha * (x * x + y * y)));
        return max_std(0.f, e - p.filter_zero);
    }
    if (p.filter_type == 2) return max_std(0.f, p.filter_radius - fabsf(x)) * max_std(0.f, p.filter_radius - fabsf(y));
    return 1.f;
}

// Film_Tile t's sum for film pixel (px, py): the samples of the tile's sample
// region whose filter footprint covers the pixel, in the tile's own sample
// order (Film_Tile::add_sample, src/ref/film.cpp:27-50), as (color sum, weight).
__device__ __forceinline__ float4 tile_pixel_sum(const Render_Params& p, const float4* __restrict__ radiance,
                                                 const float2* __restrict__ image_samples, int t, int px, int py) {
    const float r = p.filter_radius;
    // a sample in pixel q reaches pixels p with |p - q| <= ceil(r + 1/2)
    // (Film_Tile::add_sample's ceil(x - r - 1/2) .. floor(x + r - 1/2))
    const int R = (int)ceilf(r + 0.5f);
    const int qx0 = max(px - R, p.sx0), qx1 = min(px + R, p.sx0 + p.sw - 1);
    const int qy0 = max(py - R, p.sy0), qy1 = min(py + R, p.sy0 + p.sh - 1);
    int bx0, by0, bx1, by1;
    tile_pixel_bounds(p, t, bx0, by0, bx1, by1);
    int sx0, sy0, sx1, sy1;
    tile_sample_bounds(p, t, sx0, sy0, sx1, sy1);
    float tr = 0.f, tg = 0.f, tb = 0.f, tw = 0.f;
    for (int qy = max(qy0, sy0); qy <= min(qy1, sy1 - 1); qy++)
        for (int qx = max(qx0, sx0); qx <= min(qx1, sx1 - 1); qx++) {
            const size_t pix = (size_t)(qy - p.sy0) * p.sw + (qx - p.sx0);
            for (int k = 0; k < p.spp; k++) {
                const float2 s = image_samples[pix * p.spp + k];
                const float fx = (float)qx + s.x, fy = (float)qy + s.y;
                int rx0 = (int)ceilf(fx - r - 0.5f), ry0 = (int)ceilf(fy - r - 0.5f);
                int rx1 = (int)floorf(fx + r - 0.5f) + 1, ry1 = (int)floorf(fy + r - 0.5f) + 1;
                rx0 = max(rx0, bx0); ry0 = max(ry0, by0);
                rx1 = min(rx1, bx1); ry1 = min(ry1, by1);
                if (px < rx0 || px >= rx1 || py < ry0 || py >= ry1) continue;
                const float4 c = radiance[pix * p.spp + k];
                const float w = film_filter_weight(p, fx - ((float)px + 0.5f), fy - ((float)py + 0.5f));
                tr += w * c.x;
                tg += w * c.y;
                tb += w * c.z;
                tw += w;
            }
        }
    return make_float4(tr, tg, tb, tw);
}

// One film pixel: the tiles whose samples reach it are merged in tile order
// (Film::merge_tile), each tile's sum accumulated in its own sample order
// (Film_Tile::add_sample with the box filter), then resolved (Film::get_image).
__global__ void __launch_bounds__(kBlock)
film_kernel(Render_Params p, const float4* __restrict__ radiance, const float2* __restrict__ image_samples,
            float* __restrict__ rgb) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)(p.rw * p.rh)) return;
    const int px = p.rx0 + (int)(idx % (uint32_t)p.rw);
    const int py = p.ry0 + (int)(idx / (uint32_t)p.rw);
    const float r = p.filter_radius;
    const int R = (int)ceilf(r + 0.5f);  // the samples' reach, as in tile_pixel_sum
    // candidate sample pixels: [px - R, px + R] x [py - R, py + R] inside the sample region
    const int qx0 = max(px - R, p.sx0), qx1 = min(px + R, p.sx0 + p.sw - 1);
    const int qy0 = max(py - R, p.sy0), qy1 = min(py + R, p.sy0 + p.sh - 1);
    const int tx0 = (qx0 - p.sx0) / kTile, tx1 = (qx1 - p.sx0) / kTile;
    const int ty0 = (qy0 - p.sy0) / kTile, ty1 = (qy1 - p.sy0) / kTile;
    float fr = 0.f, fg = 0.f, fb = 0.f, fw = 0.f;
    for (int ty = ty0; ty <= ty1; ty++)
        for (int tx = tx0; tx <= tx1; tx++) {
            const int t = ty * p.tiles_x + tx;
            int bx0, by0, bx1, by1;
            tile_pixel_bounds(p, t, bx0, by0, bx1, by1);
            if (px < bx0 || px >= bx1 || py < by0 || py >= by1) continue;
            const float4 c = tile_pixel_sum(p, radiance, image_samples, t, px, py);
            fr += c.x;
            fg += c.y;
            fb += c.z;
            fw += c.w;
        }
    float cr = 0.f, cg = 0.f, cb = 0.f;
    if (fw != 0.f) {
        const float inv = 1.f / fw;
        cr = fr * inv;
        cg = fg * inv;
        cb = fb * inv;
    }
    rgb[3 * (size_t)idx + 0] = max_std(0.f, cr);
    rgb[3 * (size_t)idx + 1] = max_std(0.f, cg);
    rgb[3 * (size_t)idx + 2] = max_std(0.f, cb);
}

// Every tile's Film_Pixel array (color sum, weight) over its pixel bounds, tile
// t at out + offset[t], row-major: one block row per tile (blockIdx.y).
__global__ void __launch_bounds__(kBlock)
tile_film_kernel(Render_Params p, const float4* __restrict__ radiance, const float2* __restrict__ image_samples,
                 const uint32_t* __restrict__ offset, float4* __restrict__ out) {
    const int t = blockIdx.y;
    int bx0, by0, bx1, by1;
    tile_pixel_bounds(p, t, bx0, by0, bx1, by1);
    const int w = bx1 - bx0, h = by1 - by0;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (w <= 0 || h <= 0 || i >= (uint32_t)(w * h)) return;
    const int px = bx0 + (int)(i % (uint32_t)w), py = by0 + (int)(i / (uint32_t)w);
    out[offset[t] + i] = tile_pixel_sum(p, radiance, image_samples, t, px, py);
}

// ---------------------------------------------------------------- host helpers
// Film::get_tile_bounds' pixel bounds of tile t (x0, y0, x1, y1), on the host.
inline void host_tile_pixel_bounds(const Render_Params& p, int t, int b[4]) {
    const int tx = t % p.tiles_x, ty = t / p.tiles_x;
    const int sx0 = p.sx0 + tx * kTile, sy0 = p.sy0 + ty * kTile;
    const int sx1 = std::min(sx0 + kTile, p.sx0 + p.sw), sy1 = std::min(sy0 + kTile, p.sy0 + p.sh);
    const float r = p.filter_radius;
    b[0] = std::max((int)std::ceil((float)sx0 - r - 0.5f), p.rx0);
    b[1] = std::max((int)std::ceil((float)sy0 - r - 0.5f), p.ry0);
    b[2] = std::min((int)std::floor((float)sx1 + r - 0.5f) + 1, p.rx0 + p.rw);
    b[3] = std::min((int)std::floor((float)sy1 + r - 0.5f) + 1, p.ry0 + p.rh);
}
float pbrt3_roughness_to_alpha(float roughness) {
    // src/ref/scattering.cpp:240-251 (host libm logf, as the reference evaluates it)
    roughness = std::max(roughness, 1e-3f);
    float x = std::log(roughness);
    return 1.621420000f + 0.819955000f * x + 0.173400000f * x * x + 0.017120100f * x * x * x +
           0.000640711f * x * x * x * x;
}

float roughness_to_alpha(const yar_render_config& c, float r, int no_remap) {
    if (no_remap) return r;
    if (c.pbrt3_scene) return pbrt3_roughness_to_alpha(r);
    return r * r;
}

template <class T>
T* dptr(Device_Buffer& b) {
    return reinterpret_cast<T*>(b.ptr);
}

int grid_for(uint64_t n) {
    uint64_t blocks = (n + kBlock - 1) / kBlock;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks, 152ull * 64));
}

// Checks the uploaded scene and configuration against what the path tracer
// implements and derives the launch parameters: Film::Film's sample region
// (src/ref/film.cpp:53-86) and the sampler's dimension budget
// (src/ref/reference_renderer.cpp:87-99).
int prepare_render_params(yar_gpu_ctx* ctx, Render_Params& p) {
    const Render_Scene& R = ctx->render;
    const yar_render_config& c = R.config;
    if (c.rendering_algorithm != 0 && c.rendering_algorithm != 1)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "unknown rendering algorithm");
    if (c.pixel_filter_type < 0 || c.pixel_filter_type > 2) return fail(ctx, YAR_ERR_UNSUPPORTED, "unknown pixel filter");
    if (R.other_light_count)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "the scene has lights of a kind that is not implemented");
    if (R.has_environment && R.has_no_shadow_meshes)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "environment light with meshes that cast no shadows");
    if (R.host_rect_lights.empty() && R.host_delta_lights.empty() && R.mesh_light_count == 0 &&
        R.sphere_light_count == 0 && !R.has_environment)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "scene has no light");
    for (size_t i = 0; i < R.host_delta_lights.size(); i++) {
        const uint32_t t = R.host_delta_lights[i].type;
        if (t > YAR_LIGHT_DIRECTIONAL || (i > 0 && t < R.host_delta_lights[i - 1].type))
            return fail(ctx, YAR_ERR_INVALID, "point, spot and directional lights must be listed in that order");
    }
    for (const yar_material_desc& m : R.host_materials) {
        if (m.other_textured_parameters)
            return fail(ctx, YAR_ERR_UNSUPPORTED,
                        "a material parameter other than a reflectance, a transmittance or a bump map is a texture");
        const bool reflectance_slot = m.type == YAR_MATERIAL_DIFFUSE || m.type == YAR_MATERIAL_PLASTIC ||
                                      m.type == YAR_MATERIAL_COATED_DIFFUSE || m.type == YAR_MATERIAL_GLASS ||
                                      m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION;
        const bool transmittance_slot = m.type == YAR_MATERIAL_GLASS || m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION;
        if ((m.reflectance_texture && !reflectance_slot) || (m.transmittance_texture && !transmittance_slot))
            return fail(ctx, YAR_ERR_UNSUPPORTED, "an image texture in a slot the material does not read");
        if (m.reflectance_texture > R.texture_count || m.transmittance_texture > R.texture_count ||
            (m.bump == 2 && (m.bump_texture == 0 || m.bump_texture > R.texture_count)))
            return fail(ctx, YAR_ERR_INVALID, "a material names a texture the scene does not have");
        if (m.bump > 2) return fail(ctx, YAR_ERR_INVALID, "bump map kind " + std::to_string(m.bump));
        if (m.bump && m.type == YAR_MATERIAL_MIX)
            return fail(ctx, YAR_ERR_UNSUPPORTED, "a mix material has no bump map");
        if (m.type != YAR_MATERIAL_DIFFUSE && m.type != YAR_MATERIAL_METAL && m.type != YAR_MATERIAL_GLASS &&
            m.type != YAR_MATERIAL_PLASTIC && m.type != YAR_MATERIAL_COATED_DIFFUSE &&
            m.type != YAR_MATERIAL_PERFECT_REFLECTOR && m.type != YAR_MATERIAL_PERFECT_REFRACTOR &&
            m.type != YAR_MATERIAL_DIFFUSE_TRANSMISSION && m.type != YAR_MATERIAL_PBRT3_TRANSLUCENT &&
            m.type != YAR_MATERIAL_PBRT3_UBER && m.type != YAR_MATERIAL_MIX && m.type != YAR_MATERIAL_PBRT3_FOURIER)
            return fail(ctx, YAR_ERR_UNSUPPORTED, "material type " + std::to_string(m.type) + " is not implemented");
        if (m.type == YAR_MATERIAL_PBRT3_FOURIER) {
            if (m.fourier_table == 0 || m.fourier_table > R.host_fourier_tables.size())
                return fail(ctx, YAR_ERR_INVALID, "a fourier material without a table");
            if (R.host_fourier_tables[m.fourier_table - 1].eta != 1.f)  // the reference asserts eta == 1
                return fail(ctx, YAR_ERR_UNSUPPORTED, "fourier tables with refraction (eta != 1)");
        }
        if (m.type == YAR_MATERIAL_MIX) {
            // one level: sub-materials that are pure delta or have no delta event, not both delta
            int delta_subs = 0;
            for (int k = 0; k < 2; k++) {
                const int32_t si = m.mix_materials[k];
                if (si < 0 || (size_t)si >= R.host_materials.size())
                    return fail(ctx, YAR_ERR_INVALID, "mix material with an invalid sub-material");
                const yar_material_desc& sm = R.host_materials[si];
                if (sm.type == YAR_MATERIAL_MIX || sm.type == YAR_MATERIAL_PBRT3_UBER ||
                    (sm.type == YAR_MATERIAL_GLASS && !(sm.u_roughness > 0.f)) || sm.type == YAR_MATERIAL_PBRT3_FOURIER)
                    return fail(ctx, YAR_ERR_UNSUPPORTED, "mix of a mix, an uber, a smooth glass or a fourier material");
                if (sm.bump)
                    return fail(ctx, YAR_ERR_UNSUPPORTED, "a mix of a bump-mapped material");
                delta_subs += sm.type == YAR_MATERIAL_PERFECT_REFLECTOR || sm.type == YAR_MATERIAL_PERFECT_REFRACTOR;
            }
            if (delta_subs == 2) return fail(ctx, YAR_ERR_UNSUPPORTED, "mix of two pure delta materials");
        }
        if (m.type == YAR_MATERIAL_PBRT3_UBER) {
            // the reference asserts on an empty component list and has no delta transmission
            bool ok = m.component_count >= 1 && m.component_count <= 5;
            for (uint32_t k = 0; ok && k < m.component_count; k++)
                ok = m.components[k] <= YAR_UBER_OPACITY && m.components[k] != YAR_UBER_DELTA_TRANSMISSION;
            if (!ok) return fail(ctx, YAR_ERR_UNSUPPORTED, "pbrt3 uber: empty component list or delta transmission");
        }
    }
    const size_t n_obj = R.host_object_info.size() / 4;
    for (size_t i = 0; i < n_obj; i++) {
        const int32_t* o = &R.host_object_info[4 * i];
        const bool light = (uint32_t)o[2] != YAR_LIGHT_NULL;
        const bool rect_ok = (uint32_t)o[2] == YAR_LIGHT_DIFFUSE_RECTANGULAR && o[3] >= 0 &&
                             (size_t)o[3] < R.host_rect_lights.size();
        const bool mesh_ok = (uint32_t)o[2] == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH && o[3] >= 0 &&
                             (uint32_t)o[3] < R.mesh_light_count;
        const bool sphere_ok = (uint32_t)o[2] == YAR_LIGHT_DIFFUSE_SPHERE && o[3] >= 0 &&
                               (uint32_t)o[3] < R.sphere_light_count;
        if (light && !rect_ok && !mesh_ok && !sphere_ok)
            return fail(ctx, YAR_ERR_UNSUPPORTED, "object " + std::to_string(i) + ": unsupported area light");
        if (!light && (o[1] < 0 || (size_t)o[1] >= R.host_materials.size()))
            return fail(ctx, YAR_ERR_INVALID, "object " + std::to_string(i) + " has no valid material");
    }
    const int nx = c.x_pixel_sample_count, ny = c.y_pixel_sample_count;
    if (nx <= 0 || ny <= 0 || (int64_t)nx * ny > 4096)
        return fail(ctx, YAR_ERR_INVALID, "pixel sample counts must be in 1..4096 samples per pixel");
    if (c.max_light_bounces < 0 || c.max_light_bounces > 200) return fail(ctx, YAR_ERR_INVALID, "max_light_bounces");

    p = Render_Params{};
    p.camera = R.camera;
    p.rx0 = c.render_region[0];
    p.ry0 = c.render_region[1];
    p.rw = c.render_region[2] - c.render_region[0];
    p.rh = c.render_region[3] - c.render_region[1];
    if (p.rw <= 0 || p.rh <= 0 || c.render_region[2] > 0xffff + 1 || c.render_region[3] > 0xffff + 1)
        return fail(ctx, YAR_ERR_INVALID, "render region");
    const float radius = c.pixel_filter_radius;
    // Film::Film sample region (src/ref/film.cpp:53-86)
    p.sx0 = (int)std::floor((float)p.rx0 + 0.5f - radius);
    p.sy0 = (int)std::floor((float)p.ry0 + 0.5f - radius);
    const int sx1 = (int)std::ceil((float)(p.rx0 + p.rw - 1) + 0.5f + radius);
    const int sy1 = (int)std::ceil((float)(p.ry0 + p.rh - 1) + 0.5f + radius);
    p.sw = sx1 - p.sx0;
    p.sh = sy1 - p.sy0;
    p.tiles_x = (p.sw + kTile - 1) / kTile;
    p.tiles_y = (p.sh + kTile - 1) / kTile;
    p.nx = nx;
    p.ny = ny;
    p.spp = nx * ny;
    const int maxb = std::min(10, c.max_light_bounces);
    p.n1d = maxb * 4;  // src/ref/reference_renderer.cpp:87-99
    p.n2d = maxb * 3;
    p.arrays_2d_first = 0;
    if (c.rendering_algorithm == 0) {
        // direct lighting: no sample vectors, k x k arrays per rectangular and sphere
        // light (reference_renderer.cpp:101-128): 2 two-dimensional, 1 one-dimensional
        int grids_2d = 0, grids_1d = 0;
        auto add = [&](int sample_count) {
            const int k = (int)std::ceil(std::sqrt((double)sample_count));
            grids_2d += 2 * k * k;
            grids_1d += k * k;
        };
        for (const yar_rect_light_desc& l : R.host_rect_lights) add(l.sample_count);
        for (const yar_sphere_light_desc& l : R.host_sphere_lights) add(l.sample_count);
        p.n1d = grids_1d;
        p.n2d = grids_2d;
        p.arrays_2d_first = 1;
    }
    p.max_bounces = c.max_light_bounces;
    p.rr_bounce_threshold = c.russian_roulette_bounce_count_threshold;
    p.rr_threshold = c.russian_roulette_threshold;
    p.filter_radius = radius;
    p.filter_type = c.pixel_filter_type;
    p.filter_alpha = c.pixel_filter_alpha;
    // get_gaussian_filter (src/ref/film.cpp:128-135) evaluates the zero level once, in float
    p.filter_zero = c.pixel_filter_type == 1 ? std::exp(-c.pixel_filter_alpha * radius * radius) : 0.f;
    p.film_scale = c.film_radiance_scale;
    p.max_component = c.max_rgb_component_value_of_film_sample;
    p.rect_lights = (int)R.host_rect_lights.size();
    p.delta_lights = (int)R.host_delta_lights.size();
    p.mesh_lights = (int)R.mesh_light_count;
    p.sphere_lights = (int)R.sphere_light_count;
    p.env_lights = R.has_environment ? 1 : 0;
    p.total_lights = p.delta_lights + p.rect_lights + p.sphere_lights + p.mesh_lights + p.env_lights +
                     (int)R.other_light_count;
    p.full_shading = p.delta_lights > 0 || p.mesh_lights > 0 || p.sphere_lights > 0 || p.env_lights > 0;
    for (const yar_material_desc& m : R.host_materials)
        if (m.type != YAR_MATERIAL_DIFFUSE && m.type != YAR_MATERIAL_METAL &&
            !(m.type == YAR_MATERIAL_GLASS && m.u_roughness > 0.f))
            p.full_shading = 1;
    // Image textures and bump maps: FULL shading.  Image textures read the ray
    // differentials, which the path tracer's delta bounces carry on in scenes
    // with delta materials; a constant bump height reads none.  The
    // direct-lighting algorithm reads them at the camera hit only (its delta
    // ray's hit adds emission).
    bool delta_materials = false, image_textures = false;
    for (const yar_material_desc& m : R.host_materials) {
        if (m.reflectance_texture || m.transmittance_texture || m.bump == 2) image_textures = true;
        if (m.reflectance_texture || m.transmittance_texture || m.bump) p.textured = 1;
        delta_materials = delta_materials || m.type == YAR_MATERIAL_PERFECT_REFLECTOR ||
                          m.type == YAR_MATERIAL_PERFECT_REFRACTOR ||
                          (m.type == YAR_MATERIAL_GLASS && !(m.u_roughness > 0.f)) ||
                          m.type == YAR_MATERIAL_PBRT3_UBER || m.type == YAR_MATERIAL_MIX;
    }
    if (p.textured) p.full_shading = 1;
    // the path tracer's delta rays carry specular differential rays where image textures read them
    p.spec_diffs = image_textures && delta_materials && c.rendering_algorithm != 0 ? 1 : 0;
    p.seed_offset = (uint32_t)c.rng_seed_offset;
    return YAR_OK;
}

} // namespace

} // namespace yar
