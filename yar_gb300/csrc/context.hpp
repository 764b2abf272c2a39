// context.hpp - the state behind a yar_gpu_ctx (include/yar_gpu.h).
#pragma once

#include "device_scene.cuh"
#include "yar_gpu.h"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace yar {

// One device allocation; freed by the owner.
struct Device_Buffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Shading data of a triangle (only uploaded for rendering): normals and uvs
// gathered per triangle, 64 B = 4 x float4:
//   n0.xyz u0 | n1.xyz v0 | n2.xyz u1 | v1 u2 v2 flags
// flags bit0 = mesh has normals, bit1 = mesh has uvs,
//       bit2 = reverse_geometric_normal_orientation
struct Render_Scene {
    Device_Buffer shading;      // float4[4] per triangle
    Device_Buffer materials;    // yar_material_desc[]
    Device_Buffer rect_lights;  // yar_rect_light_desc[]
    Device_Buffer delta_lights; // point, spot and directional lights (Delta_Light_Dev[])
    Device_Buffer mesh_lights;  // triangle-mesh lights (Mesh_Light_Dev[])
    Device_Buffer mesh_cdf;     // their triangle-area CDFs, concatenated
    Device_Buffer sphere_lights; // Sphere_Light_Dev[]
    Device_Buffer env_map;       // environment map texels (float4 rgb), row 0 first
    Device_Buffer env_marginal;  // its Distribution_2D: marginal CDF over rows
    Device_Buffer env_cdfs;      // and the conditional CDFs, one row each
    Device_Buffer texels;        // image textures: every mip's texels (float4 rgb), mip after mip
    Device_Buffer texture_mips;  // uint4 per mip: width, height, texel offset, -
    Device_Buffer textures;      // uint2 per texture: first mip, mip count
    Device_Buffer ewa_weights;   // the EWA filter's 256 weights
    Device_Buffer fourier_floats;  // pbrt3 fourier tables: zenith cosines and coefficients
    Device_Buffer fourier_uints;   // and (offset, length) per node pair
    Device_Buffer object_info;  // int4 per object: material type, material index, light type, light index
    Device_Buffer object_to_world;         // float[12] per object
    Device_Buffer object_to_world_normal;  // float[12] per object
    std::vector<yar_material_desc> host_materials;
    std::vector<yar_fourier_desc> host_fourier_tables;
    std::vector<yar_rect_light_desc> host_rect_lights;
    std::vector<yar_delta_light_desc> host_delta_lights;
    uint32_t mesh_light_count = 0;
    uint32_t sphere_light_count = 0;
    std::vector<yar_sphere_light_desc> host_sphere_lights;
    bool has_environment = false;
    uint32_t texture_count = 0;
    yar_environment_desc environment{};  // radiance is not kept
    bool has_no_shadow_meshes = false;
    std::vector<int32_t> host_object_info;
    yar_camera_desc camera{};
    yar_render_config config{};
    uint32_t other_light_count = 0;
    uint32_t triangle_total = 0;
};

// The learned directional proposal's network (guide_mlp.cu): fp32 master
// parameters with Adam moments, the bf16 operand images the tensor-core
// kernels load, per-CTA partial gradients.
constexpr int kGuideParams = 64 * 128 + 3 * 64 * 64;  // W1 (64x128), W2, W3, W4 (64x64), [out][in]
constexpr int kGuideLobeFloats = 40;                   // 8 lobes x (mean xyz, kappa, weight)
struct Guide {
    Device_Buffer params, adam_m, adam_v, images, partials, scalars;
    int step = 0;
    float beta1 = 0.9f, beta2 = 0.99f, eps = 1e-8f;
};

} // namespace yar

struct yar_gpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;

    // scene
    bool has_scene = false;
    yar::Device_Buffer scene_nodes, mesh_nodes, objects, tris;
    yar::Device_Scene ds;
    yar::Render_Scene render;

    // staging area for host-buffer casts
    uint32_t staging_capacity = 0;
    yar::Device_Buffer d_rays, d_t, d_prim, d_obj, d_bary, d_occ;
    int* d_error = nullptr;  // device error word (stack overflow, bounded-wait expiry)
    uint32_t* d_counter = nullptr;  // ray hand-out counters of the persistent cast kernels, one per pipeline chunk
    // host-buffer casts in chunks: copies in, the traversal on two compute
    // streams (the context's and pipe_compute) and copies out overlap
    static constexpr int kPipeChunks = 32;
    // rays per chunk: on GB300 (C2, 16M rays per call) 4M overlapped best (33.8 ms
    // per closest + any step against 36.8 ms unpipelined; 35.7 at 2M, 46.5 at 1M,
    // where the persistent traversal's tail per launch outweighs the overlap)
    uint32_t pipe_chunk = 4u << 20;
    cudaStream_t pipe_in = nullptr, pipe_compute = nullptr, pipe_out = nullptr;
    // renders: the per-tile variance sums run beside the film resolve
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
    cudaEvent_t pipe_start = nullptr, pipe_in_done[kPipeChunks] = {}, pipe_cast_done[kPipeChunks] = {};
    // traversal kernel per ray kind (0 closest, 1 any) for C-ABI casts and for
    // renders; -1 until tuned on the current scene (or fixed by the options)
    int forced_kernel = -1;
    int cast_kernel[2] = {-1, -1};
    // renders: per ray kind and bounce (bounces past the last share its entry)
    static constexpr int kBounceBuckets = 5;
    int render_kernel[2][kBounceBuckets] = {{-1, -1, -1, -1, -1}, {-1, -1, -1, -1, -1}};
    // while a bucket is being chosen: per kernel the summed times of its timed
    // queues, and how many queues were timed
    float render_tune_ms[2][kBounceBuckets][4] = {};
    int render_tune_queues[2][kBounceBuckets] = {};
    // a render of the current scene has run with host-read queue lengths (and
    // tuned the buckets it filled): later renders drive their bounces on the device
    bool render_tuned = false;

    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;

    // render scratch (path state, queues, per-pixel sample tables); the guided
    // render's training passes and its network inputs and lobes keep their own.
    // Buffers stay allocated between calls and grow when a call needs more.
    std::vector<yar::Device_Buffer> render_scratch;
    std::vector<yar::Device_Buffer> guided_scratch;
    yar::Device_Buffer guide_queries, guide_lobes;

    // learned proposal (allocated on first use)
    yar::Guide guide;
    float guided_weight_scale = 1.f;  // host source of an asynchronous copy during guided renders
};

namespace yar {

int fail(yar_gpu_ctx* ctx, int code, const std::string& message);
int cuda_fail(yar_gpu_ctx* ctx, cudaError_t e, const char* what);
int device_alloc(yar_gpu_ctx* ctx, Device_Buffer& b, size_t bytes);
void device_free(Device_Buffer& b);

// Arguments of the persistent extend/shadow kernels (cast.cu).
struct Cast_Args {
    const float4* rays = nullptr;     // two float4 per ray
    uint32_t n = 0;                   // ray count, unless `count` is set
    const uint32_t* count = nullptr;  // device ray count (queues sized on the device)
    uint32_t n_max = 0;               // upper bound of *count (grid of the one-ray-per-thread kernel)
    const uint32_t* perm = nullptr;   // output index of each ray position (null: the position)
    uint32_t* next_ray = nullptr;     // one device word used to hand out rays (zeroed per launch)
    int* err = nullptr;               // error word (traversal-stack overflow)
    // closest hit, C-ABI layout (any pointer may be null)
    float* t = nullptr;
    uint32_t* prim = nullptr;
    uint32_t* object = nullptr;
    float2* bary = nullptr;
    // closest hit, render layout: {t, b0, b1, b2} and {prim, object}
    float4* hit4 = nullptr;
    uint2* hit2 = nullptr;
    // any hit
    uint8_t* occluded = nullptr;
};
// Traversal kernels: persistent warps at high occupancy (closest hit 10
// blocks per SM, any hit 12 blocks), persistent
// warps capped at 128 registers (4 blocks per SM), one ray per thread.  All
// give identical results; which is fastest depends on the scene and the rays,
// so it is chosen per scene by timing (tune_cast).
enum Cast_Kernel {
    kCastPersistent64 = 0,
    kCastPersistent128 = 1,
    kCastPerRay = 2,
    kCastPerRayVote = 3,  // one ray per thread, one mode per warp iteration
    kCastKernelCount = 4
};
cudaError_t launch_extend(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream);
cudaError_t launch_shadow(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream);
// Runs the batch once untimed and three times with each kernel (event-timed
// on `stream`), leaving the results of the last run in place; *best = the
// kernel of the shortest run.
cudaError_t tune_cast(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream, cudaEvent_t ev0,
                      cudaEvent_t ev1, int* best);
// ms[k] = kernel k's shortest of `rounds` timed runs (after one untimed run
// when `warm`); the results of the last run stay in place.
cudaError_t time_cast_kernels(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream,
                              cudaEvent_t ev0, cudaEvent_t ev1, int rounds, bool warm, float* ms);

// guide network (guide_mlp.cu).  `box` = scene bounds (min xyz, max xyz)
// for position normalisation.  Query rows: 3 float4 {pos, n.x | n.yz, wo.xy |
// wo.z, -, -, -}; training rows add a 4th float4 and carry the sampled
// direction in the 3rd: {.., wo.z, w.xyz | weight, -, -, -}.
int guide_ensure(yar_gpu_ctx* ctx);
int guide_reset(yar_gpu_ctx* ctx, uint64_t seed);
int guide_set_params(yar_gpu_ctx* ctx, const float* host_params);
void guide_release(yar_gpu_ctx* ctx);
cudaError_t guide_infer(yar_gpu_ctx* ctx, const float4* queries, uint32_t n_max, const uint32_t* count,
                        const float* box, float* lobes, cudaStream_t st);
// One training step over rows offset, offset + stride, ... (n_max of them,
// or as many as `count` holds rows when set): Adam with learning rate `lr`,
// or, with `grad_out`, only the summed gradient of the loss.  The loss sum is
// added to ctx->guide.scalars[0].
cudaError_t guide_train(yar_gpu_ctx* ctx, const float4* samples, uint32_t n_max, const uint32_t* count,
                        uint32_t stride, uint32_t offset, const float* box, const float* w_scale_dev, float lr,
                        float* grad_out, cudaStream_t st);

// render (render.cu)
int render_upload(yar_gpu_ctx* ctx, const yar_flat_scene* scene);
void render_release(yar_gpu_ctx* ctx);
int render_run(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats);
// The direct-lighting algorithm (Raytracer_Config::rendering_algorithm 0), direct.cu.
int render_direct(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats);
int guided_render(yar_gpu_ctx* ctx, const yar_guided_params* params, double* sum_out, float* rgb_out,
                  yar_guided_stats* stats);

// The learned proposal inside the stratified render (guided.cu -> render.cu):
// before each shade launch `before_shade` computes the network inputs of the
// extend queue's hits into `queries` and their lobe mixtures into `lobes`
// (both per queue position, sized for `chunk_paths`); the shade kernel then
// draws continuations from the mixture with probability `alpha`.
struct Guide_Render_Hook {
    const float* lobes = nullptr;
    const float4* queries = nullptr;
    float alpha = 0.f;
    int max_bounce = 0;        // guide the continuations of bounces below this one (0: every bounce)
    uint64_t chunk_paths = 0;  // paths in flight per chunk
    cudaError_t (*before_shade)(void* user, const float4* rays, const float4* hit4, const uint2* hit2,
                                uint32_t count, cudaStream_t st) = nullptr;
    void* user = nullptr;
};
// The path tracer with the scene's pixel sampler at nx x ny samples per
// pixel, pixel streams offset by stream_hi (non-zero: streams independent of
// the reference's), continuations guided through `hook`.
int render_guided_stratified(yar_gpu_ctx* ctx, int nx, int ny, uint32_t stream_hi, const Guide_Render_Hook& hook,
                             float* rgb_out, yar_render_stats* stats);

} // namespace yar
