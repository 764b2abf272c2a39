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
    Device_Buffer object_info;  // int4 per object: material type, material index, light type, light index
    Device_Buffer object_to_world;         // float[12] per object
    Device_Buffer object_to_world_normal;  // float[12] per object
    std::vector<yar_material_desc> host_materials;
    std::vector<yar_rect_light_desc> host_rect_lights;
    std::vector<int32_t> host_object_info;
    yar_camera_desc camera{};
    yar_render_config config{};
    uint32_t other_light_count = 0;
    uint32_t triangle_total = 0;
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
    uint32_t* d_counter = nullptr;  // ray hand-out counter of the persistent cast kernels

    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;

    // render scratch (path state, queues, per-pixel sample tables)
    std::vector<yar::Device_Buffer> render_scratch;
};

namespace yar {

int fail(yar_gpu_ctx* ctx, int code, const std::string& message);
int cuda_fail(yar_gpu_ctx* ctx, cudaError_t e, const char* what);
int device_alloc(yar_gpu_ctx* ctx, Device_Buffer& b, size_t bytes);
void device_free(Device_Buffer& b);

// kernels (cast.cu)
// `counter` is one device word the persistent kernels use to hand out rays.
cudaError_t launch_extend(const Device_Scene& s, const float4* rays, uint32_t n, float* t, uint32_t* prim,
                          uint32_t* obj, float2* bary, int* err, uint32_t* counter, cudaStream_t stream);
cudaError_t launch_shadow(const Device_Scene& s, const float4* rays, uint32_t n, uint8_t* occluded, int* err,
                          uint32_t* counter, cudaStream_t stream);

// render (render.cu)
int render_upload(yar_gpu_ctx* ctx, const yar_flat_scene* scene);
void render_release(yar_gpu_ctx* ctx);
int render_run(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats);

} // namespace yar
