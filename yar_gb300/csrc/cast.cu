// cast.cu - extend (closest-hit) and shadow (any-hit) kernels over ray batches.
//
// One thread per ray; the ray record is two float4 loads (32 B, coalesced),
// results are written as structure of arrays.  The traversal itself lives in
// device_scene.cuh.
#include "context.hpp"

namespace yar {

namespace {

constexpr int kCastBlock = 128;

__global__ void __launch_bounds__(kCastBlock)
extend_kernel(Device_Scene s, const float4* __restrict__ rays, uint32_t n, float* __restrict__ t_out,
              uint32_t* __restrict__ prim_out, uint32_t* __restrict__ obj_out, float2* __restrict__ bary_out,
              int* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = __ldg(rays + 2 * (size_t)i);
    const float4 b = __ldg(rays + 2 * (size_t)i + 1);
    const float o[3] = {a.x, a.y, a.z};
    const float d[3] = {b.x, b.y, b.z};
    Hit hit;
    const int r = scene_traverse<false>(s, o, d, a.w, hit);
    if (r < 0) {
        atomicOr(err, 1);
        hit.t = a.w;
        hit.prim = hit.object = 0xffffffffu;
        hit.b1 = hit.b2 = 0.f;
    } else if (r == 0) {
        hit.prim = hit.object = 0xffffffffu;
        hit.b1 = hit.b2 = 0.f;
    }
    if (t_out) t_out[i] = hit.t;
    if (prim_out) prim_out[i] = hit.prim;
    if (obj_out) obj_out[i] = hit.object;
    if (bary_out) bary_out[i] = make_float2(hit.b1, hit.b2);
}

__global__ void __launch_bounds__(kCastBlock)
shadow_kernel(Device_Scene s, const float4* __restrict__ rays, uint32_t n, uint8_t* __restrict__ occluded,
              int* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = __ldg(rays + 2 * (size_t)i);
    const float4 b = __ldg(rays + 2 * (size_t)i + 1);
    const float o[3] = {a.x, a.y, a.z};
    const float d[3] = {b.x, b.y, b.z};
    Hit hit;
    const int r = scene_traverse<true>(s, o, d, a.w, hit);
    if (r < 0) atomicOr(err, 1);
    occluded[i] = (uint8_t)(r > 0 ? 1 : 0);
}

} // namespace

cudaError_t launch_extend(const Device_Scene& s, const float4* rays, uint32_t n, float* t, uint32_t* prim,
                          uint32_t* obj, float2* bary, int* err, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kCastBlock - 1) / kCastBlock;
    extend_kernel<<<blocks, kCastBlock, 0, stream>>>(s, rays, n, t, prim, obj, bary, err);
    return cudaGetLastError();
}

cudaError_t launch_shadow(const Device_Scene& s, const float4* rays, uint32_t n, uint8_t* occluded, int* err,
                          cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kCastBlock - 1) / kCastBlock;
    shadow_kernel<<<blocks, kCastBlock, 0, stream>>>(s, rays, n, occluded, err);
    return cudaGetLastError();
}

} // namespace yar
