// cast.cu - extend (closest-hit) and shadow (any-hit) kernels over ray batches.
//
// Persistent warps with dynamic ray fetching: a grid of exactly the resident
// blocks runs until the batch is exhausted; every lane owns one ray's
// traversal state machine (device_scene.cuh) and, when its ray finishes,
// takes the next ray index from a per-warp batch that the warp refills with
// one atomic per kBatch rays.  Incoherent rays have a long-tailed work
// distribution, so this keeps all 32 lanes busy instead of letting a warp idle
// behind its slowest ray.  Ray records are two float4 loads (32 B); results
// are written as structure of arrays at the ray's index.
#include "context.hpp"

#include <type_traits>

namespace yar {

namespace {

constexpr int kCastBlock = 128;
constexpr uint32_t kBatch = 128;  // rays a warp takes per atomic

template <bool ANY>
__device__ __forceinline__ void write_result(const Traversal<ANY>& tr, uint32_t i, float* t_out, uint32_t* prim_out,
                                             uint32_t* obj_out, float2* bary_out, uint8_t* occluded, int* err) {
    if (tr.status < 0) atomicOr(err, 1);
    if (ANY) {
        occluded[i] = (uint8_t)(tr.status > 0 ? 1 : 0);
    } else {
        const bool hit = tr.status > 0;
        if (t_out) t_out[i] = tr.status < 0 ? tr.ray_tmax : tr.hit.t;
        if (prim_out) prim_out[i] = hit ? tr.hit.prim : 0xffffffffu;
        if (obj_out) obj_out[i] = hit ? tr.hit.object : 0xffffffffu;
        if (bary_out) bary_out[i] = hit ? make_float2(tr.hit.b1, tr.hit.b2) : make_float2(0.f, 0.f);
    }
}

template <bool ANY, int MINB, int MAXD, int SHORT>
__global__ void __launch_bounds__(kCastBlock, MINB)
cast_persistent(Device_Scene s, const float4* __restrict__ rays, uint32_t n, uint32_t* __restrict__ next_ray,
                float* __restrict__ t_out, uint32_t* __restrict__ prim_out, uint32_t* __restrict__ obj_out,
                float2* __restrict__ bary_out, uint8_t* __restrict__ occluded, int* __restrict__ err) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    Traversal<ANY> tr;
    __shared__ uint2 stack_smem[SHORT > 0 ? SHORT * kCastBlock : 1];
    typename std::conditional<(SHORT > 0), Split_Stack<SHORT, kCastBlock>, Local_Stack>::type stack;
    if constexpr (SHORT > 0) stack.smem = stack_smem + threadIdx.x;
    uint32_t ray = 0;
    bool have = false, alive = true;
    uint32_t batch_next = 0, batch_end = 0;  // warp-uniform
    for (;;) {
        // hand new rays to lanes without one
        unsigned want = __ballot_sync(full, !have && alive);
        while (want) {
            if (batch_next >= batch_end) {
                uint32_t b = 0;
                if (lane == 0) b = atomicAdd(next_ray, kBatch);
                b = __shfl_sync(full, b, 0);
                batch_next = b;
                batch_end = b + kBatch < n ? b + kBatch : n;
                if (b >= n) {
                    if (!have) alive = false;
                    break;
                }
            }
            const uint32_t avail = batch_end - batch_next;
            const uint32_t rank = (uint32_t)__popc(want & lower);
            if (((want >> lane) & 1u) && rank < avail) {
                ray = batch_next + rank;
                const float4 a = __ldg(rays + 2 * (size_t)ray);
                const float4 b = __ldg(rays + 2 * (size_t)ray + 1);
                tr.begin(s, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), a.w);
                have = true;
            }
            const uint32_t taken = (uint32_t)__popc(want) < avail ? (uint32_t)__popc(want) : avail;
            batch_next += taken;
            want = __ballot_sync(full, !have && alive);
        }
        if (!__any_sync(full, have)) break;
        if (have && !tr.template step<MAXD>(s, stack)) {
            write_result<ANY>(tr, ray, t_out, prim_out, obj_out, bary_out, occluded, err);
            have = false;
        }
    }
}

template <bool ANY, int MINB, int MAXD, int SHORT>
cudaError_t launch_persistent(const Device_Scene& s, const float4* rays, uint32_t n, uint32_t* counter, float* t,
                              uint32_t* prim, uint32_t* obj, float2* bary, uint8_t* occ, int* err,
                              cudaStream_t stream) {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cast_persistent<ANY, MINB, MAXD, SHORT>, kCastBlock, 0);
        grid = sms * (per_sm > 0 ? per_sm : 1);
    }
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    cast_persistent<ANY, MINB, MAXD, SHORT>
        <<<grid, kCastBlock, 0, stream>>>(s, rays, n, counter, t, prim, obj, bary, occ, err);
    return cudaGetLastError();
}

// Launch shape, measured on GB300 with the 2.42M-triangle ray-cast workload
// (16M + 16M incoherent rays): 8 resident blocks of 128 threads per SM
// (64 registers) beat 4 and 6 blocks (102 and 80 registers); descending to a
// leaf per step (while-while) beat one node per step and four nodes per step;
// the local-memory stack beat an 8- or 16-entry shared-memory stack with
// local overflow (770 vs 710 Mrays/s for the best shared variant).
constexpr int kMinBlocksPerSm = 8;
constexpr int kWhileWhile = 1 << 30;
constexpr int kSharedStackEntries = 0;

template <bool ANY>
cudaError_t dispatch(const Device_Scene& s, const float4* rays, uint32_t n, uint32_t* counter, float* t,
                     uint32_t* prim, uint32_t* obj, float2* bary, uint8_t* occ, int* err, cudaStream_t stream) {
    return launch_persistent<ANY, kMinBlocksPerSm, kWhileWhile, kSharedStackEntries>(s, rays, n, counter, t, prim,
                                                                                    obj, bary, occ, err, stream);
}

} // namespace

cudaError_t launch_extend(const Device_Scene& s, const float4* rays, uint32_t n, float* t, uint32_t* prim,
                          uint32_t* obj, float2* bary, int* err, uint32_t* counter, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    return dispatch<false>(s, rays, n, counter, t, prim, obj, bary, nullptr, err, stream);
}

cudaError_t launch_shadow(const Device_Scene& s, const float4* rays, uint32_t n, uint8_t* occluded, int* err,
                          uint32_t* counter, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    return dispatch<true>(s, rays, n, counter, nullptr, nullptr, nullptr, nullptr, occluded, err, stream);
}

} // namespace yar
