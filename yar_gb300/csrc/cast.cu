// cast.cu - extend (closest-hit) and shadow (any-hit) kernels over ray batches.
//
// Persistent warps with dynamic ray fetching: a grid of exactly the resident
// blocks runs until the batch is exhausted; every lane owns one ray's
// traversal state machine (device_scene.cuh) and, when its ray finishes,
// takes the next ray index from a per-warp batch that the warp refills with
// one atomic per kBatch rays.  Incoherent rays have a long-tailed work
// distribution, so this keeps all 32 lanes busy instead of letting a warp idle
// behind its slowest ray.  Ray records are two float4 loads (32 B).
//
// The same kernels serve the C-ABI casts (results as structure of arrays at
// the ray's index) and the render wavefront (hit records at the path slot).
#include "context.hpp"

#include <type_traits>

namespace yar {

namespace {

constexpr int kCastBlock = 128;
constexpr uint32_t kBatch = 128;  // rays a warp takes per atomic

template <bool ANY>
__device__ __forceinline__ void write_result(const Traversal<ANY>& tr, uint32_t i, const Cast_Args& a) {
    const int status = tr.status();
    if (status < 0) atomicOr(a.err, 1);
    if (ANY) {
        a.occluded[i] = (uint8_t)(status > 0 ? 1 : 0);
        return;
    }
    const bool hit = status > 0;
    if (a.hit4) {  // render layout
        a.hit4[i] = make_float4(tr.hit.t, tr.hit.b0, tr.hit.b1, tr.hit.b2);
        a.hit2[i] = hit ? make_uint2(tr.hit.prim, tr.hit.object) : make_uint2(0xffffffffu, 0xffffffffu);
        return;
    }
    if (a.t) a.t[i] = status < 0 ? tr.ray_tmax : tr.hit.t;
    if (a.prim) a.prim[i] = hit ? tr.hit.prim : 0xffffffffu;
    if (a.object) a.object[i] = hit ? tr.hit.object : 0xffffffffu;
    if (a.bary) a.bary[i] = hit ? make_float2(tr.hit.b1, tr.hit.b2) : make_float2(0.f, 0.f);
}

template <bool ANY, int MINB, int MAXD, int SHORT>
__global__ void __launch_bounds__(kCastBlock, MINB) cast_persistent(Device_Scene s, Cast_Args a) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    const uint32_t n = a.count ? *a.count : a.n;
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
                if (lane == 0) b = atomicAdd(a.next_ray, kBatch);
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
                const float4 r0 = __ldg(a.rays + 2 * (size_t)ray);
                const float4 r1 = __ldg(a.rays + 2 * (size_t)ray + 1);
                tr.begin(s, ray, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), r0.w);
                have = true;
            }
            const uint32_t taken = (uint32_t)__popc(want) < avail ? (uint32_t)__popc(want) : avail;
            batch_next += taken;
            want = __ballot_sync(full, !have && alive);
        }
        if (!__any_sync(full, have)) break;
        if (have && !tr.template step<MAXD>(s, a.rays, stack)) {
            write_result<ANY>(tr, a.perm ? __ldg(a.perm + ray) : ray, a);
            have = false;
        }
    }
}

// One ray per thread, start to finish: no hand-out loop and no register cap.
// Best when traversals are short and uniform (small scenes), where the
// persistent loop's per-step votes and the capped kernels' spills cost more
// than the idle lanes they save.
template <bool ANY>
__global__ void __launch_bounds__(kCastBlock) cast_per_ray(Device_Scene s, Cast_Args a) {
    const uint32_t n = a.count ? *a.count : a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r0 = __ldg(a.rays + 2 * (size_t)i);
        const float4 r1 = __ldg(a.rays + 2 * (size_t)i + 1);
        Traversal<ANY> tr;
        Local_Stack stack;
        tr.begin(s, i, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), r0.w);
        while (tr.template step<1 << 30>(s, a.rays, stack)) {
        }
        write_result<ANY>(tr, a.perm ? __ldg(a.perm + i) : i, a);
    }
}

// Persistent launch shape, measured on GB300 with the 2.42M-triangle ray-cast
// workload (16M + 16M incoherent rays).  High-occupancy variant: closest hit
// at 8 resident blocks of 128 threads per SM (64 registers: 25.3 ms, against
// 25.2 ms at 10 blocks, 26.4 ms at 12, 31.1 ms at 16), any hit at 12 blocks
// (40 registers: 12.6 ms, against 14.3 ms at 8, 13.3 ms at 10, 14.1 ms at
// 16).  Descending to a leaf per step (while-while) beat one node per step
// and four nodes per step; testing all of a leaf's triangles in one step was
// slower (27.0 against 25.3 ms); the local-memory stack beat an 8- or
// 16-entry shared-memory stack with local overflow.
constexpr int kWhileWhile = 1 << 30;
constexpr int kSharedStackEntries = 0;
template <bool ANY>
constexpr int kHighOccupancyBlocks = ANY ? 12 : 8;

template <class Kernel>
int resident_grid(Kernel kernel, int& cache) {
    if (cache == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kCastBlock, 0);
        cache = sms * (per_sm > 0 ? per_sm : 1);
    }
    return cache;
}

template <bool ANY>
cudaError_t launch(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream) {
    if (kernel == kCastPerRay) {
        const uint32_t bound = a.count ? a.n_max : a.n;
        if (bound == 0) return cudaSuccess;
        cast_per_ray<ANY><<<(bound + kCastBlock - 1) / kCastBlock, kCastBlock, 0, stream>>>(s, a);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(a.next_ray, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    if (kernel == kCastPersistent128) {
        static int grid = 0;
        auto k = cast_persistent<ANY, 4, kWhileWhile, kSharedStackEntries>;
        k<<<resident_grid(k, grid), kCastBlock, 0, stream>>>(s, a);
    } else {
        static int grid = 0;
        auto k = cast_persistent<ANY, kHighOccupancyBlocks<ANY>, kWhileWhile, kSharedStackEntries>;
        k<<<resident_grid(k, grid), kCastBlock, 0, stream>>>(s, a);
    }
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_extend(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream) {
    if (!a.count && a.n == 0) return cudaSuccess;
    return launch<false>(s, a, kernel, stream);
}

cudaError_t launch_shadow(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream) {
    if (!a.count && a.n == 0) return cudaSuccess;
    return launch<true>(s, a, kernel, stream);
}

namespace {

cudaError_t time_cast_kernels(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream,
                              cudaEvent_t ev0, cudaEvent_t ev1, float* ms_acc) {
    auto run = [&](int k) { return any ? launch_shadow(s, a, k, stream) : launch_extend(s, a, k, stream); };
    cudaError_t e = run(kCastPersistent64);  // warms the caches for the timed runs
    for (int k = 0; k < kCastKernelCount && e == cudaSuccess; k++) {
        e = cudaEventRecord(ev0, stream);
        if (e == cudaSuccess) e = run(k);
        if (e == cudaSuccess) e = cudaEventRecord(ev1, stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
        ms_acc[k] += ms;
    }
    return e;
}

int fastest_cast_kernel(const float* ms) {
    int best = 0;
    for (int k = 1; k < kCastKernelCount; k++)
        if (ms[k] < ms[best]) best = k;
    return best;
}

} // namespace

cudaError_t tune_cast(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream, cudaEvent_t ev0,
                      cudaEvent_t ev1, int* best) {
    float ms[kCastKernelCount] = {};
    cudaError_t e = time_cast_kernels(s, a, any, stream, ev0, ev1, ms);
    *best = e == cudaSuccess ? fastest_cast_kernel(ms) : kCastPersistent64;
    return e;
}

} // namespace yar
