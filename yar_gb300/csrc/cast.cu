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

#include <atomic>
#include <type_traits>

namespace yar {

namespace {

#ifndef YAR_CAST_NODES_PER_STEP
#define YAR_CAST_NODES_PER_STEP 1
#endif
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
    if (a.t) a.t[i] = status < 0 ? __ldg(a.rays + 2 * (size_t)tr.ray).w : tr.hit.t;
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
                const uint32_t ray = batch_next + rank;
                const float4 r0 = __ldg(a.rays + 2 * (size_t)ray);
                const float4 r1 = __ldg(a.rays + 2 * (size_t)ray + 1);
                tr.begin(s, ray, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), r0.w);
                if (tr.mode() == kDone)  // missed the scene box: done, take another
                    write_result<ANY>(tr, a.perm ? __ldg(a.perm + ray) : ray, a);
                else
                    have = true;
            }
            const uint32_t taken = (uint32_t)__popc(want) < avail ? (uint32_t)__popc(want) : avail;
            batch_next += taken;
            want = __ballot_sync(full, !have && alive);
        }
        // Run one mode for the whole warp: the mode most lanes are in
        // (descents win ties).  Lanes in other modes wait, so the lanes that
        // run share one code path instead of the warp running every mode's
        // code with a few lanes each.
        const int m = have ? tr.mode() : -1;  // every lane with a ray is in one of the three modes
        const unsigned md = __ballot_sync(full, m == kDescend);
        const unsigned mm = __ballot_sync(full, m == kMeshLeaf);
        const unsigned ms = __ballot_sync(full, m == kSceneLeaf);
        if (!(md | mm | ms)) break;
        const int nd = __popc(md), nm = __popc(mm), ns = __popc(ms);
        if (nd >= nm && nd >= ns) {
            if (m == kDescend) tr.template step_descend<MAXD>(s, a.rays, stack);
        } else if (nm >= ns) {
            if (m == kMeshLeaf) tr.step_mesh_leaf(s, a.rays, stack);
        } else {
            if (m == kSceneLeaf) tr.step_scene_leaf(s, a.rays, stack);
        }
        if (have && tr.mode() == kDone) {
            write_result<ANY>(tr, a.perm ? __ldg(a.perm + tr.ray) : tr.ray, a);
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

// One ray per thread as cast_per_ray, but the warp votes each iteration and
// runs one mode for all its lanes, as the persistent kernel does (no hand-out
// of new rays: a lane whose ray is done waits for its warp).  Warps iterate
// together (the grid-stride base is a multiple of 32), so every vote sees
// all 32 lanes.
template <bool ANY>
__global__ void __launch_bounds__(kCastBlock) cast_per_ray_vote(Device_Scene s, Cast_Args a) {
    const unsigned full = 0xffffffffu;
    const uint32_t n = a.count ? *a.count : a.n;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) - lane; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + lane;
        Traversal<ANY> tr;
        Local_Stack stack;
        bool have = false;
        if (i < n) {
            const float4 r0 = __ldg(a.rays + 2 * (size_t)i);
            const float4 r1 = __ldg(a.rays + 2 * (size_t)i + 1);
            tr.begin(s, i, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z), r0.w);
            if (tr.mode() == kDone)
                write_result<ANY>(tr, a.perm ? __ldg(a.perm + i) : i, a);
            else
                have = true;
        }
        for (;;) {
            const int m = have ? tr.mode() : -1;
            const unsigned md = __ballot_sync(full, m == kDescend);
            const unsigned mm = __ballot_sync(full, m == kMeshLeaf);
            const unsigned ms = __ballot_sync(full, m == kSceneLeaf);
            if (!(md | mm | ms)) break;
            const int nd = __popc(md), nm = __popc(mm), ns = __popc(ms);
            if (nd >= nm && nd >= ns) {
                if (m == kDescend) tr.template step_descend<YAR_CAST_NODES_PER_STEP>(s, a.rays, stack);
            } else if (nm >= ns) {
                if (m == kMeshLeaf) tr.step_mesh_leaf(s, a.rays, stack);
            } else {
                if (m == kSceneLeaf) tr.step_scene_leaf(s, a.rays, stack);
            }
            if (have && tr.mode() == kDone) {
                write_result<ANY>(tr, a.perm ? __ldg(a.perm + i) : i, a);
                have = false;
            }
        }
    }
}

// Persistent launch shape, measured on GB300 with the 2.42M-triangle ray-cast
// workload (16M + 16M incoherent rays).  With one mode per warp iteration,
// one node fetch per descent step: closest hit 19.8 ms against 21.3 ms at two
// nodes per step, 21.6 ms at four and 25.7 ms descending to a leaf (the
// per-lane schedule, every mode's code each iteration, took 25.4 ms); a loop
// of node fetches while half the lanes descend (one vote per node) was no
// faster (19.3 against 19.1 ms).  High-occupancy variant: closest hit at 10
// resident blocks of 128 threads per SM (19.0 ms, against 19.7 ms at 8, 19.4
// ms at 12 and 21.0 ms at 6), any hit at 12 blocks (11.2 ms, against 11.6 ms
// at 10, 11.9 ms at 16 and 12.7 ms at 8).  With the traversal state trimmed
// (direction signs in the flags word, 1/d shared by clipping and the
// watertight setup): 18.5 and 10.7 ms; a 4-, 8- or 16-entry shared-memory
// stack with local overflow was slower (18.6-19.2 and 11.4-13.6 ms).
constexpr int kWhileWhile = YAR_CAST_NODES_PER_STEP;
#ifndef YAR_CAST_SHARED_STACK
#define YAR_CAST_SHARED_STACK 0
#endif
constexpr int kSharedStackEntries = YAR_CAST_SHARED_STACK;
#ifndef YAR_CAST_BLOCKS_CLOSEST
#define YAR_CAST_BLOCKS_CLOSEST 10
#endif
#ifndef YAR_CAST_BLOCKS_ANY
#define YAR_CAST_BLOCKS_ANY 12
#endif
template <bool ANY>
constexpr int kHighOccupancyBlocks = ANY ? YAR_CAST_BLOCKS_ANY : YAR_CAST_BLOCKS_CLOSEST;

// Resident blocks of a persistent kernel on the current device: SM count x
// blocks per SM, looked up once per device (devices may differ in SM count).
constexpr int kMaxDevices = 64;
template <class Kernel>
int resident_grid(Kernel kernel, std::atomic<int>* cache) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int>& slot = cache[(unsigned)dev < (unsigned)kMaxDevices ? dev : 0];
    int g = slot.load(std::memory_order_relaxed);
    if (g == 0) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kCastBlock, 0);
        g = sms * (per_sm > 0 ? per_sm : 1);
        if ((unsigned)dev < (unsigned)kMaxDevices) slot.store(g, std::memory_order_relaxed);
    }
    return g;
}

template <bool ANY>
cudaError_t launch(const Device_Scene& s, const Cast_Args& a, int kernel, cudaStream_t stream) {
    if (kernel == kCastPerRay || kernel == kCastPerRayVote) {
        const uint32_t bound = a.count ? a.n_max : a.n;
        if (bound == 0) return cudaSuccess;
        if (kernel == kCastPerRay)
            cast_per_ray<ANY><<<(bound + kCastBlock - 1) / kCastBlock, kCastBlock, 0, stream>>>(s, a);
        else
            cast_per_ray_vote<ANY><<<(bound + kCastBlock - 1) / kCastBlock, kCastBlock, 0, stream>>>(s, a);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(a.next_ray, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    if (kernel == kCastPersistent128) {
        static std::atomic<int> grid[kMaxDevices];
        auto k = cast_persistent<ANY, 4, kWhileWhile, kSharedStackEntries>;
        k<<<resident_grid(k, grid), kCastBlock, 0, stream>>>(s, a);
    } else {
        static std::atomic<int> grid[kMaxDevices];
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

// C-ABI casts take each kernel's best of kTuneRounds timed runs on their
// first large batch (rounds interleave the kernels).
constexpr int kTuneRounds = 3;

int fastest_cast_kernel(const float* ms) {
    int best = 0;
    for (int k = 1; k < kCastKernelCount; k++)
        if (ms[k] < ms[best]) best = k;
    return best;
}

} // namespace

cudaError_t time_cast_kernels(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream,
                              cudaEvent_t ev0, cudaEvent_t ev1, int rounds, bool warm, float* ms_best) {
    auto run = [&](int k) { return any ? launch_shadow(s, a, k, stream) : launch_extend(s, a, k, stream); };
    cudaError_t e = warm ? run(kCastPersistent64) : cudaSuccess;  // warms the caches for the timed runs
    for (int k = 0; k < kCastKernelCount; k++) ms_best[k] = 3.0e38f;
    for (int r = 0; r < rounds; r++) {
        for (int k = 0; k < kCastKernelCount && e == cudaSuccess; k++) {
            e = cudaEventRecord(ev0, stream);
            if (e == cudaSuccess) e = run(k);
            if (e == cudaSuccess) e = cudaEventRecord(ev1, stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
            ms_best[k] = ms < ms_best[k] ? ms : ms_best[k];
        }
    }
    return e;
}

cudaError_t tune_cast(const Device_Scene& s, const Cast_Args& a, bool any, cudaStream_t stream, cudaEvent_t ev0,
                      cudaEvent_t ev1, int* best) {
    float ms[kCastKernelCount] = {};
    cudaError_t e = time_cast_kernels(s, a, any, stream, ev0, ev1, kTuneRounds, true, ms);
    *best = e == cudaSuccess ? fastest_cast_kernel(ms) : kCastPersistent64;
    return e;
}

} // namespace yar
