// guide_mlp.cu - the network of the learned directional proposal: a BF16
// MLP with FP32 accumulation on the tensor cores (tcgen05, accumulators in
// tensor memory), with hand-written inference and training kernels.
//
// Network: 128 inputs (16-frequency sin/cos encoding of the normalised
// position, frequencies pi f_k, f_k = (2^((k mod 3)/3) in float32) 2^(k div 3),
// k = 0..15: 96; shading normal 3,
// outgoing direction 3, zeros, input 127 = constant 1) -> 3 hidden layers of 64 ReLU units (unit 63 of each is the
// constant 1, so every bias is an ordinary weight column) -> 64 outputs, of
// which 40 parameterise a mixture of 8 von Mises-Fisher lobes in world space:
// per lobe an unnormalised mean direction m (3), log-concentration r and a
// mixture logit l.  kappa = exp(clamp(r, -3, 8)), pi = softmax(l).
//
// One CTA of 128 threads handles tiles of 128 rows (= TMEM lanes = threads);
// a single thread issues the MMAs (M = 128, N = 64, K = 16 per instruction),
// all threads run the epilogues (tcgen05.ld of their lane, bias-free ReLU,
// BF16 pack into the next layer's operand tile).  Training fuses the forward
// pass, the loss gradient, the backward pass and the weight gradients: the
// weight gradients dW^T = A^T dY accumulate in tensor memory over all tiles a
// CTA processes (the transposed operand tiles are written by the epilogues),
// and each CTA writes one partial gradient; adam_kernel sums the partials.
//
// Loss for a sample direction w drawn with pdf p at (x, n, wo) with target
// value t (incident radiance x BSDF x cosine, as luminance): -(t / p) log q(w),
// whose expectation is the KL divergence from the normalised target to the
// mixture q up to a constant (the estimator of neural importance sampling).
#include "context.hpp"
#include "tc.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <random>
#include <vector>

namespace yar {

namespace {

constexpr int kRows = 128;
constexpr int kIn = 128;
constexpr int kHid = 64;
constexpr int kOut = 64;
constexpr uint32_t kWaitLimit = 1u << 20;  // mbarrier polls before a tile is abandoned

// parameter vector, fp32, row-major [out][in]
constexpr int kW1 = 0;
constexpr int kW2 = kW1 + kHid * kIn;
constexpr int kW3 = kW2 + kHid * kHid;
constexpr int kW4 = kW3 + kHid * kHid;
static_assert(kW4 + kOut * kHid == kGuideParams, "parameter count");

// bf16 operand images in tile layout: W1 (64 x 128), W2..W4 (64 x 64), then
// the transposed W2..W4 (rows = input unit, K = output unit) for the backward pass
constexpr uint32_t kImgW1 = 0, kImgW2 = 16384, kImgW3 = 24576, kImgW4 = 32768;
constexpr uint32_t kImgW2t = 40960, kImgW3t = 49152, kImgW4t = 57344, kImgBytes = 65536;

// shared memory, training: images | R0 (32 KB rows) | H1t H2t H3t dT (16 KB each) | Xt (32 KB) | misc
// H_t tiles hold 64 rows but the M = 128 MMA reads 128: rows 64..127 come
// from the next tile in this list (their products land in TMEM lanes that
// are never read).
constexpr uint32_t kTrR0 = kImgBytes;
constexpr uint32_t kTrH1t = kTrR0 + 32768;
constexpr uint32_t kTrH2t = kTrH1t + 16384;
constexpr uint32_t kTrH3t = kTrH2t + 16384;
constexpr uint32_t kTrDT = kTrH3t + 16384;
constexpr uint32_t kTrXt = kTrDT + 16384;
constexpr uint32_t kTrMisc = kTrXt + 32768;
// shared memory, inference: W1..W4 images | R0 | misc
constexpr uint32_t kInR0 = kImgW2t;
constexpr uint32_t kInMisc = kInR0 + 32768;

constexpr uint32_t kIdesc = tc::idesc_bf16_f32(128, 64);

struct Mlp_Args {
    const uint8_t* images;
    const float4* rows;  // 3 float4 per query row, 4 per training row
    uint32_t n;
    const uint32_t* count;
    uint32_t stride, offset;  // row r of this launch is input row offset + r * stride
    float3 lo, inv_ext;
    float* lobes;          // inference: kGuideLobeFloats per row
    float* partials;       // training: kGuideParams per CTA
    const float* w_scale;  // training
    float* loss;           // training
    int* err;
};

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Encoding frequencies f_k = f_(k mod 3) 2^(k div 3), k = 0..15 (1 to 32
// half-periods across the scene box), from the float32 values of 2^(b/3),
// b = 0, 1, 2: three chains of doublings.
__constant__ float kFreq[3] = {1.000000000e+00f, 1.259921074e+00f, 1.587401032e+00f};

// Input features j and j + 1 (j even), visited in increasing j.  j < 96: sin
// and cos of pi f_k p_axis, k = j / 6, axis = (j % 6) / 2: a sincospif for
// k < 3, then each chain (axis, k mod 3) doubles its angle (sin 2x =
// 2 sin x cos x, cos 2x = (cos x - sin x)(cos x + sin x)), which leaves the
// features within 1e-6 of sincospif's, far below their BF16 rounding.  Then
// the normal, wo, zeros and the constant 1 at 127.
struct Encoding {
    float s[3][3], c[3][3];  // running sin and cos per (axis, chain)
};
__device__ __forceinline__ void feature_pair(int j, float3 p, float3 nrm, float3 wo, bool valid, Encoding& e,
                                             float& f0, float& f1) {
    if (j < 96) {
        const int k = j / 6, a = (j % 6) / 2, b = k % 3;
        if (k < 3) {
            const float x = (a == 0) ? p.x : (a == 1 ? p.y : p.z);
            sincospif(x * kFreq[b], &e.s[a][b], &e.c[a][b]);
        } else {
            const float sn = e.s[a][b], cs = e.c[a][b];
            e.s[a][b] = 2.f * sn * cs;
            e.c[a][b] = (cs - sn) * (cs + sn);
        }
        f0 = valid ? e.s[a][b] : 0.f;
        f1 = valid ? e.c[a][b] : 0.f;
        return;
    }
    if (!valid) {
        f0 = f1 = 0.f;
        return;
    }
    auto fixed = [&](int i) -> float {
        switch (i) {
            case 96: return nrm.x;
            case 97: return nrm.y;
            case 98: return nrm.z;
            case 99: return wo.x;
            case 100: return wo.y;
            case 101: return wo.z;
            case 127: return 1.f;
            default: return 0.f;
        }
    };
    f0 = fixed(j);
    f1 = fixed(j + 1);
}

// Transposed tile write: element (feature f, batch row r) of a tile with
// K = 128 batch columns; neighbouring rows pair up into one 4-byte store.
__device__ __forceinline__ void store_t(uint8_t* tile, int f, int r, float v) {
    const float u = __shfl_down_sync(0xffffffffu, v, 1);
    if ((r & 1) == 0) *reinterpret_cast<uint32_t*>(tile + tc::tile_offset(f, r, 128)) = pack_bf16(v, u);
}

__device__ __forceinline__ void store_row8(uint8_t* tile, int r, int k0, int K, const float* v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + tc::tile_offset(r, k0, K)) = q;
}

// A tile (M = 128 rows, K = ksteps * 16) times a B tile (N = 64 rows, same K).
__device__ __forceinline__ void gemm(uint32_t d_tmem, uint32_t a, uint32_t b, int K, bool accumulate) {
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int s = 0; s < K / 16; s++) {
        const uint64_t ad = tc::smem_desc(a + 256u * s, 128u, sbo);
        const uint64_t bd = tc::smem_desc(b + 256u * s, 128u, sbo);
        tc::mma(d_tmem, ad, bd, kIdesc, (accumulate || s > 0) ? 1u : 0u);
    }
}

__device__ __forceinline__ void load64(uint32_t taddr, float (&v)[64]) {
    float* p = v;
    tc::tmem_ld16(taddr + 0, *reinterpret_cast<float(*)[16]>(p + 0));
    tc::tmem_ld16(taddr + 16, *reinterpret_cast<float(*)[16]>(p + 16));
    tc::tmem_ld16(taddr + 32, *reinterpret_cast<float(*)[16]>(p + 32));
    tc::tmem_ld16(taddr + 48, *reinterpret_cast<float(*)[16]>(p + 48));
    tc::tmem_wait_ld();
}

// Issue barrier: the generic-proxy shared-memory writes of all threads become
// visible to the tensor core, and tensor-memory reads of the epilogue are
// ordered before the next MMA.
__device__ __forceinline__ void to_mma() {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
}

// Mixture parameters and the loss gradient of one row (training) from the 40
// raw outputs; `d` receives d(loss)/d(raw).
__device__ __forceinline__ float mixture_grad(const float (&o)[64], float3 w_dir, float wt, float (&d)[64]) {
    float lp[8], lv[8], kap[8], len[8], cdot[8], inrange[8];
    float3 mu[8];
    float lmax = -1e30f;
#pragma unroll
    for (int k = 0; k < 8; k++) lmax = fmaxf(lmax, o[5 * k + 4]);
    float lsum = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) lsum += __expf(o[5 * k + 4] - lmax);
    const float llse = lmax + __logf(lsum);
    float qmax = -1e30f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float mx = o[5 * k], my = o[5 * k + 1], mz = o[5 * k + 2];
        len[k] = sqrtf(mx * mx + my * my + mz * mz) + 1e-6f;
        mu[k] = make_float3(mx / len[k], my / len[k], mz / len[k]);
        const float r = o[5 * k + 3];
        const float rc = fminf(fmaxf(r, -3.f), 8.f);
        inrange[k] = (r > -3.f && r < 8.f) ? 1.f : 0.f;
        kap[k] = __expf(rc);
        cdot[k] = mu[k].x * w_dir.x + mu[k].y * w_dir.y + mu[k].z * w_dir.z;
        lp[k] = o[5 * k + 4] - llse;
        // log C(kappa) = log kappa - log(2 pi) - log(1 - exp(-2 kappa))
        lv[k] = rc - 1.8378770664f - log1pf(-__expf(-2.f * kap[k])) + kap[k] * (cdot[k] - 1.f);
        qmax = fmaxf(qmax, lp[k] + lv[k]);
    }
    float qs = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) qs += __expf(lp[k] + lv[k] - qmax);
    const float logq = qmax + __logf(qs);
#pragma unroll
    for (int j = 0; j < 64; j++) d[j] = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float gam = __expf(lp[k] + lv[k] - logq);
        const float pik = __expf(lp[k]);
        d[5 * k + 4] = -wt * (gam - pik);
        const float e2 = __expf(-2.f * kap[k]);
        const float dlv = 1.f / kap[k] - 2.f * e2 / (1.f - e2) + (cdot[k] - 1.f);
        d[5 * k + 3] = -wt * gam * dlv * kap[k] * inrange[k];
        const float s = -wt * gam * kap[k] / len[k];
        d[5 * k + 0] = s * (w_dir.x - cdot[k] * mu[k].x);
        d[5 * k + 1] = s * (w_dir.y - cdot[k] * mu[k].y);
        d[5 * k + 2] = s * (w_dir.z - cdot[k] * mu[k].z);
    }
    return -wt * logq;
}

template <bool TRAIN>
__global__ void __launch_bounds__(kRows, 1) mlp_kernel(Mlp_Args a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = tc::smem_addr(sm);
    const uint32_t misc = TRAIN ? kTrMisc : kInMisc;
    const uint32_t mbar = base + misc;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + misc + 8);
    constexpr uint32_t kCols = TRAIN ? 512u : 64u;

    const uint32_t img_bytes = TRAIN ? kImgBytes : kImgW2t;
    for (uint32_t i = tid; i < img_bytes / 16; i += kRows)
        reinterpret_cast<uint4*>(sm)[i] = __ldg(reinterpret_cast<const uint4*>(a.images) + i);
    if (warp == 0) tc::tmem_alloc(base + misc + 8, kCols);
    if (tid == 0) {
        tc::mbar_init(mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);

    const uint32_t n = a.count ? (*a.count > a.offset ? (*a.count - a.offset + a.stride - 1) / a.stride : 0u) : a.n;
    const uint32_t tiles = (n + kRows - 1) / kRows;
    const uint32_t r0 = base + (TRAIN ? kTrR0 : kInR0);
    uint8_t* R0 = sm + (TRAIN ? kTrR0 : kInR0);
    uint32_t parity = 0;
    bool ok = true;
    uint32_t done_tiles = 0;
    float loss_sum = 0.f;
    const float w_scale = TRAIN ? __ldg(a.w_scale) : 0.f;

    auto wait_mma = [&]() {
        const bool got = tc::mbar_wait(mbar, parity, kWaitLimit);
        parity ^= 1u;
        tc::fence_after_sync();
        return got;
    };

    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t row = tile * kRows + tid;
        const bool valid = row < n;
        float3 p = make_float3(0.f, 0.f, 0.f), nrm = p, wo = p, wdir = p;
        float wt = 0.f;
        if (valid) {
            const float4* q = a.rows + ((size_t)a.offset + (size_t)row * a.stride) * (TRAIN ? 4 : 3);
            const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
            p = make_float3((q0.x - a.lo.x) * a.inv_ext.x, (q0.y - a.lo.y) * a.inv_ext.y,
                            (q0.z - a.lo.z) * a.inv_ext.z);
            nrm = make_float3(q0.w, q1.x, q1.y);
            wo = make_float3(q1.z, q1.w, q2.x);
            if (TRAIN) {
                wdir = make_float3(q2.y, q2.z, q2.w);
                wt = __ldg(q + 3).x * w_scale;
            }
        }
        // ---- input features: X rows (and X^T for the weight gradient of layer 1)
        Encoding enc;
#pragma unroll
        for (int c = 0; c < 16; c++) {
            float v[8];
#pragma unroll
            for (int i = 0; i < 8; i += 2) feature_pair(8 * c + i, p, nrm, wo, valid, enc, v[i], v[i + 1]);
            store_row8(R0, tid, 8 * c, kIn, v);
            if (TRAIN) {
#pragma unroll
                for (int i = 0; i < 8; i++) store_t(sm + kTrXt, 8 * c + i, tid, v[i]);
            }
        }
        to_mma();
        if (tid == 0) {
            tc::fence_after_sync();
            gemm(tmem, r0, base + kImgW1, kIn, false);
            tc::commit(mbar);
        }
        ok = wait_mma();
        uint32_t mask[3][2];
        // ---- hidden layers
#pragma unroll 1
        for (int l = 0; l < 3; l++) {
            float v[64];
            load64(lane_addr, v);
            mask[l][0] = mask[l][1] = 0u;
#pragma unroll
            for (int j = 0; j < 64; j++) {
                if (j < 63) {
                    if (v[j] > 0.f) mask[l][j >> 5] |= 1u << (j & 31);
                    v[j] = fmaxf(v[j], 0.f);
                } else {
                    v[j] = valid ? 1.f : 0.f;
                }
            }
            // layer l's output: rows into R0 (ping-pong halves), transposed into H(l+1)t
            uint8_t* dst = R0 + ((l & 1) ? 16384 : 0);
#pragma unroll
            for (int c = 0; c < 8; c++) store_row8(dst, tid, 8 * c, kHid, v + 8 * c);
            if (TRAIN) {
                uint8_t* ht = sm + kTrH1t + 16384u * l;
#pragma unroll
                for (int j = 0; j < 64; j++) store_t(ht, j, tid, v[j]);
            }
            to_mma();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t w = base + (l == 0 ? kImgW2 : (l == 1 ? kImgW3 : kImgW4));
                gemm(tmem, r0 + ((l & 1) ? 16384u : 0u), w, kHid, false);
                tc::commit(mbar);
            }
            ok = wait_mma() && ok;
        }
        // ---- output layer: mixture parameters (inference) or loss gradient (training)
        {
            float o[64];
            load64(lane_addr, o);
            if (!TRAIN) {
                if (valid) {
                    float lmax = -1e30f;
#pragma unroll
                    for (int k = 0; k < 8; k++) lmax = fmaxf(lmax, o[5 * k + 4]);
                    float e[8], es = 0.f;
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        e[k] = __expf(o[5 * k + 4] - lmax);
                        es += e[k];
                    }
                    float4* out = reinterpret_cast<float4*>(a.lobes + (size_t)row * kGuideLobeFloats);
                    float f[40];
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const float mx = o[5 * k], my = o[5 * k + 1], mz = o[5 * k + 2];
                        const float il = 1.f / (sqrtf(mx * mx + my * my + mz * mz) + 1e-6f);
                        f[5 * k + 0] = mx * il;
                        f[5 * k + 1] = my * il;
                        f[5 * k + 2] = mz * il;
                        f[5 * k + 3] = __expf(fminf(fmaxf(o[5 * k + 3], -3.f), 8.f));
                        f[5 * k + 4] = e[k] / es;
                    }
#pragma unroll
                    for (int i = 0; i < 10; i++) out[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
                }
            } else {
                float d[64];
                const float l = mixture_grad(o, wdir, wt, d);
                if (valid) loss_sum += l;
#pragma unroll
                for (int c = 0; c < 8; c++) store_row8(R0 + 16384, tid, 8 * c, kOut, d + 8 * c);
#pragma unroll
                for (int j = 0; j < 64; j++) store_t(sm + kTrDT, j, tid, d[j]);
            }
        }
        if (TRAIN) {
            const bool acc = done_tiles > 0;
            // backward through layers 4, 3, 2: dH = (dY W) masked; dW^T += A^T dY
#pragma unroll 1
            for (int l = 2; l >= 0; l--) {
                to_mma();
                if (tid == 0) {
                    tc::fence_after_sync();
                    const uint32_t wt_img = base + (l == 2 ? kImgW4t : (l == 1 ? kImgW3t : kImgW2t));
                    const uint32_t dy_rows = r0 + ((l & 1) ? 0u : 16384u);  // dOut in R0b, dH3 in R0a, dH2 in R0b
                    gemm(tmem, dy_rows, wt_img, kOut, false);
                    gemm(tmem + 128u + 64u * (uint32_t)l, base + kTrH1t + 16384u * (uint32_t)l, base + kTrDT, kRows,
                         acc);
                    tc::commit(mbar);
                }
                ok = wait_mma() && ok;
                float v[64];
                load64(lane_addr, v);
#pragma unroll
                for (int j = 0; j < 64; j++) v[j] = ((mask[l][j >> 5] >> (j & 31)) & 1u) ? v[j] : 0.f;
                if (l > 0) {
                    uint8_t* dst = R0 + ((l & 1) ? 16384 : 0);
#pragma unroll
                    for (int c = 0; c < 8; c++) store_row8(dst, tid, 8 * c, kHid, v + 8 * c);
                }
#pragma unroll
                for (int j = 0; j < 64; j++) store_t(sm + kTrDT, j, tid, v[j]);
            }
            to_mma();
            if (tid == 0) {
                tc::fence_after_sync();
                gemm(tmem + 64u, base + kTrXt, base + kTrDT, kRows, acc);
                tc::commit(mbar);
            }
            ok = wait_mma() && ok;
        }
        done_tiles++;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.err, 2);
            break;
        }
    }

    if (TRAIN) {
        // partial gradients of this CTA, in the parameter layout [out][in]
        float* part = a.partials + (size_t)blockIdx.x * kGuideParams;
        float v[64];
        if (done_tiles > 0 && ok) {
            load64(lane_addr + 64u, v);
#pragma unroll
            for (int j = 0; j < 64; j++) part[kW1 + j * kIn + tid] = v[j];
            if (warp < 2) {
#pragma unroll 1
                for (int l = 0; l < 3; l++) {
                    load64(lane_addr + 128u + 64u * (uint32_t)l, v);
                    const int off = l == 0 ? kW2 : (l == 1 ? kW3 : kW4);
#pragma unroll
                    for (int j = 0; j < 64; j++) part[off + j * kHid + tid] = v[j];
                }
            }
        } else {
            for (int i = tid; i < kGuideParams; i += kRows) part[i] = 0.f;
        }
        float s = loss_sum;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((tid & 31) == 0 && s != 0.f) atomicAdd(a.loss, s);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// The MLP kernels' bounded mbarrier wait on a barrier that nothing arrives
// at: the limit runs out, the error word is set and the kernel returns, with
// no copy or MMA in flight.  Exercises the expiry path of the wait.
__global__ void wait_selftest_kernel(uint32_t limit, int* err) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(&mbar);
        tc::mbar_init(a, 1);
        if (!tc::mbar_wait(a, 0, limit)) atomicExch(err, 1);
    }
}

// fp32 parameters -> bf16 operand images (forward and transposed).
__global__ void images_kernel(const float* __restrict__ params, uint8_t* __restrict__ img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGuideParams) return;
    const float w = params[i];
    const __nv_bfloat16 b = __float2bfloat16_rn(w);
    auto put = [&](uint32_t off) { *reinterpret_cast<__nv_bfloat16*>(img + off) = b; };
    if (i < kW2) {
        const int nn = i / kIn, k = i % kIn;
        put(kImgW1 + tc::tile_offset(nn, k, kIn));
        return;
    }
    const int l = (i - kW2) / (kHid * kHid);  // 0: W2, 1: W3, 2: W4
    const int j = (i - kW2) % (kHid * kHid);
    const int nn = j / kHid, k = j % kHid;
    const uint32_t fwd = l == 0 ? kImgW2 : (l == 1 ? kImgW3 : kImgW4);
    const uint32_t bwd = l == 0 ? kImgW2t : (l == 1 ? kImgW3t : kImgW4t);
    put(fwd + tc::tile_offset(nn, k, kHid));
    put(bwd + tc::tile_offset(k, nn, kHid));
}

// Sum of the per-CTA partial gradients; Adam step when `lr` > 0, else the
// summed gradient is written to `grad_out`.
__global__ void adam_kernel(const float* __restrict__ partials, int parts, float* __restrict__ params,
                            float* __restrict__ m, float* __restrict__ v, float lr, float beta1, float beta2,
                            float eps, float c1, float c2, float* __restrict__ grad_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGuideParams) return;
    float g = 0.f;
    for (int c = 0; c < parts; c++) g += partials[(size_t)c * kGuideParams + i];
    if (grad_out) {
        grad_out[i] = g;
        return;
    }
    const float mi = beta1 * m[i] + (1.f - beta1) * g;
    const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    params[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// The current device's SM count (the partial-gradient slots and the grids),
// cached per device.
int sm_count() {
    static int sms[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (sms[dev] == 0) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    return sms[dev];
}

} // namespace

int guide_ensure(yar_gpu_ctx* ctx) {
    Guide& g = ctx->guide;
    if (g.params.ptr) return YAR_OK;
    int rc = YAR_OK;
    const size_t pb = kGuideParams * sizeof(float);
    cudaSetDevice(ctx->device);
    if (sm_count() <= 0) return fail(ctx, YAR_ERR_INVALID, "guide: no SM count for the device");
    if ((rc = device_alloc(ctx, g.params, pb)) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, g.adam_m, pb)) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, g.adam_v, pb)) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, g.images, kImgBytes)) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, g.partials, (size_t)sm_count() * pb)) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, g.scalars, 64)) != YAR_OK) return rc;
    cudaError_t e = cudaMemsetAsync(g.images.ptr, 0, kImgBytes, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "guide init");
    static bool attr[64] = {};  // per device
    if (ctx->device < 0 || ctx->device >= 64) return fail(ctx, YAR_ERR_INVALID, "guide: device index");
    if (!attr[ctx->device]) {
        e = cudaFuncSetAttribute(mlp_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrMisc + 64);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mlp_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kInMisc + 64);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "guide kernel attributes");
        attr[ctx->device] = true;
    }
    return guide_reset(ctx, 1);
}

int guide_reset(yar_gpu_ctx* ctx, uint64_t seed) {
    // He-uniform hidden weights, small output weights (broad, even lobes at
    // the start), zero bias columns.
    std::vector<float> w(kGuideParams, 0.f);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    auto fill = [&](int off, int rows, int cols, int fan_in, float gain, int used_rows, int used_cols) {
        const float b = gain * std::sqrt(6.f / (float)fan_in);
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < cols; c++)
                w[off + r * cols + c] = (r < used_rows && c < used_cols) ? b * u(rng) : 0.f;
    };
    fill(kW1, kHid, kIn, 102, 1.f, kHid - 1, 102);
    fill(kW2, kHid, kHid, kHid - 1, 1.f, kHid - 1, kHid - 1);
    fill(kW3, kHid, kHid, kHid - 1, 1.f, kHid - 1, kHid - 1);
    fill(kW4, kOut, kHid, kHid - 1, 0.1f, kGuideLobeFloats, kHid - 1);
    return guide_set_params(ctx, w.data());
}

int guide_set_params(yar_gpu_ctx* ctx, const float* host_params) {
    Guide& g = ctx->guide;
    const size_t pb = kGuideParams * sizeof(float);
    cudaError_t e = cudaMemcpyAsync(g.params.ptr, host_params, pb, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g.adam_m.ptr, 0, pb, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g.adam_v.ptr, 0, pb, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "guide parameters");
    g.step = 0;
    images_kernel<<<(kGuideParams + 255) / 256, 256, 0, ctx->stream>>>((const float*)g.params.ptr,
                                                                        (uint8_t*)g.images.ptr);
    e = cudaStreamSynchronize(ctx->stream);  // the host vector may die at return
    if (e != cudaSuccess) return cuda_fail(ctx, e, "guide parameters");
    return YAR_OK;
}

cudaError_t guide_infer(yar_gpu_ctx* ctx, const float4* queries, uint32_t n_max, const uint32_t* count,
                        const float* box, float* lobes, cudaStream_t st) {
    Guide& g = ctx->guide;
    if (n_max == 0) return cudaSuccess;
    Mlp_Args a{};
    a.images = (const uint8_t*)g.images.ptr;
    a.rows = queries;
    a.n = n_max;
    a.count = count;
    a.stride = 1;
    a.offset = 0;
    a.lo = make_float3(box[0], box[1], box[2]);
    a.inv_ext = make_float3(1.f / std::max(box[3] - box[0], 1e-20f), 1.f / std::max(box[4] - box[1], 1e-20f),
                            1.f / std::max(box[5] - box[2], 1e-20f));
    a.lobes = lobes;
    a.err = ctx->d_error;
    const uint32_t tiles = (n_max + kRows - 1) / kRows;
    const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sm_count() * 3u);  // 3 CTAs fit per SM
    mlp_kernel<false><<<grid, kRows, kInMisc + 64, st>>>(a);
    return cudaGetLastError();
}

cudaError_t guide_train(yar_gpu_ctx* ctx, const float4* samples, uint32_t n_max, const uint32_t* count,
                        uint32_t stride, uint32_t offset, const float* box, const float* w_scale_dev, float lr,
                        float* grad_out, cudaStream_t st) {
    Guide& g = ctx->guide;
    if (n_max == 0) return cudaSuccess;
    Mlp_Args a{};
    a.images = (const uint8_t*)g.images.ptr;
    a.rows = samples;
    a.n = n_max;
    a.count = count;
    a.stride = stride;
    a.offset = offset;
    a.lo = make_float3(box[0], box[1], box[2]);
    a.inv_ext = make_float3(1.f / std::max(box[3] - box[0], 1e-20f), 1.f / std::max(box[4] - box[1], 1e-20f),
                            1.f / std::max(box[5] - box[2], 1e-20f));
    a.partials = (float*)g.partials.ptr;
    a.w_scale = w_scale_dev;
    a.loss = (float*)g.scalars.ptr;
    a.err = ctx->d_error;
    const uint32_t tiles = (n_max + kRows - 1) / kRows;
    const int grid = (int)std::min<uint32_t>(tiles, (uint32_t)sm_count());
    mlp_kernel<true><<<grid, kRows, kTrMisc + 64, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    float c1 = 1.f, c2 = 1.f;
    if (!grad_out) {
        g.step++;
        c1 = 1.f / (1.f - std::pow(g.beta1, (float)g.step));
        c2 = 1.f / (1.f - std::pow(g.beta2, (float)g.step));
    }
    adam_kernel<<<(kGuideParams + 255) / 256, 256, 0, st>>>((const float*)g.partials.ptr, grid, (float*)g.params.ptr,
                                                            (float*)g.adam_m.ptr, (float*)g.adam_v.ptr, lr, g.beta1,
                                                            g.beta2, g.eps, c1, c2, grad_out);
    if (!grad_out)
        images_kernel<<<(kGuideParams + 255) / 256, 256, 0, st>>>((const float*)g.params.ptr, (uint8_t*)g.images.ptr);
    return cudaGetLastError();
}

void guide_release(yar_gpu_ctx* ctx) {
    Guide& g = ctx->guide;
    for (Device_Buffer* b : {&g.params, &g.adam_m, &g.adam_v, &g.images, &g.partials, &g.scalars}) device_free(*b);
}


// ---------------------------------------------------------------- C ABI
namespace {

int guide_call_prologue(yar_gpu_ctx* ctx) {
    if (!ctx) return YAR_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return guide_ensure(ctx);
}

int guide_finish(yar_gpu_ctx* ctx, cudaError_t e, const char* what, float* loss) {
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    if (loss) {
        e = cudaMemcpy(loss, ctx->guide.scalars.ptr, sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    }
    int h = 0;
    e = cudaMemcpy(&h, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    if (h) {
        cudaMemset(ctx->d_error, 0, sizeof(int));
        return fail(ctx, YAR_ERR_TIMEOUT, "tensor-core wait gave up");
    }
    return YAR_OK;
}

int guide_step(yar_gpu_ctx* ctx, const float* samples, uint32_t n, const float* box, float weight_scale, float lr,
               float* grad, float* loss) {
    int rc = guide_call_prologue(ctx);
    if (rc != YAR_OK) return rc;
    if (!box || (n && !samples) || (((uintptr_t)samples & 15u) != 0)) return fail(ctx, YAR_ERR_INVALID, "guide step");
    float* scal = (float*)ctx->guide.scalars.ptr;
    const float h[2] = {0.f, weight_scale};
    cudaError_t e = cudaMemcpyAsync(scal, h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = guide_train(ctx, (const float4*)samples, n, nullptr, 1, 0, box, scal + 1, lr, grad, ctx->stream);
    return guide_finish(ctx, e, "guide training step", loss);
}

} // namespace

extern "C" int yar_guide_set_params(yar_gpu_ctx* ctx, const float* params) {
    int rc = guide_call_prologue(ctx);
    if (rc != YAR_OK) return rc;
    if (!params) return fail(ctx, YAR_ERR_INVALID, "null parameters");
    return guide_set_params(ctx, params);
}

extern "C" int yar_guide_get_params(yar_gpu_ctx* ctx, float* params) {
    int rc = guide_call_prologue(ctx);
    if (rc != YAR_OK) return rc;
    if (!params) return fail(ctx, YAR_ERR_INVALID, "null parameters");
    cudaError_t e = cudaMemcpyAsync(params, ctx->guide.params.ptr, kGuideParams * sizeof(float),
                                    cudaMemcpyDeviceToHost, ctx->stream);
    return guide_finish(ctx, e, "guide parameters", nullptr);
}

extern "C" int yar_gpu_wait_selftest(yar_gpu_ctx* ctx, uint32_t limit) {
    if (!ctx) return YAR_ERR_INVALID;
    if (limit == 0 || limit > (1u << 24)) return fail(ctx, YAR_ERR_INVALID, "wait self-test: limit in [1, 2^24]");
    cudaSetDevice(ctx->device);
    wait_selftest_kernel<<<1, 32, 0, ctx->stream>>>(limit, ctx->d_error);
    return guide_finish(ctx, cudaGetLastError(), "wait self-test", nullptr);
}

extern "C" int yar_guide_infer(yar_gpu_ctx* ctx, const float* queries, uint32_t n, const float* box, float* lobes) {
    int rc = guide_call_prologue(ctx);
    if (rc != YAR_OK) return rc;
    if (!box || (n && (!queries || !lobes)) || (((uintptr_t)queries & 15u) != 0) || (((uintptr_t)lobes & 15u) != 0))
        return fail(ctx, YAR_ERR_INVALID, "guide inference");
    cudaError_t e = guide_infer(ctx, (const float4*)queries, n, nullptr, box, lobes, ctx->stream);
    return guide_finish(ctx, e, "guide inference", nullptr);
}

extern "C" int yar_guide_gradient(yar_gpu_ctx* ctx, const float* samples, uint32_t n, const float* box,
                                  float weight_scale, float* grad, float* loss) {
    if (ctx && !grad) return fail(ctx, YAR_ERR_INVALID, "null gradient buffer");
    return guide_step(ctx, samples, n, box, weight_scale, 0.f, grad, loss);
}

extern "C" int yar_guide_train_step(yar_gpu_ctx* ctx, const float* samples, uint32_t n, const float* box,
                                    float weight_scale, float learning_rate, float* loss) {
    return guide_step(ctx, samples, n, box, weight_scale, learning_rate, nullptr, loss);
}

} // namespace yar
