// guided.cu - yar_gpu_guided_render: the wavefront path tracer rendered as
// independent one-sample passes, optionally with the learned directional
// proposal (guide_mlp.cu) drawing path continuations.  No reference
// counterpart; its plain mode (guide fraction 0) is the reference's path
// tracer with per-pass pixel streams, and is the baseline the guided mode is
// measured against.
//
// Per pass: sample tables and camera rays for every pixel (one path each),
// then per bounce extend -> [network input per hit -> tensor-core inference
// of the hit's lobe mixture] -> shade (continuation from the mixture with
// probability alpha, one-sample MIS with the BSDF) -> shadow -> probe ->
// connect; finally each path's radiance (clamped and scaled as the film does)
// is added to a per-pixel FP64 sum.  In the training passes every continued
// vertex records (position, normal, wo, direction, f cos / p, throughput,
// radiance so far); after the pass the incident radiance along each recorded
// direction is recovered from the path's final radiance, and the records
// with a non-zero training weight feed the network's Adam steps.
#include "wavefront.cuh"

namespace yar {

namespace {

// Network input of each extend-queue hit: world position o + t d, the
// geometric normal facing the incoming ray, wo = -d.  Misses and light
// hits get zeros (they are not shaded).
__global__ void __launch_bounds__(kBlock)
guide_query_kernel(Scene_Dev S, const float4* __restrict__ rays, const float4* __restrict__ hit4,
                   const uint2* __restrict__ hit2, uint32_t count, float4* __restrict__ queries) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0;
        const uint2 h2 = hit2[i];
        if (h2.y != 0xffffffffu) {
            const float4 ra = rays[2 * (size_t)i], rb = rays[2 * (size_t)i + 1];
            const float t = hit4[i].x;
            const V3 d = v3(rb.x, rb.y, rb.z);
            const V3 pos = v3(ra.x + t * d.x, ra.y + t * d.y, ra.z + t * d.z);
            const float4* rrec = S.obj_render + 7 * (size_t)h2.y;
            const float4 n0 = __ldg(rrec + 3), n1 = __ldg(rrec + 4), n2 = __ldg(rrec + 5);
            const uint32_t tri_offset = __float_as_uint(__ldg(S.ds.objects + 6 * (size_t)h2.y + 4).w);
            const size_t g = (size_t)tri_offset + h2.x;
            const float4 a = __ldg(S.ds.tris + 3 * g), b = __ldg(S.ds.tris + 3 * g + 1), c = __ldg(S.ds.tris + 3 * g + 2);
            V3 ng = xform_vector(n0, n1, n2, cross(v3(b.x - a.x, b.y - a.y, b.z - a.z), v3(c.x - a.x, c.y - a.y, c.z - a.z)));
            const float nl = len(ng);
            ng = nl > 0.f ? divs(ng, nl) : v3(0.f, 0.f, 1.f);
            const float dl = len(d);
            const V3 wo = dl > 0.f ? divs(-d, dl) : v3(0.f, 0.f, 1.f);
            if (dot(ng, wo) < 0.f) ng = -ng;
            q0 = make_float4(pos.x, pos.y, pos.z, ng.x);
            q1 = make_float4(ng.y, ng.z, wo.x, wo.y);
            q2 = make_float4(wo.z, 0.f, 0.f, 0.f);
        }
        queries[3 * (size_t)i] = q0;
        queries[3 * (size_t)i + 1] = q1;
        queries[3 * (size_t)i + 2] = q2;
    }
}

// Adds each path's radiance, clamped and scaled as samples_kernel does for
// the film (reference_renderer.cpp:388-393), to its pixel's FP64 sum.  One
// path per pixel: slot = pixel.
__global__ void __launch_bounds__(kBlock)
accumulate_kernel(Render_Params p, uint32_t paths, const float4* __restrict__ L, double* __restrict__ sum) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < paths; i += gridDim.x * blockDim.x) {
        float4 r = L[i];
        const float mc = max_std(r.x, max_std(r.y, r.z));
        if (mc > p.max_component) {
            const float s = p.max_component / mc;
            r.x *= s;
            r.y *= s;
            r.z *= s;
        }
        if (p.film_scale != 1.f) {
            r.x *= p.film_scale;
            r.y *= p.film_scale;
            r.z *= p.film_scale;
        }
        sum[3 * (size_t)i] += (double)r.x;
        sum[3 * (size_t)i + 1] += (double)r.y;
        sum[3 * (size_t)i + 2] += (double)r.z;
    }
}

// Training samples from the pass's records: the radiance arriving along the
// recorded direction is (L_final - L_after_vertex) / throughput_after per
// channel; the sample weight is its luminance times f cos / p.  Records with
// weight 0 carry no gradient and are dropped; the kept weights are summed
// into *weight_sum.
__global__ void __launch_bounds__(kBlock)
finalize_kernel(const float4* __restrict__ records, const uint32_t* __restrict__ record_count, uint32_t capacity,
                const float4* __restrict__ L, float4* __restrict__ samples, uint32_t* __restrict__ sample_count,
                float* __restrict__ weight_sum) {
    const uint32_t n = min(*record_count, capacity);
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const float4* rec = records + (size_t)r * kGuideRecordF4;
        const float4 r3 = rec[3], beta = rec[4], la = rec[5];
        const float4 lf = L[__float_as_uint(r3.y)];
        const float li_r = beta.x > 0.f ? (lf.x - la.x) / beta.x : 0.f;
        const float li_g = beta.y > 0.f ? (lf.y - la.y) / beta.y : 0.f;
        const float li_b = beta.z > 0.f ? (lf.z - la.z) / beta.z : 0.f;
        const float lum = fmaxf(0.f, 0.2126729f * li_r + 0.7151522f * li_g + 0.0721750f * li_b);
        const float w = lum * r3.x;
        const bool keep = w > 0.f && isfinite(w);
        const uint32_t s = warp_append(sample_count, keep);
        if (keep) {
            float4* o = samples + 4 * (size_t)s;
            o[0] = rec[0];
            o[1] = rec[1];
            o[2] = rec[2];
            o[3] = make_float4(w, 0.f, 0.f, 0.f);
            atomicAdd(weight_sum, w);
        }
    }
}

template <class T>
T* dp(Device_Buffer& b) {
    return reinterpret_cast<T*>(b.ptr);
}

// The guide hook of the stratified render: network inputs of the extend
// queue's hits, then tensor-core inference of their lobe mixtures.
struct Guide_Hook_State {
    yar_gpu_ctx* ctx;
    Scene_Dev S;
    float4* queries;
    float* lobes;
    float box[6];
};

cudaError_t guided_before_shade(void* user, const float4* rays, const float4* hit4, const uint2* hit2, uint32_t count,
                                cudaStream_t st) {
    Guide_Hook_State* h = static_cast<Guide_Hook_State*>(user);
    guide_query_kernel<<<grid_for(count), kBlock, 0, st>>>(h->S, rays, hit4, hit2, count, h->queries);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return guide_infer(h->ctx, h->queries, count, nullptr, h->box, h->lobes, st);
}

constexpr uint64_t kGuidedChunkPaths = 8u << 20;  // stratified phase: paths in flight (lobes 160 B each)

} // namespace

int guided_render(yar_gpu_ctx* ctx, const yar_guided_params* gp, double* sum_out, float* rgb_out,
                  yar_guided_stats* stats) {
    if (!gp || (gp->passes == 0 && gp->samples_per_pixel == 0))
        return fail(ctx, YAR_ERR_INVALID, "guided render: no passes");
    // stratified: the training passes, then one render with the pixel sampler
    // at nx x ny strata, nx = strata_x or ceil(sqrt(n)), ny = ceil(n / nx)
    int spp_side = gp->samples_per_pixel ? (int)std::ceil(std::sqrt((double)gp->samples_per_pixel)) : 0;
    if (spp_side && gp->strata_x) {
        if (gp->strata_x > gp->samples_per_pixel) return fail(ctx, YAR_ERR_INVALID, "guided render: strata_x > spp");
        spp_side = (int)gp->strata_x;
    }
    if (spp_side > 256) return fail(ctx, YAR_ERR_INVALID, "guided render: at most 65536 samples per pixel");
    const int spp_rows = spp_side ? (int)((gp->samples_per_pixel + (uint32_t)spp_side - 1) / (uint32_t)spp_side) : 0;
    if (spp_rows > 256 || spp_side > 4 * spp_rows || 4 * spp_side < spp_rows)
        return fail(ctx, YAR_ERR_INVALID, "guided render: strata columns and rows at most 256 and 4:1");
    const uint32_t pass_count = spp_side ? (gp->guide_fraction > 0.f ? gp->train_passes : 0u) : gp->passes;
    if (!(gp->guide_fraction >= 0.f && gp->guide_fraction < 1.f))
        return fail(ctx, YAR_ERR_INVALID, "guide fraction must be in [0, 1)");
    if (ctx->render.config.rendering_algorithm == 0)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "the guided render runs the path tracer only (rendering_algorithm 1)");
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    if (!spp_side && (p.filter_radius > 0.5f || p.filter_type != 0))
        return fail(ctx, YAR_ERR_UNSUPPORTED, "guided passes: box filter of radius <= 0.5 only (one pixel per sample)");
    p.nx = p.ny = p.spp = 1;
    const uint32_t paths = (uint32_t)((uint64_t)p.sw * p.sh);
    if ((uint64_t)p.sw * p.sh > kChunkSampleBudget) return fail(ctx, YAR_ERR_CAPACITY, "guided render: image too large");
    const bool guided = gp->guide_fraction > 0.f;
    const uint32_t rec_per_path = (uint32_t)std::max(1, std::min(p.max_bounces, 64));
    const uint64_t rec_cap64 = guided ? (uint64_t)paths * rec_per_path : 0;
    if (rec_cap64 > 0xffffffffull) return fail(ctx, YAR_ERR_CAPACITY, "guided render: too many training records");
    const uint32_t rec_cap = (uint32_t)rec_cap64;
    cudaSetDevice(ctx->device);
    int rc = YAR_OK;
    if (guided) {
        if ((rc = guide_ensure(ctx)) != YAR_OK) return rc;
        if (!gp->keep_guide && (rc = guide_reset(ctx, 0x5eed0000ull + gp->stream_offset)) != YAR_OK) return rc;
    }

    std::vector<Device_Buffer>& B = ctx->guided_scratch;
    if (B.size() != 40) {
        for (Device_Buffer& b : B) device_free(b);
        B.assign(40, Device_Buffer{});
    }
    auto alloc = [&](int i, size_t bytes) {  // kept from an earlier call when large enough
        if (rc == YAR_OK && bytes && !(B[i].ptr && B[i].bytes >= bytes)) rc = device_alloc(ctx, B[i], bytes);
    };
    const size_t cap = paths;
    alloc(1, cap * sizeof(float2));                        // image-plane samples
    alloc(2, cap * std::max(1, p.n1d) * sizeof(float));    // s1d
    alloc(3, cap * std::max(1, p.n2d) * sizeof(float2));   // s2d
    alloc(4, cap * sizeof(float4));                        // coeff
    alloc(5, cap * sizeof(float4));                        // L
    alloc(6, cap * sizeof(uint32_t));                      // info
    alloc(7, cap * sizeof(uint4));                         // rng
    alloc(8, cap * sizeof(float4));                        // pend_light
    alloc(9, cap * sizeof(float4));                        // pend_probe0
    alloc(10, cap * sizeof(float4));                       // pend_probe1
    alloc(11, cap * sizeof(float4));                       // pend_probe2
    alloc(12, cap * sizeof(float4));                       // pend_coeff
    alloc(13, cap * sizeof(uint8_t));                      // occluded
    alloc(14, cap * sizeof(float4));                       // probe_hit4
    alloc(15, cap * sizeof(uint2));                        // probe_hit2
    alloc(16, cap * 2 * sizeof(float4));                   // ext rays 0
    alloc(17, cap * 2 * sizeof(float4));                   // ext rays 1
    alloc(18, cap * sizeof(uint32_t));                     // ext slot 0
    alloc(19, cap * sizeof(uint32_t));                     // ext slot 1
    alloc(20, cap * sizeof(float4));                       // ext hit4
    alloc(21, cap * sizeof(uint2));                        // ext hit2
    alloc(22, cap * 2 * sizeof(float4));                   // shadow rays
    alloc(23, cap * sizeof(uint32_t));                     // shadow slots
    alloc(24, cap * 2 * sizeof(float4));                   // probe rays
    alloc(25, cap * sizeof(uint32_t));                     // probe slots
    alloc(26, 16 * sizeof(uint32_t));                      // counters; [8] records, [9] samples, [10] weight sum
    alloc(27, cap * 3 * sizeof(double));                   // radiance sums
    if (guided) {
        alloc(30, cap * 3 * sizeof(float4));               // network inputs
        alloc(31, cap * kGuideLobeFloats * sizeof(float));  // lobes
        alloc(32, cap * sizeof(uint32_t));                 // record index per path
        alloc(33, (size_t)rec_cap * kGuideRecordF4 * sizeof(float4));
        alloc(34, (size_t)rec_cap * 4 * sizeof(float4));   // training samples
        alloc(35, 4 * sizeof(float));                      // weight scale
    }
    if (p.spec_diffs) alloc(36, cap * 3 * sizeof(float4));  // delta rays' specular differential rays
    if (rc != YAR_OK) return rc;

    Path_State ps{dp<float4>(B[4]), dp<float4>(B[5]), dp<uint32_t>(B[6]), dp<uint4>(B[7]),
                  dp<float4>(B[8]), dp<float4>(B[9]), dp<float4>(B[10]), dp<float4>(B[11]),
                  dp<float4>(B[12]), dp<uint8_t>(B[13]), dp<float4>(B[14]), dp<uint2>(B[15]),
                  guided ? dp<uint32_t>(B[32]) : nullptr};
    ps.image_samples = dp<float2>(B[1]);  // textured hits' camera differentials (one chunk per pass)
    ps.chunk_first = 0;
    ps.diff = dp<float4>(B[36]);
    Queues q{};
    q.ext_rays[0] = dp<float4>(B[16]);
    q.ext_rays[1] = dp<float4>(B[17]);
    q.ext_slot[0] = dp<uint32_t>(B[18]);
    q.ext_slot[1] = dp<uint32_t>(B[19]);
    q.ext_hit4 = dp<float4>(B[20]);
    q.ext_hit2 = dp<uint2>(B[21]);
    q.shd_rays = dp<float4>(B[22]);
    q.shd_slot = dp<uint32_t>(B[23]);
    q.prb_rays = dp<float4>(B[24]);
    q.prb_slot = dp<uint32_t>(B[25]);
    q.counters = dp<uint32_t>(B[26]);
    Scene_Dev S = scene_dev(ctx->ds, ctx->render);
    const float box[6] = {ctx->ds.scene_bounds[0], ctx->ds.scene_bounds[1], ctx->ds.scene_bounds[2],
                          ctx->ds.scene_bounds[3], ctx->ds.scene_bounds[4], ctx->ds.scene_bounds[5]};

    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemsetAsync(q.counters, 0, 16 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B[27].ptr, 0, cap * 3 * sizeof(double), st);
    uint64_t rays = 0, train_samples = 0;
    double train_seconds = 0.0;
    float last_loss = 0.f;
    uint32_t done = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t pass = 0; pass < pass_count && e == cudaSuccess; pass++) {
        p.stream_hi = (gp->stream_offset << 20) + pass + 1u;
        const bool training = guided && pass < gp->train_passes;  // (every pass, stratified)
        Guide_Shade g;
        if (guided) {
            g.queries = dp<float4>(B[30]);
            g.alpha = (pass > 0 || gp->keep_guide) ? gp->guide_fraction : 0.f;
            g.lobes = g.alpha > 0.f ? dp<float>(B[31]) : nullptr;
            if (training) {
                g.records = dp<float4>(B[33]);
                g.record_count = q.counters + 8;
                g.record_capacity = rec_cap;
                e = cudaMemsetAsync(q.counters + 8, 0, 3 * sizeof(uint32_t), st);
            }
        }
        if (e == cudaSuccess) e = launch_generate(p, 0, paths, dp<float>(B[2]), dp<float>(B[3]), dp<float2>(B[1]), ps, q, st);
        int cur = 0;
        uint32_t count = paths;
        for (int bounce = 0; count > 0 && bounce <= p.max_bounces + 1 && e == cudaSuccess; bounce++) {
            e = trace_extend(ctx, q, cur, count, bounce, st);
            if (e != cudaSuccess) break;
            if (g.queries && (g.lobes || g.records)) {
                guide_query_kernel<<<grid_for(count), kBlock, 0, st>>>(S, q.ext_rays[cur], q.ext_hit4, q.ext_hit2, count,
                                                                     dp<float4>(B[30]));
                if (g.lobes) e = guide_infer(ctx, dp<float4>(B[30]), count, nullptr, box, dp<float>(B[31]), st);
                if (e != cudaSuccess) break;
            }
            cudaMemsetAsync(q.counters, 0, 3 * sizeof(uint32_t), st);
            launch_shade<true>(p, grid_for(count), st, S, cur, count, dp<float>(B[2]), dp<float2>(B[3]), ps, q, g);
            e = trace_light_queues(ctx, q, ps, count, bounce, st);
            if (e != cudaSuccess) break;
            connect_kernel<<<grid_for(count), kBlock, 0, st>>>(p, S, q.ext_slot[cur], count, ps, g.records);
            uint32_t h[4];
            e = cudaMemcpyAsync(h, q.counters, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (h[3]) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
            rays += count + h[1] + h[2];
            count = h[0];
            cur ^= 1;
        }
        if (e != cudaSuccess) break;
        accumulate_kernel<<<grid_for(paths), kBlock, 0, st>>>(p, paths, ps.L, dp<double>(B[27]));
        if (training) {
            const auto tt = std::chrono::steady_clock::now();
            finalize_kernel<<<grid_for(rec_cap), kBlock, 0, st>>>(dp<float4>(B[33]), q.counters + 8, rec_cap, ps.L,
                                                                 dp<float4>(B[34]), q.counters + 9,
                                                                 reinterpret_cast<float*>(q.counters + 10));
            uint32_t h[3];
            e = cudaMemcpyAsync(h, q.counters + 8, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            const uint32_t n = h[1];
            float wsum;
            std::memcpy(&wsum, &h[2], sizeof(float));
            const uint32_t steps = std::max(1u, std::min(gp->train_steps ? gp->train_steps : 1u, n));
            if (n > 0 && wsum > 0.f) {
                const uint32_t per_step = (n + steps - 1) / steps;
                // mean weight 1 over the pass, loss averaged over a minibatch
                ctx->guided_weight_scale = (float)n / (wsum * (float)per_step);
                float* scal = dp<float>(B[35]);
                e = cudaMemcpyAsync(scal, &ctx->guided_weight_scale, sizeof(float), cudaMemcpyHostToDevice, st);
                for (uint32_t s = 0; s < steps && e == cudaSuccess; s++) {
                    const uint32_t rows = (n - s + steps - 1) / steps;
                    if (s + 1 == steps) e = cudaMemsetAsync(ctx->guide.scalars.ptr, 0, sizeof(float), st);
                    if (e == cudaSuccess)
                        e = guide_train(ctx, dp<float4>(B[34]), rows, nullptr, steps, s, box, scal,
                                        gp->learning_rate, nullptr, st);
                }
                float l = 0.f;
                if (e == cudaSuccess) e = cudaMemcpyAsync(&l, ctx->guide.scalars.ptr, sizeof(float), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                last_loss = l;
                train_samples += n;
            }
            train_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - tt).count();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        done = pass + 1;
        const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (!spp_side && gp->time_budget > 0.f && elapsed >= gp->time_budget) break;
    }
    if (spp_side && e == cudaSuccess) {
        // the image: the scene's pixel sampler at spp_side x spp_rows samples per pixel,
        // continuations from the trained proposal
        Device_Buffer& qbuf = ctx->guide_queries;
        Device_Buffer& lbuf = ctx->guide_lobes;
        Guide_Hook_State hs{ctx, S, nullptr, nullptr, {box[0], box[1], box[2], box[3], box[4], box[5]}};
        Guide_Render_Hook hook;
        hook.alpha = guided ? gp->guide_fraction : 0.f;
        hook.max_bounce = (int)std::min<uint32_t>(gp->guide_bounces, 1u << 20);
        hook.chunk_paths = std::max<uint64_t>(kGuidedChunkPaths, (uint64_t)spp_side * spp_rows);
        if (guided) {
            const size_t qbytes = hook.chunk_paths * 3 * sizeof(float4);
            const size_t lbytes = hook.chunk_paths * kGuideLobeFloats * sizeof(float);
            if (!(qbuf.ptr && qbuf.bytes >= qbytes)) rc = device_alloc(ctx, qbuf, qbytes);
            if (rc == YAR_OK && !(lbuf.ptr && lbuf.bytes >= lbytes)) rc = device_alloc(ctx, lbuf, lbytes);
            if (rc != YAR_OK) return rc;
            hs.queries = dp<float4>(qbuf);
            hs.lobes = dp<float>(lbuf);
            hook.queries = hs.queries;
            hook.lobes = hs.lobes;
            hook.before_shade = guided_before_shade;
            hook.user = &hs;
        }
        std::vector<float> img((size_t)p.rw * p.rh * 3);
        yar_render_stats rs{};
        if (!guided) hook.chunk_paths = std::max<uint64_t>(kChunkSampleBudget, (uint64_t)spp_side * spp_rows);
        rc = render_guided_stratified(ctx, spp_side, spp_rows, (gp->stream_offset << 20) | 0xfffffu, hook, img.data(),
                                      &rs);
        if (rc != YAR_OK) return rc;
        int h_err = 0;
        e = cudaMemcpy(&h_err, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "guided render");
        if (h_err) {
            cudaMemset(ctx->d_error, 0, sizeof(int));
            return fail(ctx, YAR_ERR_TIMEOUT, "tensor-core wait gave up");
        }
        const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const double n = (double)spp_side * spp_rows;
        for (size_t k = 0; k < img.size(); k++) {
            if (rgb_out) rgb_out[k] = img[k];
            if (sum_out) sum_out[k] = (double)img[k] * n;
        }
        if (stats) {
            stats->passes = done;
            stats->seconds = (float)seconds;
            stats->train_seconds = (float)train_seconds;
            stats->rays = rays + rs.rays_closest + rs.rays_any;
            stats->train_samples = train_samples;
            stats->loss = last_loss;
        }
        return YAR_OK;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h_err, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "guided render");
    if (h_err) {
        cudaMemset(ctx->d_error, 0, sizeof(int));
        return fail(ctx, YAR_ERR_TIMEOUT, "tensor-core wait gave up");
    }
    // the sample region equals the render region for a box filter of radius <= 0.5
    if (sum_out || rgb_out) {
        std::vector<double> sums(cap * 3);
        e = cudaMemcpy(sums.data(), B[27].ptr, cap * 3 * sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "guided render");
        for (int y = 0; y < p.rh; y++)
            for (int x = 0; x < p.rw; x++) {
                const size_t src = 3 * ((size_t)(y + p.ry0 - p.sy0) * p.sw + (x + p.rx0 - p.sx0));
                const size_t dst = 3 * ((size_t)y * p.rw + x);
                for (int c = 0; c < 3; c++) {
                    if (sum_out) sum_out[dst + c] = sums[src + c];
                    if (rgb_out) rgb_out[dst + c] = (float)(sums[src + c] / (double)done);
                }
            }
    }
    if (stats) {
        stats->passes = done;
        stats->seconds = (float)seconds;
        stats->train_seconds = (float)train_seconds;
        stats->rays = rays;
        stats->train_samples = train_samples;
        stats->loss = last_loss;
    }
    return YAR_OK;
}

extern "C" int yar_gpu_guided_render(yar_gpu_ctx* ctx, const yar_guided_params* params, double* radiance_sum,
                                     float* rgb_out, yar_guided_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    return guided_render(ctx, params, radiance_sum, rgb_out, stats);
}

} // namespace yar
