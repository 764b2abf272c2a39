// batch.cu - yar_gpu_render_batch: many scenes of uneven triangle count,
// resolution and sample count rendered by one CUDA graph launch.
//
// No reference counterpart (the reference renders one scene per process).
// Each scene is uploaded into its own internal context; each renders exactly
// as yar_gpu_render would (same kernels, same per-path results), but without
// host round trips: the bounce loop is device-driven (a one-thread kernel
// turns the shade kernel's append counter into the next extend count; every
// kernel reads its queue length from device memory and exits early on an
// empty queue), so a scene's whole chunk/bounce sequence can be captured.
// The graph forks into `branches` streams; scenes are assigned to branches
// longest-first (balancing their loads) and each branch runs its scenes
// shortest-first, so small scenes overlap with each other and with the tails
// of large ones and finish early.  A one-thread kernel stamps the GPU clock when each scene's
// film is resolved: per-scene completion times come from the device.
//
// Autotuner: before capture, (1) each scene's traversal kernel is chosen by
// timing the traversal kernels on 2^16 random rays in its box (tune_cast), and
// (2) the branch count and the chunk capacity (paths in flight per branch)
// are chosen by capturing and timing the whole batch at one sample per pixel
// for each candidate; the full-sample graph is then captured with the winner.
#include "wavefront.cuh"

#include <random>

namespace yar {

namespace {

__global__ void stamp_kernel(unsigned long long* out) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}

__global__ void random_rays_kernel(float4* rays, uint32_t n, float3 lo, float3 ext, uint64_t seed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Pcg r = pcg_seed(seed, i);
    const float3 o = make_float3(lo.x + ext.x * pcg_float(r), lo.y + ext.y * pcg_float(r), lo.z + ext.z * pcg_float(r));
    const float z = 1.f - 2.f * pcg_float(r);
    const float s = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincospif(2.f * pcg_float(r), &sp, &cp);
    rays[2 * (size_t)i] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
    rays[2 * (size_t)i + 1] = make_float4(s * cp, s * sp, z, 0.f);
}

template <class T>
T* dp(Device_Buffer& b) {
    return reinterpret_cast<T*>(b.ptr);
}

struct Batch_Scene {
    yar_gpu_ctx* sub = nullptr;
    Render_Params p{};
    uint64_t pixels = 0, samples = 0;
    Device_Buffer radiance, image_samples, pixel_var, tile_var, variance, rgb;
    int kernel[2] = {kCastPersistent64, kCastPersistent64};
    int branch = 0;
};

struct Branch {
    cudaStream_t stream = nullptr;
    uint64_t cap = 0;  // paths per chunk
    int n1d = 1, n2d = 1;
    bool diffs = false;  // a scene of the branch carries specular differential rays
    std::vector<Device_Buffer> B;
    Path_State ps{};
    Queues q{};
};

struct Batch {
    yar_gpu_ctx* ctx;
    std::vector<Batch_Scene> scenes;
    std::vector<Branch> branches;
    Device_Buffer stamps;  // [0] start, [1 + i] scene i done
    Device_Buffer rays;    // per branch: closest, any
    ~Batch() {
        for (Batch_Scene& s : scenes) {
            for (Device_Buffer* b : {&s.radiance, &s.image_samples, &s.pixel_var, &s.tile_var, &s.variance, &s.rgb})
                device_free(*b);
            if (s.sub) yar_gpu_destroy(s.sub);
        }
        for (Branch& b : branches) {
            for (Device_Buffer& x : b.B) device_free(x);
            if (b.stream) cudaStreamDestroy(b.stream);
        }
        device_free(stamps);
        device_free(rays);
    }
};

constexpr uint32_t kFixedGrid = 152 * 16;  // shade/connect grid when queue lengths live on the device

int alloc_branches(Batch& bt, int nb, uint64_t chunk_cap, bool one_spp) {
    yar_gpu_ctx* ctx = bt.ctx;
    for (Branch& b : bt.branches) {
        for (Device_Buffer& x : b.B) device_free(x);
        if (b.stream) cudaStreamDestroy(b.stream);
    }
    bt.branches.assign(nb, Branch{});
    std::vector<uint64_t> load(nb, 0);
    std::vector<int> order(bt.scenes.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    auto spp_of = [&](const Batch_Scene& s) { return one_spp ? 1 : s.p.spp; };
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return bt.scenes[a].pixels * spp_of(bt.scenes[a]) > bt.scenes[b].pixels * spp_of(bt.scenes[b]);
    });
    for (int i : order) {  // longest first onto the least loaded branch
        const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        Batch_Scene& s = bt.scenes[i];
        s.branch = b;
        load[b] += s.pixels * spp_of(s);
        Branch& br = bt.branches[b];
        const uint64_t spp = spp_of(s);
        const uint64_t cp = std::max<uint64_t>(1, std::min<uint64_t>(s.pixels, chunk_cap / spp)) * spp;
        br.cap = std::max(br.cap, cp);
        br.n1d = std::max(br.n1d, s.p.n1d);
        br.n2d = std::max(br.n2d, s.p.n2d);
        br.diffs = br.diffs || s.p.spec_diffs;
    }
    int rc = YAR_OK;
    for (Branch& br : bt.branches) {
        cudaError_t e = cudaStreamCreateWithFlags(&br.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "batch streams");
        if (br.cap == 0) continue;
        br.B.assign(33, Device_Buffer{});
        const size_t cap = br.cap;
        const size_t sizes[32] = {0, 0, cap * br.n1d * sizeof(float), cap * br.n2d * sizeof(float2),
                                  cap * 16, cap * 16, cap * 4, cap * 16, cap * 16, cap * 16, cap * 16, cap * 16,
                                  cap * 16, cap, cap * 16, cap * 8, cap * 32, cap * 32, cap * 4, cap * 4, cap * 16,
                                  cap * 8, cap * 32, cap * 4, cap * 32, cap * 4, 16 * sizeof(uint32_t),
                                  cap, cap * 4, 2 * kShadeClasses * sizeof(uint32_t),  // shading order
                                  cap * 2, kRayBins * sizeof(uint32_t)};              // extend-queue sort
        for (int i = 2; i < 32 && rc == YAR_OK; i++) rc = device_alloc(ctx, br.B[i], sizes[i]);
        if (br.diffs && rc == YAR_OK) rc = device_alloc(ctx, br.B[32], cap * 3 * sizeof(float4));
        if (rc != YAR_OK) return rc;
        std::vector<Device_Buffer>& B = br.B;
        br.ps = Path_State{dp<float4>(B[4]), dp<float4>(B[5]), dp<uint32_t>(B[6]), dp<uint4>(B[7]),
                           dp<float4>(B[8]), dp<float4>(B[9]), dp<float4>(B[10]), dp<float4>(B[11]),
                           dp<float4>(B[12]), dp<uint8_t>(B[13]), dp<float4>(B[14]), dp<uint2>(B[15]), nullptr};
        br.ps.diff = dp<float4>(B[32]);
        br.q = Queues{};
        br.q.ext_rays[0] = dp<float4>(B[16]);
        br.q.ext_rays[1] = dp<float4>(B[17]);
        br.q.ext_slot[0] = dp<uint32_t>(B[18]);
        br.q.ext_slot[1] = dp<uint32_t>(B[19]);
        br.q.ext_hit4 = dp<float4>(B[20]);
        br.q.ext_hit2 = dp<uint2>(B[21]);
        br.q.shd_rays = dp<float4>(B[22]);
        br.q.shd_slot = dp<uint32_t>(B[23]);
        br.q.prb_rays = dp<float4>(B[24]);
        br.q.prb_slot = dp<uint32_t>(B[25]);
        br.q.counters = dp<uint32_t>(B[26]);
        br.q.ext_count = br.q.counters + 7;
    }
    return rc;
}

// The kernels of one scene on its branch's stream: chunks of device-driven
// bounces, then the film.  Everything is capturable (no host reads).
cudaError_t enqueue_scene(Batch& bt, int si, bool one_spp, unsigned long long* stamp, unsigned long long* rays) {
    Batch_Scene& sc = bt.scenes[si];
    Branch& br = bt.branches[sc.branch];
    cudaStream_t st = br.stream;
    Render_Params p = sc.p;
    if (one_spp) p.nx = p.ny = p.spp = 1;
    yar_gpu_ctx* sub = sc.sub;
    Scene_Dev S = scene_dev(sub->ds, sub->render);
    const uint64_t chunk_pixels = std::max<uint64_t>(1, std::min<uint64_t>(sc.pixels, br.cap / p.spp));
    Queues q = br.q;
    Path_State ps = br.ps;
    uint32_t* ctr = q.counters;
    // the shading order of each extend queue when the scene mixes BSDF classes
    // (as render_run_params decides it)
    uint32_t seen = 0;
    const std::vector<int32_t>& oi = sub->render.host_object_info;
    for (size_t o = 0; o + 3 < oi.size(); o += 4) {
        if ((uint32_t)oi[o + 2] != YAR_LIGHT_NULL || (uint32_t)oi[o] == YAR_MATERIAL_NULL) continue;
        const uint32_t m = (uint32_t)oi[o];
        seen |= m == YAR_MATERIAL_DIFFUSE ? 1u : (m == YAR_MATERIAL_METAL ? 2u : 4u);
    }
    const bool mixed = (seen & (seen - 1)) != 0;
    // the extend queues after the camera bounce sorted by direction octant and
    // origin cell, in scenes up to 1M triangles (as render_run_params does)
    const bool sort_rays = sub->tris.bytes / (3 * sizeof(float4)) <= (1u << 20);
    Ray_Grid grid_box;
    for (int k = 0; k < 3; k++) {
        const float lo = sub->ds.scene_bounds[k], ext = sub->ds.scene_bounds[3 + k] - lo;
        grid_box.lo[k] = lo;
        grid_box.scale[k] = ext > 0.f ? 8.f / ext : 0.f;
    }
    Queues qs = q;  // q with the order, for the shade kernel
    qs.order = mixed ? dp<uint32_t>(br.B[28]) : nullptr;
    ps.image_samples = dp<float2>(sc.image_samples);  // textured hits' camera differentials
    cudaError_t e = cudaSuccess;
    for (uint64_t first = 0; first < sc.pixels && e == cudaSuccess; first += chunk_pixels) {
        const uint32_t cp = (uint32_t)std::min<uint64_t>(chunk_pixels, sc.pixels - first);
        const uint32_t paths = cp * (uint32_t)p.spp;
        ps.chunk_first = (uint32_t)first;
        e = cudaMemsetAsync(ctr, 0, 8 * sizeof(uint32_t), st);
        if (e == cudaSuccess)
            e = launch_generate(p, (uint32_t)first, cp, dp<float>(br.B[2]), dp<float>(br.B[3]),
                                dp<float2>(sc.image_samples), ps, q, st);
        int cur = 0;
        for (int bounce = 0; bounce <= p.max_bounces + 1 && e == cudaSuccess; bounce++) {
            bounce_begin_kernel<<<1, 1, 0, st>>>(ctr, bounce == 0 ? paths : 0u, rays);
            if (sort_rays && bounce > 0) {
                uint16_t* keys = dp<uint16_t>(br.B[30]);
                uint32_t* hist = dp<uint32_t>(br.B[31]);
                cudaMemsetAsync(hist, 0, kRayBins * sizeof(uint32_t), st);
                ray_hist_kernel<<<152 * 2, 256, 0, st>>>(grid_box, q.ext_rays[cur], ctr + 7, 0u, keys, hist);
                ray_scan_kernel<<<1, 1024, 0, st>>>(hist);
                ray_scatter_kernel<<<kFixedGrid, kBlock, 0, st>>>(q.ext_rays[cur], q.ext_slot[cur], q.ext_rays[cur ^ 1],
                                                                  q.ext_slot[cur ^ 1], keys, hist, ctr + 7, 0u);
                cur ^= 1;
            }
            Cast_Args a;
            a.rays = q.ext_rays[cur];
            a.count = ctr + 7;
            a.n_max = paths;
            a.next_ray = ctr + 4;
            a.err = reinterpret_cast<int*>(ctr + 3);
            a.hit4 = q.ext_hit4;
            a.hit2 = q.ext_hit2;
            e = launch_extend(sub->ds, a, sc.kernel[0], st);
            if (e != cudaSuccess) break;
            if (mixed) {
                uint32_t* bins = dp<uint32_t>(br.B[29]);
                cudaMemsetAsync(bins, 0, 2 * kShadeClasses * sizeof(uint32_t), st);
                shade_bin_kernel<<<kFixedGrid, kBlock, 0, st>>>(S, q, paths, dp<uint8_t>(br.B[27]), bins);
                shade_order_kernel<<<kFixedGrid, kBlock, 0, st>>>(q, paths, dp<uint8_t>(br.B[27]), bins,
                                                                  dp<uint32_t>(br.B[28]));
            }
            launch_shade<false>(p, kFixedGrid, st, S, cur, paths, dp<float>(br.B[2]), dp<float2>(br.B[3]), ps, qs,
                                Guide_Shade{});
            Cast_Args sh;
            sh.rays = q.shd_rays;
            sh.count = ctr + 1;
            sh.n_max = paths;
            sh.perm = q.shd_slot;
            sh.next_ray = ctr + 5;
            sh.err = reinterpret_cast<int*>(ctr + 3);
            sh.occluded = ps.occluded;
            e = launch_shadow(sub->ds, sh, sc.kernel[1], st);
            if (e != cudaSuccess) break;
            Cast_Args pr;
            pr.rays = q.prb_rays;
            pr.count = ctr + 2;
            pr.n_max = paths;
            pr.perm = q.prb_slot;
            pr.next_ray = ctr + 6;
            pr.err = reinterpret_cast<int*>(ctr + 3);
            pr.hit4 = ps.probe_hit4;
            pr.hit2 = ps.probe_hit2;
            e = launch_extend(sub->ds, pr, sc.kernel[0], st);
            if (e != cudaSuccess) break;
            connect_kernel<<<kFixedGrid, kBlock, 0, st>>>(p, S, q.ext_slot[cur], paths, ps, nullptr, ctr + 7);
            cur ^= 1;
        }
        bounce_begin_kernel<<<1, 1, 0, st>>>(ctr, 0u, rays);  // counts of the last bounce
        finish_chunk_kernel<<<grid_for(paths), kBlock, 0, st>>>(paths, first * p.spp, ps, dp<float4>(sc.radiance));
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    samples_kernel<<<(uint32_t)((sc.pixels + kBlock - 1) / kBlock), kBlock, 0, st>>>(p, dp<float4>(sc.radiance),
                                                                                   dp<double>(sc.pixel_var));
    tile_variance_kernel<<<p.tiles_x * p.tiles_y, kTileVarThreads, 0, st>>>(p, dp<double>(sc.pixel_var),
                                                                            dp<double>(sc.tile_var));
    variance_total_kernel<<<1, 1, 0, st>>>(p, dp<double>(sc.tile_var), dp<double>(sc.variance));
    film_kernel<<<(uint32_t)(((uint64_t)p.rw * p.rh + kBlock - 1) / kBlock), kBlock, 0, st>>>(
        p, dp<float4>(sc.radiance), dp<float2>(sc.image_samples), dp<float>(sc.rgb));
    stamp_kernel<<<1, 1, 0, st>>>(stamp);
    return cudaGetLastError();
}

// Captures the batch into one graph (fork into the branch streams, join).
cudaError_t capture(Batch& bt, bool one_spp, cudaGraphExec_t* exec) {
    yar_gpu_ctx* ctx = bt.ctx;
    cudaStream_t main = ctx->stream;
    unsigned long long* stamps = dp<unsigned long long>(bt.stamps);
    unsigned long long* rays = dp<unsigned long long>(bt.rays);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(main, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return e;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join(bt.branches.size(), nullptr);
    e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemsetAsync(rays, 0, 2 * bt.branches.size() * sizeof(unsigned long long), main);
    if (e == cudaSuccess) stamp_kernel<<<1, 1, 0, main>>>(stamps);
    if (e == cudaSuccess) e = cudaEventRecord(fork, main);
    for (size_t b = 0; b < bt.branches.size() && e == cudaSuccess; b++)
        e = cudaStreamWaitEvent(bt.branches[b].stream, fork, 0);
    // scenes went longest-first onto the least-loaded branch; within a branch
    // they run shortest-first, which leaves the makespan and brings most
    // completions forward
    std::vector<int> run_order(bt.scenes.size());
    for (size_t i = 0; i < run_order.size(); i++) run_order[i] = (int)i;
    std::stable_sort(run_order.begin(), run_order.end(), [&](int a, int b) {
        return bt.scenes[a].pixels * bt.scenes[a].p.spp < bt.scenes[b].pixels * bt.scenes[b].p.spp;
    });
    for (size_t k = 0; k < run_order.size() && e == cudaSuccess; k++) {
        const int i = run_order[k];
        e = enqueue_scene(bt, i, one_spp, stamps + 1 + i, rays + 2 * bt.scenes[i].branch);
    }
    for (size_t b = 0; b < bt.branches.size() && e == cudaSuccess; b++) {
        e = cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(join[b], bt.branches[b].stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(main, join[b], 0);
    }
    const cudaError_t e_end = cudaStreamEndCapture(main, &graph);
    if (e == cudaSuccess) e = e_end;
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (fork) cudaEventDestroy(fork);
    for (cudaEvent_t ev : join)
        if (ev) cudaEventDestroy(ev);
    return e;
}

cudaError_t run_graph(Batch& bt, cudaGraphExec_t exec, double* gpu_seconds) {
    cudaError_t e = cudaGraphLaunch(exec, bt.ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(bt.ctx->stream);
    if (e != cudaSuccess) return e;
    std::vector<unsigned long long> st(1 + bt.scenes.size());
    e = cudaMemcpy(st.data(), bt.stamps.ptr, st.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    unsigned long long last = st[0];
    for (size_t i = 1; i < st.size(); i++) last = std::max(last, st[i]);
    *gpu_seconds = (double)(last - st[0]) * 1e-9;
    return cudaSuccess;
}

} // namespace

int render_batch(yar_gpu_ctx* ctx, const yar_flat_scene* const* scenes, uint32_t count, float* const* rgb_out,
                 yar_batch_scene_stats* scene_stats, yar_batch_stats* stats) {
    if (!scenes || count == 0 || !rgb_out) return fail(ctx, YAR_ERR_INVALID, "render batch: no scenes");
    cudaSetDevice(ctx->device);
    Batch bt;
    bt.ctx = ctx;
    bt.scenes.resize(count);
    const auto t0 = std::chrono::steady_clock::now();
    int rc = YAR_OK;
    // upload every scene into its own internal context (same device)
    yar_gpu_options opt{};
    opt.device = ctx->device;
    opt.max_batch_rays = 1u << 16;
    opt.traversal_kernel = ctx->forced_kernel < 0 ? YAR_TRAVERSAL_AUTO : ctx->forced_kernel + YAR_TRAVERSAL_PERSISTENT_64;
    for (uint32_t i = 0; i < count; i++) {
        Batch_Scene& s = bt.scenes[i];
        if (!scenes[i] || !rgb_out[i]) return fail(ctx, YAR_ERR_INVALID, "render batch: null scene or image");
        if ((rc = yar_gpu_create(&s.sub, &opt)) != YAR_OK) return fail(ctx, rc, "render batch: context");
        if ((rc = yar_gpu_upload_scene(s.sub, scenes[i])) != YAR_OK)
            return fail(ctx, rc, "scene " + std::to_string(i) + ": " + yar_gpu_last_error(s.sub));
        if ((rc = prepare_render_params(s.sub, s.p)) != YAR_OK)
            return fail(ctx, rc, "scene " + std::to_string(i) + ": " + yar_gpu_last_error(s.sub));
        if (s.sub->render.config.rendering_algorithm == 0)
            return fail(ctx, YAR_ERR_UNSUPPORTED, "scene " + std::to_string(i) +
                                                      ": batched renders run the path tracer only (rendering_algorithm 1)");
        s.pixels = (uint64_t)s.p.sw * s.p.sh;
        s.samples = s.pixels * s.p.spp;
        if (s.samples > 0xffffffffull) return fail(ctx, YAR_ERR_CAPACITY, "render batch: too many samples in a scene");
        if ((rc = device_alloc(ctx, s.radiance, s.samples * sizeof(float4))) != YAR_OK) return rc;
        if ((rc = device_alloc(ctx, s.image_samples, s.samples * sizeof(float2))) != YAR_OK) return rc;
        if ((rc = device_alloc(ctx, s.pixel_var, s.pixels * sizeof(double))) != YAR_OK) return rc;
        if ((rc = device_alloc(ctx, s.tile_var, (size_t)s.p.tiles_x * s.p.tiles_y * sizeof(double))) != YAR_OK)
            return rc;
        if ((rc = device_alloc(ctx, s.variance, sizeof(double))) != YAR_OK) return rc;
        if ((rc = device_alloc(ctx, s.rgb, (size_t)s.p.rw * s.p.rh * 3 * sizeof(float))) != YAR_OK) return rc;
    }
    if ((rc = device_alloc(ctx, bt.stamps, (1 + count) * sizeof(unsigned long long))) != YAR_OK) return rc;
    if ((rc = device_alloc(ctx, bt.rays, 2 * 16 * sizeof(unsigned long long))) != YAR_OK) return rc;
    const double upload_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    // autotuner, step 1: traversal kernel per scene on random rays in its box
    const auto t1 = std::chrono::steady_clock::now();
    {
        Device_Buffer rays_buf, hits;
        const uint32_t n = 1u << 16;
        if ((rc = device_alloc(ctx, rays_buf, (size_t)n * 32)) != YAR_OK) return rc;
        if ((rc = device_alloc(ctx, hits, (size_t)n * 24)) != YAR_OK) return rc;
        cudaError_t e = cudaSuccess;
        for (uint32_t i = 0; i < count && e == cudaSuccess; i++) {
            Batch_Scene& s = bt.scenes[i];
            const float* b = s.sub->ds.scene_bounds;
            random_rays_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
                dp<float4>(rays_buf), n, make_float3(b[0], b[1], b[2]), make_float3(b[3] - b[0], b[4] - b[1], b[5] - b[2]),
                0x9e3779b9ull + i);
            Cast_Args a;
            a.rays = dp<float4>(rays_buf);
            a.n = n;
            a.next_ray = ctx->d_counter;
            a.err = ctx->d_error;
            a.hit4 = dp<float4>(hits);
            a.hit2 = reinterpret_cast<uint2*>(dp<float4>(hits) + n);
            for (int kind = 0; kind < 2 && e == cudaSuccess; kind++) {
                if (s.sub->forced_kernel >= 0) {
                    s.kernel[kind] = s.sub->forced_kernel;
                    continue;
                }
                Cast_Args k = a;
                if (kind == 1) {
                    k.hit4 = nullptr;
                    k.hit2 = nullptr;
                    k.occluded = reinterpret_cast<uint8_t*>(dp<float4>(hits));
                }
                e = tune_cast(s.sub->ds, k, kind == 1, ctx->stream, ctx->ev_start, ctx->ev_stop, &s.kernel[kind]);
            }
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        device_free(rays_buf);
        device_free(hits);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "render batch: traversal kernel timing");
    }
    if (cudaError_t pe = generate_prepare()) return cuda_fail(ctx, pe, "render batch");
    // autotuner, step 2: branches x chunk capacity on the one-sample batch
    static const int kBranches[] = {2, 4, 8};
    static const uint64_t kChunks[] = {4u << 20, 16u << 20};
    int best_b = 4;
    uint64_t best_c = 16u << 20;
    double best_t = 1e30;
    cudaError_t e = cudaSuccess;
    for (int nb : kBranches) {
        for (uint64_t cc : kChunks) {
            if ((rc = alloc_branches(bt, nb, cc, true)) != YAR_OK) return rc;
            cudaGraphExec_t ex = nullptr;
            e = capture(bt, true, &ex);
            double gs = 0.0;
            if (e == cudaSuccess) e = run_graph(bt, ex, &gs);
            if (ex) cudaGraphExecDestroy(ex);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "render batch: tuning");
            if (gs < best_t) {
                best_t = gs;
                best_b = nb;
                best_c = cc;
            }
        }
    }
    const double tune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();

    // the batch: capture with the chosen shape, one launch
    const auto t2 = std::chrono::steady_clock::now();
    if ((rc = alloc_branches(bt, best_b, best_c, false)) != YAR_OK) return rc;
    cudaGraphExec_t exec = nullptr;
    e = capture(bt, false, &exec);
    const double capture_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t2).count();
    double gpu_seconds = 0.0;
    if (e == cudaSuccess) e = run_graph(bt, exec, &gpu_seconds);
    if (exec) cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render batch");
    uint32_t err = 0;
    for (Branch& br : bt.branches) {
        uint32_t h = 0;
        if (br.q.counters) e = cudaMemcpy(&h, br.q.counters + 3, sizeof(h), cudaMemcpyDeviceToHost);
        err |= h;
    }
    if (err) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
    std::vector<unsigned long long> st(1 + count), rays(2 * bt.branches.size());
    e = cudaMemcpy(st.data(), bt.stamps.ptr, st.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(rays.data(), bt.rays.ptr, rays.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    uint64_t total_paths = 0;
    for (uint32_t i = 0; i < count && e == cudaSuccess; i++) {
        Batch_Scene& s = bt.scenes[i];
        e = cudaMemcpy(rgb_out[i], s.rgb.ptr, (size_t)s.p.rw * s.p.rh * 3 * sizeof(float), cudaMemcpyDeviceToHost);
        double var = 0.0;
        if (e == cudaSuccess) e = cudaMemcpy(&var, s.variance.ptr, sizeof(double), cudaMemcpyDeviceToHost);
        total_paths += s.samples;
        if (scene_stats) {
            scene_stats[i].variance = var;
            scene_stats[i].completion_seconds = (float)((double)(st[1 + i] - st[0]) * 1e-9);
            scene_stats[i].paths = s.samples;
            scene_stats[i].traversal_kernel[0] = (uint32_t)s.kernel[0] + YAR_TRAVERSAL_PERSISTENT_64;
            scene_stats[i].traversal_kernel[1] = (uint32_t)s.kernel[1] + YAR_TRAVERSAL_PERSISTENT_64;
        }
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render batch: results");
    if (stats) {
        stats->gpu_seconds = (float)gpu_seconds;
        stats->paths = total_paths;
        uint64_t rc_closest = 0, rc_any = 0;
        for (size_t b = 0; b < bt.branches.size(); b++) {
            rc_closest += rays[2 * b];
            rc_any += rays[2 * b + 1];
        }
        stats->rays_closest = rc_closest;
        stats->rays_any = rc_any;
        stats->branches = (uint32_t)best_b;
        stats->chunk_paths = (uint32_t)best_c;
        stats->upload_seconds = (float)upload_seconds;
        stats->tune_seconds = (float)tune_seconds;
        stats->capture_seconds = (float)capture_seconds;
    }
    return YAR_OK;
}

extern "C" int yar_gpu_render_batch(yar_gpu_ctx* ctx, const yar_flat_scene* const* scenes, uint32_t count,
                                    float* const* rgb_out, yar_batch_scene_stats* scene_stats,
                                    yar_batch_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    return render_batch(ctx, scenes, count, rgb_out, scene_stats, stats);
}

} // namespace yar
