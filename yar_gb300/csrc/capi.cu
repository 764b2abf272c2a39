// capi.cu - the C ABI of include/yar_gpu.h: contexts, scene upload and the
// ray-cast entry points.  Scene upload validates every index the kernels will
// follow (node links, leaf primitive indices, mesh and object references), so
// a malformed scene is rejected on the host with YAR_ERR_INVALID instead of
// reaching the device.
#include "context.hpp"

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace yar {

namespace {
// Casts of at least this many rays choose the traversal kernel by timing
// (smaller batches use the persistent 64-register kernel until then).
constexpr uint32_t kTuneMinRays = 1u << 20;
}  // namespace

int fail(yar_gpu_ctx* ctx, int code, const std::string& message) {
    if (ctx) ctx->last_error = message;
    return code;
}

int cuda_fail(yar_gpu_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, YAR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int device_alloc(yar_gpu_ctx* ctx, Device_Buffer& b, size_t bytes) {
    device_free(b);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        cudaGetLastError();
        return fail(ctx, YAR_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) + "): " +
                                            cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return YAR_OK;
}

void device_free(Device_Buffer& b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

namespace {

int upload(yar_gpu_ctx* ctx, Device_Buffer& b, const void* src, size_t bytes) {
    int rc = device_alloc(ctx, b, bytes);
    if (rc != YAR_OK) return rc;
    if (bytes) {
        cudaError_t e = cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "scene upload");
    }
    return YAR_OK;
}

// Structural check of a KdNode array (src/ref/kdtree.h:18-77): every reachable
// node index, leaf index-word range and primitive index stays inside bounds,
// and no root-to-leaf path is deeper than the traversal stack.
bool validate_tree(const yar_kdtree_view& t, uint32_t primitive_count, std::string& why) {
    if (!t.nodes || t.node_count == 0) { why = "empty kd-tree"; return false; }
    struct Item { uint32_t node; int depth; };
    std::vector<Item> todo{{0u, 0}};
    std::vector<uint8_t> seen(t.node_count, 0);
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        if (it.node >= t.node_count) { why = "node index out of range"; return false; }
        if (seen[it.node]) continue;  // DAG sharing would be unusual but harmless
        seen[it.node] = 1;
        if (it.depth > kMaxTraversalDepth) { why = "kd-tree deeper than the traversal stack"; return false; }
        const yar_kd_node n = t.nodes[it.node];
        if ((n.word0 & 3u) == 3u) {
            const uint32_t count = n.word0 >> 2;
            const uint64_t words_end = 2ull * it.node + 1 + count;  // word index one past the last index
            if (count > 0 && words_end > 2ull * t.node_count) { why = "leaf index array out of range"; return false; }
            const uint32_t* words = &t.nodes[it.node].word1;
            for (uint32_t i = 0; i < count; i++)
                if (words[i] >= primitive_count) { why = "leaf primitive index out of range"; return false; }
        } else {
            const uint32_t above = n.word0 >> 2;
            if (it.node + 1 >= t.node_count || above >= t.node_count || above <= it.node) {
                why = "interior child index out of range";
                return false;
            }
            todo.push_back({it.node + 1, it.depth + 1});
            todo.push_back({above, it.depth + 1});
        }
    }
    return true;
}

} // namespace
} // namespace yar

using namespace yar;

extern "C" int yar_gpu_traversal_kernels(yar_gpu_ctx* ctx, int32_t cast[2], int32_t render_closest[5],
                                         int32_t render_any[5]) {
    if (!ctx || !cast || !render_closest || !render_any) return YAR_ERR_INVALID;
    static_assert(yar_gpu_ctx::kBounceBuckets == YAR_TRAVERSAL_BOUNCE_BUCKETS, "bucket count");
    auto code = [](int k) { return k < 0 ? 0 : k + YAR_TRAVERSAL_PERSISTENT_64; };
    for (int i = 0; i < 2; i++) cast[i] = code(ctx->cast_kernel[i]);
    for (int b = 0; b < yar_gpu_ctx::kBounceBuckets; b++) {
        render_closest[b] = code(ctx->render_kernel[0][b]);
        render_any[b] = code(ctx->render_kernel[1][b]);
    }
    return YAR_OK;
}

extern "C" int yar_gpu_create(yar_gpu_ctx** out, const yar_gpu_options* options) {
    if (!out) return YAR_ERR_INVALID;
    *out = nullptr;
    yar_gpu_ctx* ctx = new (std::nothrow) yar_gpu_ctx();
    if (!ctx) return YAR_ERR_NOMEM;
    ctx->device = options ? options->device : 0;
    ctx->staging_capacity = (options && options->max_batch_rays) ? options->max_batch_rays : (16u << 20);
    if (options && options->pipeline_chunk_rays) ctx->pipe_chunk = options->pipeline_chunk_rays;
    if (options && options->traversal_kernel != YAR_TRAVERSAL_AUTO) {
        if (options->traversal_kernel < YAR_TRAVERSAL_PERSISTENT_64 ||
            options->traversal_kernel > YAR_TRAVERSAL_PER_RAY_VOTE) {
            delete ctx;
            return YAR_ERR_INVALID;
        }
        ctx->forced_kernel = options->traversal_kernel - YAR_TRAVERSAL_PERSISTENT_64;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        delete ctx;
        return YAR_ERR_CUDA;
    }
    if (ctx->device < 0 || ctx->device >= count) {
        delete ctx;
        return YAR_ERR_INVALID;
    }
    e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_error, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_error, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counter, yar_gpu_ctx::kPipeChunks * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_start);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_stop);
    if (e != cudaSuccess) {
        cudaGetLastError();
        yar_gpu_destroy(ctx);
        return YAR_ERR_CUDA;
    }
    *out = ctx;
    return YAR_OK;
}

extern "C" void yar_gpu_destroy(yar_gpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    render_release(ctx);
    guide_release(ctx);
    for (Device_Buffer* b : {&ctx->scene_nodes, &ctx->mesh_nodes, &ctx->objects, &ctx->tris, &ctx->d_rays, &ctx->d_t,
                             &ctx->d_prim, &ctx->d_obj, &ctx->d_bary, &ctx->d_occ})
        device_free(*b);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    for (cudaStream_t s : {ctx->pipe_in, ctx->pipe_compute, ctx->pipe_out, ctx->aux_stream})
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t ev : {ctx->aux_fork, ctx->aux_join})
        if (ev) cudaEventDestroy(ev);
    if (ctx->pipe_start) cudaEventDestroy(ctx->pipe_start);
    for (int c = 0; c < yar_gpu_ctx::kPipeChunks; c++) {
        if (ctx->pipe_in_done[c]) cudaEventDestroy(ctx->pipe_in_done[c]);
        if (ctx->pipe_cast_done[c]) cudaEventDestroy(ctx->pipe_cast_done[c]);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char* yar_gpu_last_error(const yar_gpu_ctx* ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" void* yar_gpu_stream(yar_gpu_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int yar_gpu_synchronize(yar_gpu_ctx* ctx) {
    if (!ctx) return YAR_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
    return YAR_OK;
}

extern "C" int yar_gpu_upload_scene(yar_gpu_ctx* ctx, const yar_flat_scene* scene) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!scene || scene->mesh_count == 0 || scene->object_count == 0 || !scene->meshes || !scene->objects)
        return fail(ctx, YAR_ERR_INVALID, "scene has no meshes or objects");
    cudaSetDevice(ctx->device);
    ctx->has_scene = false;
    std::string why;
    // meshes: validate, gather triangles, concatenate node arrays
    std::vector<uint32_t> node_offset(scene->mesh_count), tri_offset(scene->mesh_count);
    uint64_t total_nodes = 0, total_tris = 0;
    for (uint32_t m = 0; m < scene->mesh_count; m++) {
        const yar_mesh_desc& mesh = scene->meshes[m];
        if (!mesh.vertices || !mesh.indices || mesh.triangle_count == 0)
            return fail(ctx, YAR_ERR_INVALID, "mesh " + std::to_string(m) + " has no triangles");
        for (uint64_t i = 0; i < 3ull * mesh.triangle_count; i++)
            if (mesh.indices[i] < 0 || (uint32_t)mesh.indices[i] >= mesh.vertex_count)
                return fail(ctx, YAR_ERR_INVALID, "mesh " + std::to_string(m) + " index out of range");
        if (!validate_tree(mesh.kdtree, mesh.triangle_count, why))
            return fail(ctx, YAR_ERR_INVALID, "mesh " + std::to_string(m) + ": " + why);
        node_offset[m] = (uint32_t)total_nodes;
        tri_offset[m] = (uint32_t)total_tris;
        total_nodes += mesh.kdtree.node_count;
        total_tris += mesh.triangle_count;
        if (total_nodes > 0xffffffffull || total_tris > 0x3fffffffull)
            return fail(ctx, YAR_ERR_CAPACITY, "scene exceeds 2^32 nodes or 2^30 triangles");
    }
    if (!validate_tree(scene->scene_kdtree, scene->object_count, why))
        return fail(ctx, YAR_ERR_INVALID, "scene tree: " + why);

    std::vector<uint2> nodes;
    std::vector<float4> tris;
    std::vector<float4> objects;
    try {
        nodes.resize(total_nodes);
        tris.resize(3 * total_tris);
        objects.resize(6 * (size_t)scene->object_count);
    } catch (const std::bad_alloc&) {
        return fail(ctx, YAR_ERR_NOMEM, "host staging for scene upload");
    }
    for (uint32_t m = 0; m < scene->mesh_count; m++) {
        const yar_mesh_desc& mesh = scene->meshes[m];
        memcpy(&nodes[node_offset[m]], mesh.kdtree.nodes, mesh.kdtree.node_count * sizeof(uint2));
        for (uint32_t t = 0; t < mesh.triangle_count; t++) {
            const float* p[3];
            for (int k = 0; k < 3; k++) p[k] = mesh.vertices + 3 * (size_t)mesh.indices[3 * (size_t)t + k];
            // cross(p1 - p0, p2 - p0).length_squared() == 0, as src/ref/kdtree.cpp:27-29 evaluates it
            const float a0 = p[1][0] - p[0][0], a1 = p[1][1] - p[0][1], a2 = p[1][2] - p[0][2];
            const float c0 = p[2][0] - p[0][0], c1 = p[2][1] - p[0][1], c2 = p[2][2] - p[0][2];
            const float x = a1 * c2 - a2 * c1, y = a2 * c0 - a0 * c2, z = a0 * c1 - a1 * c0;
            const float len2 = x * x + y * y + z * z;
            const float flag = (len2 == 0.f) ? 1.f : 0.f;
            float4* dst = &tris[3 * ((size_t)tri_offset[m] + t)];
            dst[0] = make_float4(p[0][0], p[0][1], p[0][2], flag);
            dst[1] = make_float4(p[1][0], p[1][1], p[1][2], 0.f);
            dst[2] = make_float4(p[2][0], p[2][1], p[2][2], 0.f);
        }
    }
    for (uint32_t i = 0; i < scene->object_count; i++) {
        const yar_object_desc& o = scene->objects[i];
        if (o.mesh_index < 0 || (uint32_t)o.mesh_index >= scene->mesh_count)
            return fail(ctx, YAR_ERR_INVALID, "object " + std::to_string(i) + " has an invalid mesh index");
        const yar_mesh_desc& mesh = scene->meshes[o.mesh_index];
        float4* r = &objects[6 * (size_t)i];
        const float* w = o.world_to_object;
        r[0] = make_float4(w[0], w[1], w[2], w[3]);
        r[1] = make_float4(w[4], w[5], w[6], w[7]);
        r[2] = make_float4(w[8], w[9], w[10], w[11]);
        uint32_t no = node_offset[o.mesh_index], to = tri_offset[o.mesh_index];
        float nof, tof;
        memcpy(&nof, &no, 4);
        memcpy(&tof, &to, 4);
        r[3] = make_float4(mesh.kdtree.bounds_min[0], mesh.kdtree.bounds_min[1], mesh.kdtree.bounds_min[2], nof);
        r[4] = make_float4(mesh.kdtree.bounds_max[0], mesh.kdtree.bounds_max[1], mesh.kdtree.bounds_max[2], tof);
        // info.z: the first mip of the mesh's alpha texture, -1 without one
        int32_t alpha_mip = -1;
        if (mesh.alpha_texture) {
            if (mesh.alpha_texture > scene->texture_count || !mesh.uvs || !scene->texture_mips)
                return fail(ctx, YAR_ERR_INVALID, "mesh " + std::to_string(o.mesh_index) +
                                                      ": alpha texture without uvs or out of range");
            const uint32_t first = scene->textures[mesh.alpha_texture - 1].first_mip;
            if (first >= scene->texture_mip_count)
                return fail(ctx, YAR_ERR_INVALID, "alpha texture with an invalid mip");
            alpha_mip = (int32_t)first;
        }
        int32_t info[4] = {o.mesh_index, mesh.visibility, alpha_mip, 0};
        memcpy(&r[5], info, 16);
    }
    int rc;
    if ((rc = upload(ctx, ctx->mesh_nodes, nodes.data(), nodes.size() * sizeof(uint2))) != YAR_OK) return rc;
    if ((rc = upload(ctx, ctx->tris, tris.data(), tris.size() * sizeof(float4))) != YAR_OK) return rc;
    if ((rc = upload(ctx, ctx->objects, objects.data(), objects.size() * sizeof(float4))) != YAR_OK) return rc;
    if ((rc = upload(ctx, ctx->scene_nodes, scene->scene_kdtree.nodes,
                     scene->scene_kdtree.node_count * sizeof(uint2))) != YAR_OK)
        return rc;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);  // host staging vectors die at return
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scene upload");

    Device_Scene& ds = ctx->ds;
    ds.scene_nodes = (const uint2*)ctx->scene_nodes.ptr;
    ds.mesh_nodes = (const uint2*)ctx->mesh_nodes.ptr;
    ds.objects = (const float4*)ctx->objects.ptr;
    ds.tris = (const float4*)ctx->tris.ptr;
    memcpy(ds.scene_bounds, scene->scene_kdtree.bounds_min, 12);
    memcpy(ds.scene_bounds + 3, scene->scene_kdtree.bounds_max, 12);
    ds.object_count = scene->object_count;

    rc = render_upload(ctx, scene);
    if (rc != YAR_OK) return rc;
    // the alpha test reads the triangles' uvs and the textures' texels
    ds.shading = (const float4*)ctx->render.shading.ptr;
    ds.texels = (const float4*)ctx->render.texels.ptr;
    ds.texture_mips = (const uint4*)ctx->render.texture_mips.ptr;
    for (int k = 0; k < 2; k++) {
        ctx->cast_kernel[k] = ctx->forced_kernel;
        for (int b = 0; b < yar_gpu_ctx::kBounceBuckets; b++) ctx->render_kernel[k][b] = ctx->forced_kernel;
    }
    ctx->render_tuned = ctx->forced_kernel >= 0;
    memset(ctx->render_tune_ms, 0, sizeof(ctx->render_tune_ms));
    memset(ctx->render_tune_queues, 0, sizeof(ctx->render_tune_queues));
    ctx->has_scene = true;
    return YAR_OK;
}

namespace {

int ensure_staging(yar_gpu_ctx* ctx, uint32_t n, bool closest) {
    if (n > ctx->staging_capacity)
        return fail(ctx, YAR_ERR_CAPACITY, "batch of " + std::to_string(n) + " rays exceeds max_batch_rays");
    int rc;
    if (ctx->d_rays.bytes < (size_t)n * 32 && (rc = device_alloc(ctx, ctx->d_rays, (size_t)n * 32)) != YAR_OK) return rc;
    if (closest) {
        if (ctx->d_t.bytes < (size_t)n * 4 && (rc = device_alloc(ctx, ctx->d_t, (size_t)n * 4)) != YAR_OK) return rc;
        if (ctx->d_prim.bytes < (size_t)n * 4 && (rc = device_alloc(ctx, ctx->d_prim, (size_t)n * 4)) != YAR_OK) return rc;
        if (ctx->d_obj.bytes < (size_t)n * 4 && (rc = device_alloc(ctx, ctx->d_obj, (size_t)n * 4)) != YAR_OK) return rc;
        if (ctx->d_bary.bytes < (size_t)n * 8 && (rc = device_alloc(ctx, ctx->d_bary, (size_t)n * 8)) != YAR_OK) return rc;
    } else {
        if (ctx->d_occ.bytes < (size_t)n && (rc = device_alloc(ctx, ctx->d_occ, (size_t)n)) != YAR_OK) return rc;
    }
    return YAR_OK;
}

int check_error_word(yar_gpu_ctx* ctx) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel");
    if (h) {
        cudaMemsetAsync(ctx->d_error, 0, sizeof(int), ctx->stream);
        return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
    }
    return YAR_OK;
}

// Host-buffer casts of at least two pipeline chunks: chunk c's rays go up on
// pipe_in, its traversal runs on the context's stream or pipe_compute
// (alternating, so one chunk's tail overlaps the next chunk's start), its
// results come down on pipe_out.  Every chunk keeps its own offsets in the
// staging buffers and its own hand-out counter.
uint32_t pipeline_chunks(const yar_gpu_ctx* ctx, uint32_t n) {
    if (ctx->pipe_chunk == 0xffffffffu) return 1;
    const uint64_t c = ((uint64_t)n + ctx->pipe_chunk - 1) / ctx->pipe_chunk;
    return (uint32_t)std::min<uint64_t>(c, yar_gpu_ctx::kPipeChunks - 2);  // room for the two short chunks
}

int ensure_pipeline(yar_gpu_ctx* ctx) {
    cudaError_t e = cudaSuccess;
    for (cudaStream_t* s : {&ctx->pipe_in, &ctx->pipe_compute, &ctx->pipe_out})
        if (!*s && e == cudaSuccess) e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
    if (!ctx->pipe_start && e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->pipe_start, cudaEventDisableTiming);
    for (int c = 0; c < yar_gpu_ctx::kPipeChunks && e == cudaSuccess; c++) {
        if (!ctx->pipe_in_done[c]) e = cudaEventCreateWithFlags(&ctx->pipe_in_done[c], cudaEventDisableTiming);
        if (!ctx->pipe_cast_done[c] && e == cudaSuccess)
            e = cudaEventCreateWithFlags(&ctx->pipe_cast_done[c], cudaEventDisableTiming);
    }
    return e == cudaSuccess ? YAR_OK : cuda_fail(ctx, e, "cast pipeline streams");
}

int cast_pipelined(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n, const yar_hit_soa* hits, uint8_t* occluded,
                   int kernel) {
    const bool closest = hits != nullptr;
    int rc = ensure_pipeline(ctx);
    if (rc != YAR_OK) return rc;
    // chunk boundaries: a short first chunk (the traversal starts after a
    // quarter of a chunk's copy) and a short last one (its results come down
    // sooner), equal chunks between
    std::vector<uint32_t> bounds{0u};
    {
        const uint32_t mid_chunks = pipeline_chunks(ctx, n);
        const uint32_t ramp = std::min<uint32_t>(ctx->pipe_chunk / 4u, n / 8u) & ~31u;
        const uint32_t head = ramp, tail = ramp;
        const uint32_t middle = n - head - tail;
        const uint32_t per = (uint32_t)((((uint64_t)middle + mid_chunks - 1) / mid_chunks + 31u) & ~31ull);
        if (head) bounds.push_back(head);
        for (uint32_t c = 0; c < mid_chunks; c++) {
            const uint64_t b = std::min<uint64_t>((uint64_t)head + (uint64_t)(c + 1) * per, (uint64_t)n - tail);
            if (b > bounds.back()) bounds.push_back((uint32_t)b);
        }
        if (n > bounds.back()) bounds.push_back(n);
    }
    const uint32_t chunks = (uint32_t)bounds.size() - 1u;
    if (chunks > (uint32_t)yar_gpu_ctx::kPipeChunks) return fail(ctx, YAR_ERR_INVALID, "pipeline chunks");
    cudaStream_t compute[2] = {ctx->stream, ctx->pipe_compute};
    cudaError_t e = cudaEventRecord(ctx->pipe_start, ctx->stream);  // after the context's earlier work
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->pipe_in, ctx->pipe_start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->pipe_compute, ctx->pipe_start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->pipe_out, ctx->pipe_start, 0);
    float4* d_rays = (float4*)ctx->d_rays.ptr;
    for (uint32_t c = 0; c < chunks && e == cudaSuccess; c++) {
        const uint32_t first = bounds[c];
        const uint32_t m = bounds[c + 1] - first;
        e = cudaMemcpyAsync(d_rays + 2 * (size_t)first, rays + first, (size_t)m * 32, cudaMemcpyHostToDevice,
                            ctx->pipe_in);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->pipe_in_done[c], ctx->pipe_in);
        cudaStream_t ks = compute[c & 1];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ks, ctx->pipe_in_done[c], 0);
        if (e != cudaSuccess) break;
        Cast_Args a;
        a.rays = d_rays + 2 * (size_t)first;
        a.n = m;
        a.next_ray = ctx->d_counter + c;
        a.err = ctx->d_error;
        if (closest) {
            a.t = hits->t ? (float*)ctx->d_t.ptr + first : nullptr;
            a.prim = hits->prim ? (uint32_t*)ctx->d_prim.ptr + first : nullptr;
            a.object = hits->object ? (uint32_t*)ctx->d_obj.ptr + first : nullptr;
            a.bary = hits->bary ? (float2*)ctx->d_bary.ptr + first : nullptr;
        } else {
            a.occluded = (uint8_t*)ctx->d_occ.ptr + first;
        }
        e = closest ? launch_extend(ctx->ds, a, kernel, ks) : launch_shadow(ctx->ds, a, kernel, ks);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->pipe_cast_done[c], ks);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->pipe_out, ctx->pipe_cast_done[c], 0);
        cudaStream_t os = ctx->pipe_out;
        if (closest) {
            if (e == cudaSuccess && hits->t)
                e = cudaMemcpyAsync(hits->t + first, a.t, (size_t)m * 4, cudaMemcpyDeviceToHost, os);
            if (e == cudaSuccess && hits->prim)
                e = cudaMemcpyAsync(hits->prim + first, a.prim, (size_t)m * 4, cudaMemcpyDeviceToHost, os);
            if (e == cudaSuccess && hits->object)
                e = cudaMemcpyAsync(hits->object + first, a.object, (size_t)m * 4, cudaMemcpyDeviceToHost, os);
            if (e == cudaSuccess && hits->bary)
                e = cudaMemcpyAsync(hits->bary + 2 * (size_t)first, a.bary, (size_t)m * 8, cudaMemcpyDeviceToHost, os);
        } else if (e == cudaSuccess) {
            e = cudaMemcpyAsync(occluded + first, a.occluded, m, cudaMemcpyDeviceToHost, os);
        }
    }
    // every stream finishes before the call returns; the context's stream last
    for (cudaStream_t s : {ctx->pipe_in, ctx->pipe_compute, ctx->pipe_out}) {
        const cudaError_t e2 = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pipelined cast");
    return check_error_word(ctx);
}

int cast(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n, const yar_hit_soa* hits, uint8_t* occluded,
         int32_t buffers, float* kernel_ms) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    const bool closest = hits != nullptr;
    if (n && !rays) return fail(ctx, YAR_ERR_INVALID, "null ray buffer");
    if (!closest && n && !occluded) return fail(ctx, YAR_ERR_INVALID, "null output buffer");
    if (buffers != YAR_BUFFERS_HOST && buffers != YAR_BUFFERS_DEVICE) return fail(ctx, YAR_ERR_INVALID, "buffers flag");
    if (n == 0) return YAR_OK;
    cudaSetDevice(ctx->device);
    cudaError_t e;
    const float4* d_rays;
    float* d_t = nullptr;
    uint32_t *d_prim = nullptr, *d_obj = nullptr;
    float2* d_bary = nullptr;
    uint8_t* d_occ = nullptr;
    if (buffers == YAR_BUFFERS_HOST) {
        int rc = ensure_staging(ctx, n, closest);
        if (rc != YAR_OK) return rc;
        // a tuned (or fixed) traversal kernel and at least two chunks: overlap copies and traversal
        const int tuned = ctx->cast_kernel[closest ? 0 : 1];
        if (!kernel_ms && pipeline_chunks(ctx, n) >= 2 && (tuned >= 0 || n < kTuneMinRays))
            return cast_pipelined(ctx, rays, n, hits, occluded, tuned < 0 ? kCastPersistent64 : tuned);
        e = cudaMemcpyAsync(ctx->d_rays.ptr, rays, (size_t)n * 32, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "ray upload");
        d_rays = (const float4*)ctx->d_rays.ptr;
        if (closest) {
            d_t = hits->t ? (float*)ctx->d_t.ptr : nullptr;
            d_prim = hits->prim ? (uint32_t*)ctx->d_prim.ptr : nullptr;
            d_obj = hits->object ? (uint32_t*)ctx->d_obj.ptr : nullptr;
            d_bary = hits->bary ? (float2*)ctx->d_bary.ptr : nullptr;
        } else {
            d_occ = (uint8_t*)ctx->d_occ.ptr;
        }
    } else {
        if (((uintptr_t)rays & 15u) != 0) return fail(ctx, YAR_ERR_INVALID, "device ray buffer must be 16-byte aligned");
        d_rays = (const float4*)rays;
        if (closest) {
            d_t = hits->t;
            d_prim = hits->prim;
            d_obj = hits->object;
            d_bary = (float2*)hits->bary;
            if (((uintptr_t)d_bary & 7u) != 0) return fail(ctx, YAR_ERR_INVALID, "bary buffer must be 8-byte aligned");
        } else {
            d_occ = occluded;
        }
    }
    Cast_Args a;
    a.rays = d_rays;
    a.n = n;
    a.next_ray = ctx->d_counter;
    a.err = ctx->d_error;
    a.t = d_t;
    a.prim = d_prim;
    a.object = d_obj;
    a.bary = d_bary;
    a.occluded = d_occ;
    int& kernel = ctx->cast_kernel[closest ? 0 : 1];
    if (kernel < 0 && n >= kTuneMinRays) {
        e = tune_cast(ctx->ds, a, !closest, ctx->stream, ctx->ev_start, ctx->ev_stop, &kernel);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "traversal kernel timing");
    }
    if (kernel_ms) cudaEventRecord(ctx->ev_start, ctx->stream);
    const int k = kernel < 0 ? kCastPersistent64 : kernel;
    e = closest ? launch_extend(ctx->ds, a, k, ctx->stream) : launch_shadow(ctx->ds, a, k, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, closest ? "extend launch" : "shadow launch");
    if (kernel_ms) cudaEventRecord(ctx->ev_stop, ctx->stream);
    if (buffers == YAR_BUFFERS_HOST) {
        if (closest) {
            if (hits->t) e = cudaMemcpyAsync(hits->t, d_t, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess && hits->prim)
                e = cudaMemcpyAsync(hits->prim, d_prim, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess && hits->object)
                e = cudaMemcpyAsync(hits->object, d_obj, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess && hits->bary)
                e = cudaMemcpyAsync(hits->bary, d_bary, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream);
        } else {
            e = cudaMemcpyAsync(occluded, d_occ, n, cudaMemcpyDeviceToHost, ctx->stream);
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "result download");
    }
    int rc = check_error_word(ctx);
    if (rc != YAR_OK) return rc;
    if (kernel_ms) {
        e = cudaEventElapsedTime(kernel_ms, ctx->ev_start, ctx->ev_stop);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "event timing");
    }
    return YAR_OK;
}

} // namespace

extern "C" int yar_gpu_cast_closest(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n, const yar_hit_soa* hits,
                                    int32_t buffers) {
    if (!hits) return fail(ctx, YAR_ERR_INVALID, "null hit buffers");
    return cast(ctx, rays, n, hits, nullptr, buffers, nullptr);
}

extern "C" int yar_gpu_cast_any(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n, uint8_t* occluded,
                                int32_t buffers) {
    return cast(ctx, rays, n, nullptr, occluded, buffers, nullptr);
}

extern "C" int yar_gpu_cast_closest_timed(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n,
                                          const yar_hit_soa* hits, float* kernel_ms) {
    if (!hits || !kernel_ms) return fail(ctx, YAR_ERR_INVALID, "null argument");
    return cast(ctx, rays, n, hits, nullptr, YAR_BUFFERS_DEVICE, kernel_ms);
}

extern "C" int yar_gpu_cast_any_timed(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t n, uint8_t* occluded,
                                      float* kernel_ms) {
    if (!kernel_ms) return fail(ctx, YAR_ERR_INVALID, "null argument");
    return cast(ctx, rays, n, nullptr, occluded, YAR_BUFFERS_DEVICE, kernel_ms);
}
