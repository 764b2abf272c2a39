// render.cu - wavefront path tracer (placeholder until the render kernels land).
#include "context.hpp"

namespace yar {

int render_upload(yar_gpu_ctx* ctx, const yar_flat_scene* scene) {
    ctx->render.camera = scene->camera;
    ctx->render.config = scene->config;
    return YAR_OK;
}

void render_release(yar_gpu_ctx* ctx) { (void)ctx; }

int render_run(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats) {
    (void)rgb_out;
    (void)stats;
    return fail(ctx, YAR_ERR_UNSUPPORTED, "render path not built");
}

} // namespace yar

extern "C" int yar_gpu_render(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return yar::fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    return yar::render_run(ctx, rgb_out, stats);
}
