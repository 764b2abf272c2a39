// render_scene_gpu.cpp - the reference-side drop-in for render_scene
// (src/ref/reference_renderer.h:55), compiled against the reference's own
// headers and linked with the reference's sources (libyarref.a) and the
// product library (libyar_gb300.so) by oracle/build_ref.sh into
// oracle/_ref/yar_ref_gpu.  This is the binding a maintainer adds to YAR:
// the reference loads the pbrt-v3 scene and builds its kd-trees as always
// (load_scene, init_scene_context); render_scene_gpu flattens the result
// (ref_flatten.hpp) and renders it through the C ABI.
//
//   yar_ref_gpu <scene.pbrt> <out.img> [--spp=N] [--seedoffset=S] [--device=D]
//
// writes the same file as `yar_ref render`: u32 w, u32 h, f64 variance,
// f32 seconds, f32 rgb[w*h*3].
#include "std.h"
#include "lib/common.h"
#include "lib/scene.h"
#include "lib/scene_loader.h"
#include "ref/reference_renderer.h"
#include "ref/scene_context.h"

#include "ref_flatten.hpp"
#include "yar_gpu.h"
#include "yfs.hpp"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <unistd.h>

// render_scene's signature and results (Image, variance estimate, render
// time), with the scene the context was initialised from.
Image render_scene_gpu(const Scene& scene, const Scene_Context& scene_ctx, double* variance_estimate,
                       float* render_time, int device = 0) {
    yfs::Scene flat = flatten(scene, scene_ctx);
    const yar_flat_scene desc = flat.view();
    yar_gpu_ctx* ctx = nullptr;
    yar_gpu_options opts{};
    opts.device = device;
    if (yar_gpu_create(&ctx, &opts) != YAR_OK) error("yar_gpu_create: no CUDA device");
    if (yar_gpu_upload_scene(ctx, &desc) != YAR_OK) error("yar_gpu_upload_scene: %s", yar_gpu_last_error(ctx));
    Image image(scene_ctx.render_region.size().x, scene_ctx.render_region.size().y);
    yar_render_stats stats{};
    if (yar_gpu_render(ctx, &image.data[0].r, &stats) != YAR_OK) error("yar_gpu_render: %s", yar_gpu_last_error(ctx));
    if (variance_estimate) *variance_estimate = stats.variance;
    if (render_time) *render_time = stats.seconds;
    yar_gpu_destroy(ctx);
    return image;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: yar_ref_gpu <scene.pbrt> <out.img> [--spp=N] [--seedoffset=S] [--device=D]\n");
        return 2;
    }
    int spp = 0, seed_offset = 0, device = 0;
    for (int i = 3; i < argc; i++) {
        const std::string s = argv[i];
        if (s.rfind("--spp=", 0) == 0) spp = atoi(s.c_str() + 6);
        else if (s.rfind("--seedoffset=", 0) == 0) seed_offset = atoi(s.c_str() + 13);
        else if (s.rfind("--device=", 0) == 0) device = atoi(s.c_str() + 9);
    }
    Scene scene = load_scene(argv[1]);
    if (spp > 0) {  // src/ref/main.cpp:386-390
        const int k = (int)std::ceil(std::sqrt(spp));
        scene.raytracer_config.x_pixel_sample_count = k;
        scene.raytracer_config.y_pixel_sample_count = k;
    }
    // the reference's kd-tree cache goes to a private directory, rebuilt every time
    const std::string data_dir = (fs::temp_directory_path() / ("yar_ref_gpu_" + std::to_string(getpid()))).string();
    fs::create_directories(data_dir);
    set_data_directory(data_dir);
    Reference_Renderer_Config config;
    config.rebuild_kdtree_cache = true;
    config.rng_seed_offset = seed_offset;
    Scene_Context ctx;
    init_scene_context(ctx, scene, config);
    std::error_code ec;
    fs::remove_all(data_dir, ec);

    double variance = 0.0;
    float seconds = 0.f;
    Image image = render_scene_gpu(scene, ctx, &variance, &seconds, device);
    FILE* f = fopen(argv[2], "wb");
    if (!f) return 1;
    const uint32_t w = (uint32_t)image.width, h = (uint32_t)image.height;
    fwrite(&w, 4, 1, f);
    fwrite(&h, 4, 1, f);
    fwrite(&variance, 8, 1, f);
    fwrite(&seconds, 4, 1, f);
    fwrite(image.data.data(), sizeof(ColorRGB), image.data.size(), f);
    fclose(f);
    printf("{\"render_seconds\": %.6f, \"variance\": %.9g, \"width\": %u, \"height\": %u}\n", seconds, variance, w, h);
    return 0;
}
