// ref_harness.cpp - test infrastructure: drives the reference renderer's own
// code (compiled by oracle/build_ref.sh into oracle/_ref/libyarref.a) so the
// oracle restatement and the GPU path can be pinned against it.
//
// Its flatten command runs the reference-side adapter of the C ABI
// (ref_flatten.hpp): a reference Scene + Scene_Context converted into the flat
// scene (include/yar_gpu.h) that yar_gpu_upload_scene consumes.
//
// commands
//   flatten  <scene.pbrt> <out.yfs> [--spp=N] [--seedoffset=S]
//       load_scene (src/lib/scene_loader.cpp:74-133) + init_scene_context
//       (src/ref/reference_renderer.cpp:586-621, reference kd-tree builder)
//       and write the flat scene.
//   render   <scene.pbrt> <out.img> [--spp=N] [--seedoffset=S] [--threads=T]
//       render_scene (src/ref/reference_renderer.cpp:479-584); writes
//       u32 w, u32 h, f64 variance, f32 seconds, f32 rgb[w*h*3].
//   build    <in.yfs> <out.yfs> [--threads=T]
//       build_triangle_mesh_kdtree / build_scene_kdtree
//       (src/ref/kdtree_builder.cpp:425-463) for the meshes and objects of a
//       flat scene; prints the build time.
//   cast     <in.yfs> <rays.bin> <out.bin> [--threads=T] [--any] [--repeat=R]
//       KdTree::intersect / intersect_any (src/ref/kdtree.cpp:219-439) over
//       the scene tree for a batch of yar_ray records; closest writes
//       f32 t[n], u32 prim[n], u32 obj[n], f32 bary[2n]; any writes u8[n].
//       Prints {"rays":..,"seconds":..,"threads":..} on stdout.
//   bench-cast <in.yfs> <rays.bin> <shadow_rays.bin> [--build] [--threads=T] [--warmup=W] [--steps=K]
//       the ray-cast benchmark: reference kd-tree build (--build), then timed
//       steps of one closest-hit and one any-hit batch.
#include "std.h"
// render-yfs sets the reference Camera's fields to the flat scene's exact
// values; Camera keeps them private (src/ref/camera.h:41-48).
#define private public
#include "ref/camera.h"
#undef private
#include "lib/common.h"
#include "lib/scene.h"
#include "lib/scene_loader.h"
#include "lib/scene_object.h"
#include "lib/triangle_mesh.h"
#include "ref/camera.h"
#include "ref/intersection.h"
#include "ref/kdtree.h"
#include "ref/kdtree_builder.h"
#include "ref/reference_renderer.h"
#include "ref/sampling.h"
#include "lib/math.h"
#include "lib/random.h"
#include "ref/scene_context.h"

#include "ref_flatten.hpp"
#include "yfs.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Args {
    std::vector<std::string> pos;
    int spp = 0;
    int seed_offset = 0;
    int threads = 0;
    bool any = false;
    int repeat = 1;
    int steps = 1;
    int warmup = 0;
    bool build = false;
    bool compress = false;
    float variance = 0.f;
    std::string input_file;
    std::string cache_dir;
    std::string checkpoint_dir;
    std::string textures_from;
};

Args parse(int argc, char** argv) {
    Args a;
    for (int i = 2; i < argc; i++) {
        std::string s = argv[i];
        if (s.rfind("--spp=", 0) == 0) a.spp = atoi(s.c_str() + 6);
        else if (s.rfind("--seedoffset=", 0) == 0) a.seed_offset = atoi(s.c_str() + 13);
        else if (s.rfind("--threads=", 0) == 0) a.threads = atoi(s.c_str() + 10);
        else if (s.rfind("--repeat=", 0) == 0) a.repeat = atoi(s.c_str() + 9);
        else if (s.rfind("--steps=", 0) == 0) a.steps = atoi(s.c_str() + 8);
        else if (s.rfind("--warmup=", 0) == 0) a.warmup = atoi(s.c_str() + 9);
        else if (s == "--build") a.build = true;
        else if (s == "--any") a.any = true;
        else if (s.rfind("--checkpoint-dir=", 0) == 0) a.checkpoint_dir = s.substr(17);
        else if (s == "--compress") a.compress = true;
        else if (s.rfind("--variance=", 0) == 0) a.variance = (float)atof(s.c_str() + 11);
        else if (s.rfind("--input=", 0) == 0) a.input_file = s.substr(8);
        else if (s.rfind("--cache-dir=", 0) == 0) a.cache_dir = s.substr(12);
        else if (s.rfind("--textures-from=", 0) == 0) a.textures_from = s.substr(16);
        else a.pos.push_back(s);
    }
    if (a.threads <= 0) a.threads = std::max(1u, std::thread::hardware_concurrency());
    return a;
}

Scene load_with_overrides(const Args& a) {
    Scene scene = load_scene(a.pos[0]);
    if (a.spp > 0) {
        int k = (int)std::ceil(std::sqrt(a.spp));  // src/ref/main.cpp:386-390
        scene.raytracer_config.x_pixel_sample_count = k;
        scene.raytracer_config.y_pixel_sample_count = k;
    }
    return scene;
}

void init_context(Scene_Context& ctx, const Scene& scene, const Args& a) {
    // the kd-tree cache goes to a private directory, rebuilt every time
    std::string data_dir = (fs::temp_directory_path() / ("yar_ref_data_" + std::to_string(getpid()))).string();
    fs::create_directories(data_dir);
    set_data_directory(data_dir);
    Reference_Renderer_Config config;
    config.thread_count = a.threads;
    config.rebuild_kdtree_cache = true;
    config.rng_seed_offset = a.seed_offset;
    config.checkpoint_directory = a.checkpoint_dir;
    init_scene_context(ctx, scene, config);
    std::error_code ec;
    fs::remove_all(data_dir, ec);
}

// Reference objects reconstructed from a flat scene (for build and cast).
struct Ref_Scene {
    std::vector<Triangle_Mesh> meshes;
    std::vector<Triangle_Mesh_Geometry_Data> geometry_data;
    std::vector<KdTree> kdtrees;
    std::vector<Scene_Object> objects;
    Scene_Geometry_Data scene_data;
    KdTree scene_kdtree;
};

void load_ref_meshes(const yfs::Scene& fs_scene, Ref_Scene& rs) {
    rs.meshes.resize(fs_scene.meshes.size());
    for (size_t i = 0; i < fs_scene.meshes.size(); i++) {
        const yfs::Mesh& fm = fs_scene.meshes[i];
        Triangle_Mesh& m = rs.meshes[i];
        m.vertices.resize(fm.vertices.size() / 3);
        memcpy(m.vertices.data(), fm.vertices.data(), fm.vertices.size() * 4);
        m.normals.resize(fm.normals.size() / 3);
        if (!fm.normals.empty()) memcpy(m.normals.data(), fm.normals.data(), fm.normals.size() * 4);
        m.uvs.resize(fm.uvs.size() / 2);
        if (!fm.uvs.empty()) memcpy(m.uvs.data(), fm.uvs.data(), fm.uvs.size() * 4);
        m.indices = fm.indices;
        m.reverse_geometric_normal_orientation = fm.reverse_orientation != 0;
        m.visibility = (Visibility)fm.visibility;
    }
    rs.geometry_data.resize(rs.meshes.size());
    for (size_t i = 0; i < rs.meshes.size(); i++) {
        rs.geometry_data[i].mesh = &rs.meshes[i];
        if (rs.meshes[i].visibility == Visibility::invisible) {
            rs.geometry_data[i].ignore_intersector = true;
            rs.geometry_data[i].ignore_any_intersector = true;
        } else if (rs.meshes[i].visibility == Visibility::visible_no_shadows) {
            rs.geometry_data[i].ignore_any_intersector = true;
        }
    }
    rs.objects.resize(fs_scene.objects.size());
    for (size_t i = 0; i < fs_scene.objects.size(); i++) {
        const yar_object_desc& d = fs_scene.objects[i];
        Scene_Object& o = rs.objects[i];
        o.geometry = {Geometry_Type::triangle_mesh, d.mesh_index};
        o.material = {(Material_Type)d.material_type, d.material_index};
        o.area_light = {(Light_Type)d.area_light_type, d.area_light_index};
        o.object_to_world_transform = floats_to_matrix(d.object_to_world);
        o.world_to_object_transform = floats_to_matrix(d.world_to_object);
        o.object_to_world_normal_transform = floats_to_matrix(d.object_to_world_normal);
    }
}

void attach_scene(Ref_Scene& rs) {
    rs.scene_data.scene_objects = &rs.objects;
    rs.scene_data.kdtrees = &rs.kdtrees;
    rs.scene_data.geometry_type_offsets.fill(0);
}

int cmd_flatten(const Args& a) {
    if (a.pos.size() < 2) return 2;
    Scene scene = load_with_overrides(a);
    Scene_Context ctx;
    init_context(ctx, scene, a);
    yfs::Scene out = flatten(scene, ctx);
    if (!yfs::write(a.pos[1], out)) { fprintf(stderr, "write failed\n"); return 1; }
    return 0;
}

int cmd_render(const Args& a) {
    if (a.pos.size() < 2) return 2;
    Scene scene = load_with_overrides(a);
    Scene_Context ctx;
    init_context(ctx, scene, a);
    double variance = 0.0;
    float seconds = 0.f;
    Image image = render_scene(ctx, &variance, &seconds);
    FILE* f = fopen(a.pos[1].c_str(), "wb");
    if (!f) return 1;
    uint32_t w = (uint32_t)image.width, h = (uint32_t)image.height;
    fwrite(&w, 4, 1, f);
    fwrite(&h, 4, 1, f);
    fwrite(&variance, 8, 1, f);
    fwrite(&seconds, 4, 1, f);
    fwrite(image.data.data(), sizeof(ColorRGB), image.data.size(), f);
    fclose(f);
    printf("{\"render_seconds\": %.6f, \"variance\": %.9g, \"threads\": %d, \"spp\": %d, \"width\": %u, \"height\": %u}\n",
           seconds, variance, a.threads, ctx.pixel_sampler_config.get_samples_per_pixel(), w, h);
    return 0;
}

// build_triangle_mesh_kdtree for every mesh (meshes on `threads` threads) and
// build_scene_kdtree (src/ref/kdtree_builder.cpp:425-463); the trees are also
// copied into the flat scene.
void build_ref_trees(yfs::Scene& fs_scene, Ref_Scene& rs, int thread_count, float* mesh_seconds_out,
                     float* scene_seconds_out) {
    Timestamp t;
    rs.kdtrees.resize(rs.meshes.size());
    std::atomic_int counter{0};
    auto worker = [&] {
        int i = counter.fetch_add(1);
        while (i < (int)rs.meshes.size()) {
            rs.kdtrees[i] = build_triangle_mesh_kdtree(&rs.geometry_data[i]);
            i = counter.fetch_add(1);
        }
    };
    {
        std::vector<std::jthread> threads;
        for (int i = 1; i < std::min<int>(thread_count, (int)rs.meshes.size()); i++) threads.emplace_back(worker);
        worker();
    }
    float mesh_seconds = elapsed_seconds(t);
    attach_scene(rs);
    Timestamp t2;
    rs.scene_kdtree = build_scene_kdtree(&rs.scene_data);
    float scene_seconds = elapsed_seconds(t2);
    for (size_t i = 0; i < rs.meshes.size(); i++) {
        yfs::Mesh& fm = fs_scene.meshes[i];
        const KdTree& kt = rs.kdtrees[i];
        memcpy(fm.bounds, &kt.bounds.min_p.x, 12);
        memcpy(fm.bounds + 3, &kt.bounds.max_p.x, 12);
        fm.nodes.resize(kt.nodes.size());
        memcpy(fm.nodes.data(), kt.nodes.data(), kt.nodes.size() * 8);
    }
    memcpy(fs_scene.scene_bounds, &rs.scene_kdtree.bounds.min_p.x, 12);
    memcpy(fs_scene.scene_bounds + 3, &rs.scene_kdtree.bounds.max_p.x, 12);
    fs_scene.scene_nodes.resize(rs.scene_kdtree.nodes.size());
    memcpy(fs_scene.scene_nodes.data(), rs.scene_kdtree.nodes.data(), rs.scene_kdtree.nodes.size() * 8);
    for (size_t i = 0; i < rs.meshes.size(); i++) rs.kdtrees[i].set_geometry_data(&rs.geometry_data[i]);
    rs.scene_kdtree.set_geometry_data(&rs.scene_data);
    *mesh_seconds_out = mesh_seconds;
    *scene_seconds_out = scene_seconds;
}

int cmd_build(const Args& a) {
    if (a.pos.size() < 2) return 2;
    yfs::Scene fs_scene;
    std::string err;
    if (!yfs::read(a.pos[0], fs_scene, &err)) { fprintf(stderr, "read: %s\n", err.c_str()); return 1; }
    Ref_Scene rs;
    load_ref_meshes(fs_scene, rs);
    float mesh_seconds = 0.f, scene_seconds = 0.f;
    build_ref_trees(fs_scene, rs, a.threads, &mesh_seconds, &scene_seconds);
    if (!yfs::write(a.pos[1], fs_scene)) return 1;
    if (!a.cache_dir.empty()) {  // the reference's own cache files (KdTree::save)
        for (size_t i = 0; i < rs.kdtrees.size(); i++)
            rs.kdtrees[i].save(a.cache_dir + "/mesh_" + std::to_string(i) + ".kdtree");
        rs.scene_kdtree.save(a.cache_dir + "/scene.kdtree");
    }
    printf("{\"mesh_build_seconds\": %.3f, \"scene_build_seconds\": %.3f, \"threads\": %d}\n",
           mesh_seconds, scene_seconds, a.threads);
    return 0;
}

// The kd-trees stored in a flat scene, as reference KdTree objects.
void load_ref_trees(const yfs::Scene& fs_scene, Ref_Scene& rs) {
    rs.kdtrees.resize(rs.meshes.size());
    for (size_t i = 0; i < rs.meshes.size(); i++) {
        KdTree& kt = rs.kdtrees[i];
        const yfs::Mesh& fm = fs_scene.meshes[i];
        kt.bounds = Bounding_Box(Vector3(fm.bounds), Vector3(fm.bounds + 3));
        kt.nodes.resize(fm.nodes.size());
        memcpy(kt.nodes.data(), fm.nodes.data(), fm.nodes.size() * 8);
        kt.set_geometry_data(&rs.geometry_data[i]);
    }
    attach_scene(rs);
    rs.scene_kdtree.bounds = Bounding_Box(Vector3(fs_scene.scene_bounds), Vector3(fs_scene.scene_bounds + 3));
    rs.scene_kdtree.nodes.resize(fs_scene.scene_nodes.size());
    memcpy(rs.scene_kdtree.nodes.data(), fs_scene.scene_nodes.data(), fs_scene.scene_nodes.size() * 8);
    rs.scene_kdtree.set_geometry_data(&rs.scene_data);
}

bool read_file(const std::string& path, std::vector<uint8_t>& raw) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    raw.resize((size_t)size);
    const bool ok = fread(raw.data(), 1, raw.size(), f) == raw.size();
    fclose(f);
    return ok;
}

// Casts a batch of yar_ray records through the scene tree on `thread_count`
// threads (chunks of 4096 rays taken from a shared counter); returns seconds.
struct Cast_Out {
    std::vector<float> t, bary;
    std::vector<uint32_t> prim, obj;
    std::vector<uint8_t> occluded;
};

double cast_rays(const Ref_Scene& rs, const yar_ray* rays, size_t n, bool any, int thread_count, Cast_Out& o) {
    if (any) {
        o.occluded.resize(n);
    } else {
        o.t.resize(n);
        o.bary.resize(2 * n);
        o.prim.resize(n);
        o.obj.resize(n);
    }
    std::vector<float>& t = o.t;
    std::vector<float>& bary = o.bary;
    std::vector<uint32_t>& prim = o.prim;
    std::vector<uint32_t>& obj = o.obj;
    std::vector<uint8_t>& occluded = o.occluded;
    std::atomic<size_t> next{0};
    const size_t chunk = 4096;
    auto worker = [&] {
        initialize_fp_state();
        for (;;) {
            size_t begin = next.fetch_add(chunk);
            if (begin >= n) break;
            size_t end = std::min(n, begin + chunk);
            for (size_t i = begin; i < end; i++) {
                Ray ray{Vector3(rays[i].origin), Vector3(rays[i].direction)};
                if (any) {
                    occluded[i] = rs.scene_kdtree.intersect_any(ray, rays[i].tmax) ? 1 : 0;
                } else {
                    Intersection isect;
                    isect.t = rays[i].tmax;
                    if (rs.scene_kdtree.intersect(ray, isect)) {
                        t[i] = isect.t;
                        prim[i] = isect.triangle_intersection.triangle_index;
                        obj[i] = (uint32_t)(isect.scene_object - rs.objects.data());
                        bary[2 * i] = isect.triangle_intersection.barycentrics.y;
                        bary[2 * i + 1] = isect.triangle_intersection.barycentrics.z;
                    } else {
                        t[i] = rays[i].tmax;
                        prim[i] = 0xffffffffu;
                        obj[i] = 0xffffffffu;
                        bary[2 * i] = 0.f;
                        bary[2 * i + 1] = 0.f;
                    }
                }
            }
        }
    };
    Timestamp ts;
    {
        std::vector<std::jthread> threads;
        for (int i = 1; i < thread_count; i++) threads.emplace_back(worker);
        worker();
    }
    return (double)elapsed_nanoseconds(ts) / 1e9;
}

int cmd_cast(const Args& a) {
    if (a.pos.size() < 3) return 2;
    yfs::Scene fs_scene;
    std::string err;
    if (!yfs::read(a.pos[0], fs_scene, &err)) { fprintf(stderr, "read: %s\n", err.c_str()); return 1; }
    Ref_Scene rs;
    load_ref_meshes(fs_scene, rs);
    load_ref_trees(fs_scene, rs);
    std::vector<uint8_t> raw;
    if (!read_file(a.pos[1], raw)) return 1;
    const size_t n = raw.size() / sizeof(yar_ray);
    const yar_ray* rays = (const yar_ray*)raw.data();
    Cast_Out o;
    double best = 1e30;
    for (int r = 0; r < std::max(1, a.repeat); r++) best = std::min(best, cast_rays(rs, rays, n, a.any, a.threads, o));
    FILE* f = fopen(a.pos[2].c_str(), "wb");
    if (!f) return 1;
    if (a.any) {
        fwrite(o.occluded.data(), 1, n, f);
    } else {
        fwrite(o.t.data(), 4, n, f);
        fwrite(o.prim.data(), 4, n, f);
        fwrite(o.obj.data(), 4, n, f);
        fwrite(o.bary.data(), 4, 2 * n, f);
    }
    fclose(f);
    printf("{\"rays\": %zu, \"seconds\": %.6f, \"threads\": %d, \"kind\": \"%s\"}\n", n, best, a.threads,
           a.any ? "any" : "closest");
    return 0;
}

// bench-cast <in.yfs> <rays.bin> <shadow_rays.bin> [--build] [--threads=T] [--warmup=W] [--steps=K]
// The reference's ray-cast path end to end for the ray-cast benchmark: with
// --build the kd-trees come from the reference's own builder (else from the
// flat scene), then W untimed and K timed steps, each one closest-hit batch
// (KdTree::intersect) and one any-hit batch (KdTree::intersect_any) over all
// rays on T threads.  Prints the build and per-step times.
int cmd_bench_cast(const Args& a) {
    if (a.pos.size() < 3) return 2;
    yfs::Scene fs_scene;
    std::string err;
    if (!yfs::read(a.pos[0], fs_scene, &err)) { fprintf(stderr, "read: %s\n", err.c_str()); return 1; }
    Ref_Scene rs;
    load_ref_meshes(fs_scene, rs);
    float mesh_seconds = 0.f, scene_seconds = 0.f;
    if (a.build) build_ref_trees(fs_scene, rs, a.threads, &mesh_seconds, &scene_seconds);
    else load_ref_trees(fs_scene, rs);
    std::vector<uint8_t> raw_c, raw_a;
    if (!read_file(a.pos[1], raw_c) || !read_file(a.pos[2], raw_a)) return 1;
    const size_t nc = raw_c.size() / sizeof(yar_ray), na = raw_a.size() / sizeof(yar_ray);
    Cast_Out oc, oa;
    for (int w = 0; w < a.warmup; w++) {
        cast_rays(rs, (const yar_ray*)raw_c.data(), nc, false, a.threads, oc);
        cast_rays(rs, (const yar_ray*)raw_a.data(), na, true, a.threads, oa);
    }
    std::string steps;
    for (int s = 0; s < std::max(1, a.steps); s++) {
        const double c = cast_rays(rs, (const yar_ray*)raw_c.data(), nc, false, a.threads, oc);
        const double y = cast_rays(rs, (const yar_ray*)raw_a.data(), na, true, a.threads, oa);
        char buf[96];
        snprintf(buf, sizeof(buf), "%s[%.6f, %.6f]", s ? ", " : "", c, y);
        steps += buf;
    }
    printf("{\"closest_rays\": %zu, \"any_rays\": %zu, \"threads\": %d, \"built\": %s, "
           "\"mesh_build_seconds\": %.3f, \"scene_build_seconds\": %.3f, \"steps\": [%s]}\n",
           nc, na, a.threads, a.build ? "true" : "false", mesh_seconds, scene_seconds, steps.c_str());
    return 0;
}

// regress <mesh.yfs> <out.bin> <ray_count>
// The ray stream of validate_triangle_mesh_kdtree (src/ref/test_kdtree.cpp:20-83,
// :138-194) against a single-mesh flat scene: 25% of the rays restart from the
// previous hit point, axis-aligned directions with probability 1/32 per axis.
// Checks kd-tree t == brute-force t like the reference test and writes
// f32 origin[3], f32 direction[3], f32 t, u32 prim per ray.
// An RGB material parameter of a flat material: its texture slot (1-based,
// with the uv scale) or its constant.
static RGB_Parameter flat_rgb(const float c[3], uint32_t texture, const float uv_scale[2]) {
    RGB_Parameter p;
    if (texture) {
        set_texture_parameter(p, (int)texture - 1);
        p.value.texture.u_scale = uv_scale[0];
        p.value.texture.v_scale = uv_scale[1];
    } else {
        set_constant_parameter(p, ColorRGB(c));
    }
    return p;
}

// The bump map of a flat material: none, a constant height or a texture.
static Float_Parameter flat_bump(const yar_material_desc& d) {
    Float_Parameter p;
    if (d.bump == 1) {
        set_constant_parameter(p, d.bump_height);
    } else if (d.bump == 2) {
        set_texture_parameter(p, (int)d.bump_texture - 1);
        p.value.texture.u_scale = d.bump_uv_scale[0];
        p.value.texture.v_scale = d.bump_uv_scale[1];
    }
    return p;
}

// render-yfs <in.yfs> <out.img> [--threads=T] [--spp=N] [--textures-from=<scene.pbrt>]
// A flat scene (meshes, materials, lights, camera, config) rebuilt as a
// reference Scene, initialised with init_scene_context (reference kd-tree
// builder) and rendered with render_scene.  Used for scenes generated
// without a pbrt file (the large wavefront workload) and for flat scenes
// edited after flattening a pbrt scene: a textured one names that pbrt scene,
// whose texture files the reference loads (its texture indices are the flat
// scene's, as flattening keeps them).
int cmd_render_yfs(const Args& a) {
    if (a.pos.size() < 2) return 2;
    yfs::Scene fs_scene;
    std::string err;
    if (!yfs::read(a.pos[0], fs_scene, &err)) { fprintf(stderr, "read: %s\n", err.c_str()); return 1; }
    if (fs_scene.has_environment) {
        fprintf(stderr, "render-yfs: environment lights are rendered from their pbrt scene only\n");
        return 1;
    }
    Scene texture_source;
    if (!fs_scene.textures.empty()) {
        if (a.textures_from.empty()) {
            fprintf(stderr, "render-yfs: a textured scene needs --textures-from=<the pbrt scene it came from>\n");
            return 1;
        }
        texture_source = load_scene(a.textures_from);
        if (texture_source.texture_descriptors.size() != fs_scene.textures.size()) {
            fprintf(stderr, "render-yfs: %zu textures in the pbrt scene, %zu in the flat scene\n",
                    texture_source.texture_descriptors.size(), fs_scene.textures.size());
            return 1;
        }
    }
    if (fs_scene.other_light_count) {
        fprintf(stderr, "only rectangular, point, spot, directional, triangle-mesh and sphere lights are supported\n");
        return 1;
    }
    Scene scene;
    scene.type = fs_scene.config.pbrt3_scene ? Scene_Type::pbrt : Scene_Type::obj;
    scene.path = a.pos[0];
    if (!fs_scene.textures.empty()) {
        scene.path = a.textures_from;  // texture file names are relative to it
        scene.texture_descriptors = texture_source.texture_descriptors;
    }
    for (const yfs::Mesh& fm : fs_scene.meshes) {
        Triangle_Mesh m;
        m.vertices.resize(fm.vertices.size() / 3);
        memcpy(m.vertices.data(), fm.vertices.data(), fm.vertices.size() * 4);
        m.normals.resize(fm.normals.size() / 3);
        if (!fm.normals.empty()) memcpy(m.normals.data(), fm.normals.data(), fm.normals.size() * 4);
        m.uvs.resize(fm.uvs.size() / 2);
        if (!fm.uvs.empty()) memcpy(m.uvs.data(), fm.uvs.data(), fm.uvs.size() * 4);
        m.indices = fm.indices;
        m.reverse_geometric_normal_orientation = fm.reverse_orientation != 0;
        m.visibility = (Visibility)fm.visibility;
        m.alpha_texture_index = fm.alpha_texture ? (int)fm.alpha_texture - 1 : -1;
        scene.geometries.triangle_meshes.push_back(std::move(m));
    }
    std::vector<Material_Handle> handles;
    for (const yar_material_desc& d : fs_scene.materials) {
        if (d.type == YAR_MATERIAL_DIFFUSE) {
            Diffuse_Material m;
            m.reflectance = flat_rgb(d.reflectance, d.reflectance_texture, d.reflectance_uv_scale);
            m.bump_map = flat_bump(d);
            scene.materials.diffuse.push_back(m);
            handles.push_back({Material_Type::diffuse, (int)scene.materials.diffuse.size() - 1});
        } else if (d.type == YAR_MATERIAL_METAL) {
            Metal_Material m;
            set_constant_parameter(m.u_roughness, d.u_roughness);
            set_constant_parameter(m.v_roughness, d.v_roughness);
            m.roughness_is_alpha = d.roughness_is_alpha != 0;
            set_constant_parameter(m.eta_i, d.eta_i);
            set_constant_parameter(m.eta, ColorRGB(d.eta));
            set_constant_parameter(m.k, ColorRGB(d.k));
            m.bump_map = flat_bump(d);
            scene.materials.metal.push_back(m);
            handles.push_back({Material_Type::metal, (int)scene.materials.metal.size() - 1});
        } else if (d.type == YAR_MATERIAL_GLASS) {
            Glass_Material m;
            m.reflectance = flat_rgb(d.reflectance, d.reflectance_texture, d.reflectance_uv_scale);
            m.transmittance = flat_rgb(d.transmittance, d.transmittance_texture, d.transmittance_uv_scale);
            set_constant_parameter(m.index_of_refraction, d.index_of_refraction);
            set_constant_parameter(m.roughness, d.u_roughness);
            m.roughness_is_alpha = d.roughness_is_alpha != 0;
            m.bump_map = flat_bump(d);
            scene.materials.glass.push_back(m);
            handles.push_back({Material_Type::glass, (int)scene.materials.glass.size() - 1});
        } else if (d.type == YAR_MATERIAL_PLASTIC) {
            Plastic_Material m;
            set_constant_parameter(m.roughness, d.u_roughness);
            m.roughness_is_alpha = d.roughness_is_alpha != 0;
            set_constant_parameter(m.r0, d.transmittance[0]);
            m.diffuse_reflectance = flat_rgb(d.reflectance, d.reflectance_texture, d.reflectance_uv_scale);
            m.bump_map = flat_bump(d);
            scene.materials.plastic.push_back(m);
            handles.push_back({Material_Type::plastic, (int)scene.materials.plastic.size() - 1});
        } else if (d.type == YAR_MATERIAL_COATED_DIFFUSE) {
            Coated_Diffuse_Material m;
            set_constant_parameter(m.u_roughness, d.u_roughness);
            set_constant_parameter(m.v_roughness, d.v_roughness);
            m.roughness_is_alpha = d.roughness_is_alpha != 0;
            set_constant_parameter(m.r0, ColorRGB(d.transmittance));
            m.diffuse_reflectance = flat_rgb(d.reflectance, d.reflectance_texture, d.reflectance_uv_scale);
            m.bump_map = flat_bump(d);
            scene.materials.coated_diffuse.push_back(m);
            handles.push_back({Material_Type::coated_diffuse, (int)scene.materials.coated_diffuse.size() - 1});
        } else if (d.type == YAR_MATERIAL_PERFECT_REFLECTOR) {
            Perfect_Reflector_Material m;
            set_constant_parameter(m.reflectance, ColorRGB(d.reflectance));
            m.bump_map = flat_bump(d);
            scene.materials.perfect_reflector.push_back(m);
            handles.push_back({Material_Type::perfect_reflector, (int)scene.materials.perfect_reflector.size() - 1});
        } else if (d.type == YAR_MATERIAL_PERFECT_REFRACTOR) {
            Perfect_Refractor_Material m;
            set_constant_parameter(m.index_of_refraction, d.index_of_refraction);
            m.bump_map = flat_bump(d);
            scene.materials.perfect_refractor.push_back(m);
            handles.push_back({Material_Type::perfect_refractor, (int)scene.materials.perfect_refractor.size() - 1});
        } else if (d.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) {
            Diffuse_Transmission_Material m;
            m.reflectance = flat_rgb(d.reflectance, d.reflectance_texture, d.reflectance_uv_scale);
            m.transmittance = flat_rgb(d.transmittance, d.transmittance_texture, d.transmittance_uv_scale);
            set_constant_parameter(m.scale, ColorRGB(d.diffuse));
            m.bump_map = flat_bump(d);
            scene.materials.diffuse_transmission.push_back(m);
            handles.push_back({Material_Type::diffuse_transmission,
                               (int)scene.materials.diffuse_transmission.size() - 1});
        } else if (d.type == YAR_MATERIAL_PBRT3_TRANSLUCENT) {
            Pbrt3_Translucent_Material m;
            set_constant_parameter(m.reflectance, ColorRGB(d.reflectance));
            set_constant_parameter(m.transmittance, ColorRGB(d.transmittance));
            set_constant_parameter(m.diffuse, ColorRGB(d.diffuse));
            set_constant_parameter(m.specular, ColorRGB(d.specular));
            set_constant_parameter(m.roughness, d.u_roughness);
            m.bump_map = flat_bump(d);
            scene.materials.pbrt3_translucent.push_back(m);
            handles.push_back({Material_Type::pbrt3_translucent, (int)scene.materials.pbrt3_translucent.size() - 1});
        } else if (d.type == YAR_MATERIAL_PBRT3_UBER) {
            Pbrt3_Uber_Material m;
            set_constant_parameter(m.diffuse_reflectance, ColorRGB(d.reflectance));
            set_constant_parameter(m.specular_reflectance, ColorRGB(d.specular));
            set_constant_parameter(m.delta_reflectance, ColorRGB(d.delta_reflectance));
            set_constant_parameter(m.delta_transmission, ColorRGB(d.transmittance));
            set_constant_parameter(m.opacity, ColorRGB(d.opacity));
            set_constant_parameter(m.u_roughness, d.u_roughness);
            set_constant_parameter(m.v_roughness, d.v_roughness);
            set_constant_parameter(m.index_of_refraction, d.index_of_refraction);
            m.bump_map = flat_bump(d);
            m.component_count = (uint8_t)d.component_count;
            for (uint32_t k = 0; k < d.component_count && k < 5; k++)
                m.components[k] = (Pbrt3_Uber_Material::Component_Type)d.components[k];
            scene.materials.pbrt3_uber.push_back(m);
            handles.push_back({Material_Type::pbrt3_uber, (int)scene.materials.pbrt3_uber.size() - 1});
        } else if (d.type == YAR_MATERIAL_PBRT3_FOURIER) {
            // the table as load_bsdf_file leaves it (src/lib/material_pbrt.cpp:24-102)
            if (d.fourier_table == 0 || d.fourier_table > fs_scene.fourier_tables.size()) {
                fprintf(stderr, "fourier material without a table\n");
                return 1;
            }
            const yar_fourier_desc& t = fs_scene.fourier_tables[d.fourier_table - 1];
            const uint64_t pairs = (uint64_t)t.node_count * t.node_count;
            if (t.nodes + t.node_count > fs_scene.fourier_floats.size() ||
                t.coeffs + t.coeff_count > fs_scene.fourier_floats.size() ||
                t.series + 2 * pairs > fs_scene.fourier_uints.size()) {
                fprintf(stderr, "fourier table out of range\n");
                return 1;
            }
            Pbrt3_Fourier_Material m;
            m.max_order = t.max_order;
            m.channel_count = t.channel_count;
            m.eta = t.eta;
            const float* ff = fs_scene.fourier_floats.data();
            m.zenith_angle_discretization.assign(ff + t.nodes, ff + t.nodes + t.node_count);
            m.coeffs.assign(ff + t.coeffs, ff + t.coeffs + t.coeff_count);
            m.coeff_offset.resize(pairs);
            m.coeff_count.resize(pairs);
            m.first_coeffs.resize(pairs);
            for (uint64_t k = 0; k < pairs; k++) {
                m.coeff_offset[k] = fs_scene.fourier_uints[t.series + 2 * k];
                m.coeff_count[k] = fs_scene.fourier_uints[t.series + 2 * k + 1];
                m.first_coeffs[k] = m.coeff_count[k] > 0 ? m.coeffs[m.coeff_offset[k]] : 0.f;
            }
            scene.materials.pbrt3_fourier.push_back(m);
            handles.push_back({Material_Type::pbrt3_fourier, (int)scene.materials.pbrt3_fourier.size() - 1});
        } else if (d.type == YAR_MATERIAL_MIX) {
            scene.materials.mix.push_back(Mix_Material{});  // sub-materials below, once every handle exists
            handles.push_back({Material_Type::mix, (int)scene.materials.mix.size() - 1});
        } else {
            fprintf(stderr, "unsupported material type %u\n", d.type);
            return 1;
        }
    }
    for (size_t i = 0; i < fs_scene.materials.size(); i++) {
        const yar_material_desc& d = fs_scene.materials[i];
        if (d.type != YAR_MATERIAL_MIX) continue;
        for (int k = 0; k < 2; k++)
            if (d.mix_materials[k] < 0 || (size_t)d.mix_materials[k] >= handles.size()) {
                fprintf(stderr, "mix material %zu: bad sub-material\n", i);
                return 1;
            }
        Mix_Material& m = scene.materials.mix[handles[i].index];
        m.material1 = handles[d.mix_materials[0]];
        m.material2 = handles[d.mix_materials[1]];
        set_constant_parameter(m.mix_amount, ColorRGB(d.mix_amount));
    }
    for (const yar_rect_light_desc& d : fs_scene.rect_lights) {
        Diffuse_Rectangular_Light l;
        l.light_to_world_transform = floats_to_matrix(d.light_to_world);
        l.emitted_radiance = ColorRGB(d.emitted_radiance);
        l.size = Vector2(d.size[0], d.size[1]);
        l.sample_count = d.sample_count;
        scene.lights.diffuse_rectangular_lights.push_back(l);
    }
    for (const yar_delta_light_desc& d : fs_scene.delta_lights) {
        if (d.type == YAR_LIGHT_POINT) {
            Point_Light l;
            l.position = Vector3(d.position);
            l.intensity = ColorRGB(d.intensity);
            scene.lights.point_lights.push_back(l);
        } else if (d.type == YAR_LIGHT_SPOT) {
            Spot_Light l;
            l.position = Vector3(d.position);
            l.direction = Vector3(d.direction);
            l.intensity = ColorRGB(d.intensity);
            l.cone_angle = d.cone_angle;
            l.penumbra_angle = d.penumbra_angle;
            scene.lights.spot_lights.push_back(l);
        } else if (d.type == YAR_LIGHT_DIRECTIONAL) {
            Directional_Light l;
            l.direction = Vector3(d.direction);
            l.irradiance = ColorRGB(d.intensity);
            scene.lights.directional_lights.push_back(l);
        } else {
            fprintf(stderr, "unsupported light type %u\n", d.type);
            return 1;
        }
    }
    for (const yar_sphere_light_desc& d : fs_scene.sphere_lights) {
        Diffuse_Sphere_Light l;
        l.position = Vector3(d.position);
        l.emitted_radiance = ColorRGB(d.emitted_radiance);
        l.radius = d.radius;
        l.sample_count = d.sample_count;
        scene.lights.diffuse_sphere_lights.push_back(l);
    }
    for (const yar_mesh_light_desc& d : fs_scene.mesh_lights) {
        Diffuse_Triangle_Mesh_Light l;
        l.light_to_world_transform = floats_to_matrix(d.light_to_world);
        l.emitted_radiance = ColorRGB(d.emitted_radiance);
        l.triangle_mesh_index = d.triangle_mesh_index;
        scene.lights.diffuse_triangle_mesh_lights.push_back(l);
    }
    scene.lights.update_total_light_count();
    for (const yar_object_desc& d : fs_scene.objects) {
        Scene_Object o;
        o.geometry = {Geometry_Type::triangle_mesh, d.mesh_index};
        o.material = d.material_index >= 0 ? handles[d.material_index] : Null_Material;
        o.area_light = {(Light_Type)d.area_light_type, d.area_light_index};
        o.object_to_world_transform = floats_to_matrix(d.object_to_world);
        o.world_to_object_transform = floats_to_matrix(d.world_to_object);
        o.object_to_world_normal_transform = floats_to_matrix(d.object_to_world_normal);
        scene.objects.push_back(o);
    }
    const yar_render_config& c = fs_scene.config;
    scene.film_resolution = Vector2i{(int)fs_scene.camera.image_extent[0], (int)fs_scene.camera.image_extent[1]};
    scene.render_region = Bounds2i{{c.render_region[0], c.render_region[1]}, {c.render_region[2], c.render_region[3]}};
    scene.camera_fov_y = 40.f;  // replaced by the flat scene's exact camera below
    scene.z_is_up = fs_scene.camera.z_is_up != 0;
    scene.view_points = {floats_to_matrix(fs_scene.camera.camera_to_world)};
    Raytracer_Config& rc = scene.raytracer_config;
    rc.rendering_algorithm = (Raytracer_Config::Rendering_Algorithm)c.rendering_algorithm;
    rc.max_light_bounces = c.max_light_bounces;
    rc.russian_roulette_threshold = c.russian_roulette_threshold;
    rc.russian_roulette_bounce_count_threshold = c.russian_roulette_bounce_count_threshold;
    rc.pixel_filter_type = (Raytracer_Config::Pixel_Filter_Type)c.pixel_filter_type;
    rc.pixel_filter_radius = c.pixel_filter_radius;
    rc.pixel_filter_alpha = c.pixel_filter_alpha;
    rc.x_pixel_sample_count = c.x_pixel_sample_count;
    rc.y_pixel_sample_count = c.y_pixel_sample_count;
    if (a.spp > 0) {
        int k = (int)std::ceil(std::sqrt(a.spp));
        rc.x_pixel_sample_count = k;
        rc.y_pixel_sample_count = k;
    }
    rc.film_radiance_scale = c.film_radiance_scale;
    rc.max_rgb_component_value_of_film_sample = c.max_rgb_component_value_of_film_sample;
    Args b = a;
    b.seed_offset = c.rng_seed_offset;
    Scene_Context ctx;
    init_context(ctx, scene, b);
    ctx.camera.camera_to_world = floats_to_matrix(fs_scene.camera.camera_to_world);
    ctx.camera.image_extent = Vector2(fs_scene.camera.image_extent[0], fs_scene.camera.image_extent[1]);
    ctx.camera.horz_half_dist = fs_scene.camera.horz_half_dist;
    ctx.camera.vert_half_dist = fs_scene.camera.vert_half_dist;
    ctx.camera.z_is_up = fs_scene.camera.z_is_up != 0;
    double variance = 0.0;
    float seconds = 0.f;
    Image image = render_scene(ctx, &variance, &seconds);
    FILE* f = fopen(a.pos[1].c_str(), "wb");
    if (!f) return 1;
    uint32_t w = (uint32_t)image.width, h = (uint32_t)image.height;
    fwrite(&w, 4, 1, f);
    fwrite(&h, 4, 1, f);
    fwrite(&variance, 8, 1, f);
    fwrite(&seconds, 4, 1, f);
    fwrite(image.data.data(), sizeof(ColorRGB), image.data.size(), f);
    fclose(f);
    printf("{\"render_seconds\": %.6f, \"variance\": %.9g, \"threads\": %d, \"spp\": %d, \"width\": %u, \"height\": %u}\n",
           seconds, variance, b.threads, ctx.pixel_sampler_config.get_samples_per_pixel(), w, h);
    return 0;
}

int cmd_regress(const Args& a) {
    if (a.pos.size() < 3) return 2;
    yfs::Scene fs_scene;
    std::string err;
    if (!yfs::read(a.pos[0], fs_scene, &err) || fs_scene.meshes.empty()) return 1;
    Ref_Scene rs;
    load_ref_meshes(fs_scene, rs);
    Triangle_Mesh_Geometry_Data& gd = rs.geometry_data[0];
    KdTree kdtree = build_triangle_mesh_kdtree(&gd);
    const int count = atoi(a.pos[2].c_str());

    RNG rng;
    Vector3 diagonal = kdtree.bounds.max_p - kdtree.bounds.min_p;
    float delta = 2.0f * diagonal.length();
    Bounding_Box ray_bounds(kdtree.bounds.min_p - Vector3(delta), kdtree.bounds.max_p + Vector3(delta));
    Vector3 last_hit_position = (kdtree.bounds.min_p + kdtree.bounds.max_p) * 0.5f;
    Vector3 last_hit_normal = Vector3(1, 0, 0);
    FILE* f = fopen(a.pos[1].c_str(), "wb");
    if (!f) return 1;
    int mismatches = 0;
    for (int i = 0; i < count; i++) {
        Vector3 origin, direction;
        if (rng.get_float() < 0.25f) {
            origin = last_hit_position;
            direction = sample_hemisphere_uniform(rng.get_vector2());
            Vector3 axis_a, axis_b;
            coordinate_system_from_vector(last_hit_normal, &axis_a, &axis_b);
            Matrix3x4 m = Matrix3x4::identity;
            m.set_column(0, axis_a);
            m.set_column(1, axis_b);
            m.set_column(2, last_hit_normal);
            direction = transform_vector(m, direction);
        } else {
            auto range = [&rng](float lo, float hi) { return lo + (hi - lo) * rng.get_float(); };
            origin.x = range(ray_bounds.min_p.x, ray_bounds.max_p.x);
            origin.y = range(ray_bounds.min_p.y, ray_bounds.max_p.y);
            origin.z = range(ray_bounds.min_p.z, ray_bounds.max_p.z);
            direction = sample_sphere_uniform(rng.get_vector2());
            if (rng.get_float() < 1.0f / 32.0f && direction.z != 0.0) direction.x = direction.y = 0.0;
            else if (rng.get_float() < 1.0f / 32.0f && direction.y != 0.0) direction.x = direction.z = 0.0;
            else if (rng.get_float() < 1.0f / 32.0f && direction.x != 0.0) direction.y = direction.z = 0.0;
            direction = direction.normalized();
        }
        Ray ray{origin, direction};
        Intersection isect;
        kdtree.intersect(ray, isect);
        Intersection brute;
        const Triangle_Mesh& mesh = rs.meshes[0];
        for (int k = 0; k < mesh.get_triangle_count(); k++) kdtree.intersector(ray, kdtree.geometry_data, k, brute);
        if (isect.t != brute.t) mismatches++;
        uint32_t prim = isect.t != Infinity ? isect.triangle_intersection.triangle_index : 0xffffffffu;
        fwrite(&origin.x, 4, 3, f);
        fwrite(&direction.x, 4, 3, f);
        fwrite(&isect.t, 4, 1, f);
        fwrite(&prim, 4, 1, f);
        if (isect.t != Infinity) {
            const Triangle_Intersection& ti = isect.triangle_intersection;
            Vector3 hit_pos = ti.mesh->get_position(ti.triangle_index, ti.barycentrics);
            Vector3 p[3];
            ti.mesh->get_positions(ti.triangle_index, p);
            Vector3 ng = cross(p[1] - p[0], p[2] - p[0]).normalized();
            ng = dot(ng, -ray.direction) < 0 ? -ng : ng;
            last_hit_position = offset_ray_origin(hit_pos, ng);
            last_hit_normal = ng;
        }
    }
    fclose(f);
    printf("{\"rays\": %d, \"kdtree_vs_brute_force_mismatches\": %d}\n", count, mismatches);
    return 0;
}

// exr <image.f32> <width> <height> <out.exr> [--spp=N] [--variance=V] [--compress]
// The reference's write_openexr_image (reference_renderer.cpp:673-705) on a
// raw float RGB image: the golden files of the EXR writer's parity test.
int cmd_exr(const Args& a) {
    if (a.pos.size() < 4) return 2;
    const int w = atoi(a.pos[1].c_str()), h = atoi(a.pos[2].c_str());
    Image img(w, h);
    FILE* f = fopen(a.pos[0].c_str(), "rb");
    if (!f) return 1;
    const size_t got = fread(&img.data[0].r, sizeof(float), (size_t)w * h * 3, f);
    fclose(f);
    if (got != (size_t)w * h * 3) return 1;
    EXR_Write_Params params;
    params.enable_compression = a.compress;
    params.attributes.input_file = a.input_file;
    params.attributes.spp = a.spp;
    params.attributes.variance = a.variance;
    return write_openexr_image(a.pos[3], img, params) ? 0 : 1;
}

} // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: yar_ref flatten|render|build|cast ...\n");
        return 2;
    }
    Args a = parse(argc, argv);
    std::string cmd = argv[1];
    int rc = 2;
    if (cmd == "flatten") rc = cmd_flatten(a);
    else if (cmd == "render") rc = cmd_render(a);
    else if (cmd == "build") rc = cmd_build(a);
    else if (cmd == "cast") rc = cmd_cast(a);
    else if (cmd == "bench-cast") rc = cmd_bench_cast(a);
    else if (cmd == "regress") rc = cmd_regress(a);
    else if (cmd == "render-yfs") rc = cmd_render_yfs(a);
    else if (cmd == "exr") rc = cmd_exr(a);
    if (rc == 2) fprintf(stderr, "bad arguments for %s\n", cmd.c_str());
    return rc;
}
