/*
 * yar_gpu.h - C ABI of the GB300 (sm_103a) path-tracing hot path.
 *
 * This is the drop-in boundary for the CPU reference renderer of
 * kennyalive/YAR.  The reference has no C ABI: its seams are C++ functions,
 * and every entry point below names the function it replaces:
 *
 *   yar_gpu_cast_closest  <- bool KdTree::intersect(const Ray&, Intersection&) const
 *                            src/ref/kdtree.h:116, src/ref/kdtree.cpp:219-327
 *   yar_gpu_cast_any      <- bool KdTree::intersect_any(const Ray&, float tmax) const
 *                            src/ref/kdtree.h:117, src/ref/kdtree.cpp:329-439
 *   yar_gpu_upload_scene  <- init_scene_context(Scene_Context&, const Scene&, ...)
 *                            src/ref/reference_renderer.h:48-53 (the device-side part:
 *                            kd-trees, meshes, objects, materials, lights, camera)
 *   yar_gpu_render        <- Image render_scene(const Scene_Context&, double* variance,
 *                            float* render_time)  src/ref/reference_renderer.h:55
 *   yar_build_mesh_kdtree <- KdTree build_triangle_mesh_kdtree(const Triangle_Mesh_Geometry_Data*)
 *                            src/ref/kdtree_builder.h:6, src/ref/kdtree_builder.cpp:425-441
 *   yar_build_scene_kdtree<- KdTree build_scene_kdtree(const Scene_Geometry_Data*)
 *                            src/ref/kdtree_builder.h:10, src/ref/kdtree_builder.cpp:443-463
 *
 * Conventions
 *   - Plain pointers and sizes only.  Every function returns a status code
 *     (YAR_OK == 0, negative on error) and never exits the process; the
 *     reference calls exit(1) from error() (src/lib/common.cpp:10-28).
 *   - Matrices are 3x4 row-major floats, the layout of Matrix3x4::a[3][4]
 *     (src/lib/matrix.h:7-20).
 *   - kd-tree nodes are the reference's 8-byte KdNode words (src/ref/kdtree.h:18-77),
 *     bit for bit: interior word0 = axis | above_child << 2, word1 = split bits;
 *     leaf word0 = 3 | count << 2, word1.. = sorted primitive indices.
 *   - Enumerations reuse the reference's numeric values: Material_Type
 *     (src/lib/material.h:6-21) and Light_Type (src/lib/light.h:7-17).
 *   - A context owns one CUDA stream and its device memory.  A context is not
 *     thread-safe; separate contexts are independent.
 */
#ifndef YAR_GPU_H
#define YAR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YAR_GPU_ABI_VERSION 1

/* status codes */
#define YAR_OK                 0
#define YAR_ERR_INVALID       -1  /* bad argument or malformed scene */
#define YAR_ERR_NOMEM         -2  /* device or host allocation failed */
#define YAR_ERR_CAPACITY      -3  /* a fixed capacity (stack depth, queue) was exceeded */
#define YAR_ERR_TIMEOUT       -4  /* a bounded device wait gave up */
#define YAR_ERR_CUDA          -5  /* CUDA runtime error (see yar_gpu_last_error) */
#define YAR_ERR_UNSUPPORTED   -6  /* scene feature outside the implemented path */
#define YAR_ERR_IO            -7  /* file read/write failure */
#define YAR_ERR_NO_SCENE      -8  /* no scene uploaded */

/* buffer residency flags for the ray-cast entry points */
#define YAR_BUFFERS_HOST    0   /* pointers are host memory; copies happen inside the call */
#define YAR_BUFFERS_DEVICE  1   /* pointers are device memory of the context's device */

/* Material_Type values (src/lib/material.h:6-21) */
#define YAR_MATERIAL_PERFECT_REFLECTOR 0
#define YAR_MATERIAL_PERFECT_REFRACTOR 1
#define YAR_MATERIAL_DIFFUSE           2
#define YAR_MATERIAL_DIFFUSE_TRANSMISSION 3
#define YAR_MATERIAL_METAL             4
#define YAR_MATERIAL_PLASTIC           5
#define YAR_MATERIAL_COATED_DIFFUSE    6
#define YAR_MATERIAL_GLASS             7
#define YAR_MATERIAL_MIX               8
#define YAR_MATERIAL_PBRT3_UBER        9
#define YAR_MATERIAL_PBRT3_TRANSLUCENT 10
#define YAR_MATERIAL_PBRT3_FOURIER     11
#define YAR_MATERIAL_NULL              0xffffffffu

/* Light_Type values (src/lib/light.h:7-17) */
#define YAR_LIGHT_POINT                0
#define YAR_LIGHT_SPOT                 1
#define YAR_LIGHT_DIRECTIONAL          2
#define YAR_LIGHT_DIFFUSE_RECTANGULAR  3
#define YAR_LIGHT_DIFFUSE_SPHERE       4
#define YAR_LIGHT_DIFFUSE_TRIANGLE_MESH 5
#define YAR_LIGHT_ENVIRONMENT_MAP      6
#define YAR_LIGHT_NULL                 0xffffffffu

/* Visibility (src/lib/triangle_mesh.h:7-11) */
#define YAR_VISIBLE            0
#define YAR_VISIBLE_NO_SHADOWS 1
#define YAR_INVISIBLE          2

typedef struct yar_gpu_ctx yar_gpu_ctx;

/* KdNode, src/ref/kdtree.h:18-77 */
typedef struct yar_kd_node {
    uint32_t word0;
    uint32_t word1;
} yar_kd_node;

/* KdTree::bounds + KdTree::nodes, src/ref/kdtree.h:119-126 */
typedef struct yar_kdtree_view {
    float bounds_min[3];
    float bounds_max[3];
    const yar_kd_node* nodes;
    uint32_t node_count;
} yar_kdtree_view;

/* Triangle_Mesh, src/lib/triangle_mesh.h:13-131 */
typedef struct yar_mesh_desc {
    const float* vertices;      /* float3 x vertex_count */
    const float* normals;       /* float3 x vertex_count, or NULL */
    const float* uvs;           /* float2 x vertex_count, or NULL */
    const int32_t* indices;     /* int3 x triangle_count */
    uint32_t vertex_count;
    uint32_t triangle_count;
    int32_t reverse_geometric_normal_orientation;
    int32_t visibility;         /* YAR_VISIBLE, ... */
    yar_kdtree_view kdtree;     /* per-mesh tree (object space) */
    /* Alpha test (src/ref/kdtree.cpp:31-38, :69-77): 0 none, else 1 + an index
     * into yar_flat_scene::textures.  A triangle hit whose texture value at
     * the hit's uv (mip 0, bilinear, repeat) has red 0 is skipped by both
     * casts.  Needs uvs. */
    uint32_t alpha_texture;
} yar_mesh_desc;

/* Scene_Object, src/lib/scene_object.h:8-25 */
typedef struct yar_object_desc {
    int32_t mesh_index;
    uint32_t material_type;     /* YAR_MATERIAL_* (YAR_MATERIAL_NULL for lights) */
    int32_t material_index;     /* index into yar_flat_scene::materials */
    uint32_t area_light_type;   /* YAR_LIGHT_* */
    int32_t area_light_index;
    float object_to_world[12];
    float world_to_object[12];
    float object_to_world_normal[12];
} yar_object_desc;

/* Constant-parameter materials (Perfect_Reflector/Perfect_Refractor/Diffuse/Metal/
 * Plastic/Coated_Diffuse/Glass_Material, src/lib/material.h:48-150).  Glass with
 * roughness 0 scatters as the reference's smooth (delta) glass; plastic in a scene
 * with pbrt3_scene set is shaded as pbrt-v3's plastic, as the reference does.
 * Image textures on the reflectance and transmittance slots and bump maps are
 * evaluated by yar_gpu_render (both rendering algorithms),
 * yar_gpu_render_checkpoint, yar_gpu_render_batch and yar_gpu_guided_render,
 * behind delta bounces too; the static render, and textures on any other
 * parameter, return YAR_ERR_UNSUPPORTED. */
typedef struct yar_material_desc {
    uint32_t type;              /* YAR_MATERIAL_PERFECT_REFLECTOR / PERFECT_REFRACTOR / DIFFUSE / METAL /
                                   PLASTIC / COATED_DIFFUSE / GLASS */
    float reflectance[3];       /* perfect reflector: reflectance; diffuse, plastic, coated diffuse:
                                   diffuse reflectance; glass: reflectance (kr) */
    float transmittance[3];     /* glass: transmittance (kt); plastic, coated diffuse: specular r0
                                   (plastic: all three equal) */
    float eta[3];               /* metal */
    float k[3];                 /* metal */
    float eta_i;                /* metal: IOR of the adjacent dielectric */
    float u_roughness;          /* metal, coated diffuse: u roughness; glass, plastic: roughness */
    float v_roughness;          /* metal, coated diffuse (plastic: = u_roughness) */
    float index_of_refraction;  /* glass, perfect refractor, pbrt3 uber */
    int32_t roughness_is_alpha;
    /* Fields of the layered and mixed materials (zero for the other kinds). */
    float specular[3];          /* pbrt3 uber, pbrt3 translucent: Ks */
    float diffuse[3];           /* pbrt3 translucent: Kd; diffuse transmission: scale */
    float delta_reflectance[3]; /* pbrt3 uber: Kr */
    float opacity[3];           /* pbrt3 uber */
    uint32_t component_count;   /* pbrt3 uber: its layers (YAR_UBER_*) in the reference's order */
    uint32_t components[5];
    int32_t mix_materials[2];   /* mix: the two materials, indices into yar_flat_scene::materials */
    float mix_amount[3];        /* mix */
    /* Image textures (RGB_Parameter in value mode with a texture leaf,
       src/lib/material_parameter.h): the texture of `reflectance` and its uv
       scale.  0: the constant above; k > 0: yar_flat_scene::textures[k - 1].
       `reflectance` is the diffuse reflectance of diffuse, plastic and coated
       diffuse materials, Kr of glass, the reflectance of diffuse transmission. */
    uint32_t reflectance_texture;
    float reflectance_uv_scale[2];
    uint32_t other_textured_parameters;  /* parameters given by textures the library does not evaluate */
    /* the texture of `transmittance` (Kt of glass, the transmittance of
       diffuse transmission), as reflectance_texture */
    uint32_t transmittance_texture;
    float transmittance_uv_scale[2];
    /* Bump map (Float_Parameter, applied by Shading_Context::apply_bump_map,
       src/ref/shading_context.cpp:419-462): 0 none, 1 the constant height
       bump_height, 2 the luminance of texture bump_texture (1 + index) at uv x
       bump_uv_scale. */
    uint32_t bump;
    float bump_height;
    uint32_t bump_texture;
    float bump_uv_scale[2];
    /* pbrt3 fourier: 1 + the index of its table in yar_flat_scene::fourier_tables */
    uint32_t fourier_table;
} yar_material_desc;

/* Image_Texture (src/ref/image_texture.h) as the reference builds it from the
 * file: the base level (scaled, decoded from sRGB, upsampled to powers of two)
 * and its mip chain.  Mips are listed level 0 first in
 * yar_flat_scene::texture_mips; texels are RGB float triples, row 0 first. */
typedef struct yar_texture_desc {
    uint32_t first_mip;   /* index into texture_mips */
    uint32_t mip_count;
} yar_texture_desc;

typedef struct yar_texture_mip_desc {
    uint32_t width, height;   /* powers of two */
    uint64_t texel_offset;    /* into yar_flat_scene::texels, in texels (3 floats each) */
} yar_texture_mip_desc;

/* Pbrt3_Uber_Material component kinds (src/lib/material_pbrt.h) */
#define YAR_UBER_DIFFUSE            0
#define YAR_UBER_SPECULAR           1
#define YAR_UBER_DELTA_REFLECTION   2
#define YAR_UBER_DELTA_TRANSMISSION 3
#define YAR_UBER_OPACITY            4

/* Diffuse_Rectangular_Light, src/lib/light.h:66-73 */
typedef struct yar_rect_light_desc {
    float light_to_world[12];
    float emitted_radiance[3];
    float size[2];
    int32_t sample_count;
} yar_rect_light_desc;

/* Point_Light, Spot_Light and Directional_Light (src/lib/light.h:35-64) in one
 * record: the lights without geometry, which are sampled but never hit.  A scene
 * lists them in the reference's selection order (src/ref/direct_lighting.cpp:
 * 522-547): all point lights, then all spot lights, then all directional lights. */
typedef struct yar_delta_light_desc {
    uint32_t type;              /* YAR_LIGHT_POINT / SPOT / DIRECTIONAL */
    float position[3];          /* point, spot */
    float direction[3];         /* spot: the cone axis; directional: towards the light */
    float intensity[3];         /* point, spot: intensity; directional: irradiance */
    float cone_angle;           /* spot, radians */
    float penumbra_angle;       /* spot, radians */
} yar_delta_light_desc;

/* Diffuse_Sphere_Light, src/lib/light.h:75-80: sampled over the cone it
 * subtends (Diffuse_Sphere_Light_Sampler, src/ref/light_sampling.cpp:76-123);
 * the scene object that shows it (a tessellated sphere) carries
 * YAR_LIGHT_DIFFUSE_SPHERE with this light's index. */
typedef struct yar_sphere_light_desc {
    float position[3];
    float emitted_radiance[3];
    float radius;
    int32_t sample_count;
} yar_sphere_light_desc;

/* Diffuse_Triangle_Mesh_Light, src/lib/light.h:82-86: a one-sided emitting
 * mesh.  It is sampled in proportion to triangle area over the mesh's own
 * vertices (Diffuse_Triangle_Mesh_Light_Sampler, src/ref/light_sampling.cpp:
 * 126-184), and the scene object that shows it carries
 * YAR_LIGHT_DIFFUSE_TRIANGLE_MESH with this light's index. */
typedef struct yar_mesh_light_desc {
    float light_to_world[12];
    float emitted_radiance[3];
    uint32_t triangle_mesh_index;  /* into yar_flat_scene::meshes */
} yar_mesh_light_desc;

/* Environment_Light (src/lib/light.h:88-94) with its latitude-longitude map as
 * the reference sees it: the texture's mip 0 (a constant light is a 1 x 1 map).
 * Sampled by Environment_Light_Sampler (src/ref/light_sampling.cpp:29-71). */
typedef struct yar_environment_desc {
    float light_to_world[12];
    float world_to_light[12];
    float scale[3];
    int32_t sample_count;
    uint32_t width, height;
    const float* radiance;      /* width * height RGB triples, row 0 first */
} yar_environment_desc;

/* A pbrt3 fourier BSDF table (Pbrt3_Fourier_Material, src/lib/material_pbrt.h:4-38,
 * as Pbrt3_Fourier_Material::load_bsdf_file reads a layerlab file): the
 * zenith-angle cosines, increasing, the last at least 1; per pair of nodes
 * (outgoing-major) the offset and length of its Fourier series; the
 * coefficients, channel-major within a series (Y, then R and B for three
 * channels).  Offsets index the flat scene's fourier_floats / fourier_uints. */
typedef struct yar_fourier_desc {
    uint32_t node_count;
    uint32_t channel_count;     /* 1 or 3 */
    uint32_t max_order;
    float eta;                  /* relative IOR; the reference evaluates reflection only (eta 1) */
    uint64_t nodes;             /* fourier_floats offset of node_count cosines */
    uint64_t coeffs;            /* fourier_floats offset of the coefficients */
    uint64_t coeff_count;       /* coefficients of this table */
    uint64_t series;            /* fourier_uints offset of node_count^2 (offset into coeffs, length) pairs */
} yar_fourier_desc;

/* Camera, src/ref/camera.h:35-49 (fields as computed by Camera::Camera, camera.cpp:5-14) */
typedef struct yar_camera_desc {
    float camera_to_world[12];
    float image_extent[2];
    float horz_half_dist;
    float vert_half_dist;
    int32_t z_is_up;
} yar_camera_desc;

/* Raytracer_Config (src/lib/raytracer_config.h:5-49) plus the Scene_Context
 * fields the render loop reads (render_region, rng_seed_offset, pbrt3_scene). */
typedef struct yar_render_config {
    int32_t render_region[4];       /* x0, y0, x1, y1 (x1/y1 exclusive) */
    int32_t rendering_algorithm;    /* 0 direct lighting, 1 path tracer */
    int32_t max_light_bounces;
    float russian_roulette_threshold;
    int32_t russian_roulette_bounce_count_threshold;
    int32_t pixel_filter_type;      /* 0 box, 1 gaussian, 2 triangle */
    float pixel_filter_radius;
    float pixel_filter_alpha;
    int32_t x_pixel_sample_count;
    int32_t y_pixel_sample_count;
    float film_radiance_scale;
    float max_rgb_component_value_of_film_sample;
    int32_t pbrt3_scene;            /* roughness remap: 1 pbrt3 polynomial, 0 alpha = r^2 */
    int32_t rng_seed_offset;
} yar_render_config;

typedef struct yar_flat_scene {
    uint32_t mesh_count;
    const yar_mesh_desc* meshes;
    uint32_t object_count;
    const yar_object_desc* objects;
    yar_kdtree_view scene_kdtree;   /* over objects (world space) */
    uint32_t material_count;
    const yar_material_desc* materials;
    uint32_t rect_light_count;
    const yar_rect_light_desc* rect_lights;
    /* lights the library does not carry: counted for total_light_count;
       rendering with any of them is unsupported */
    uint32_t other_light_count;
    yar_camera_desc camera;
    yar_render_config config;
    uint32_t delta_light_count;     /* point, spot and directional lights */
    const yar_delta_light_desc* delta_lights;
    uint32_t mesh_light_count;      /* triangle-mesh lights */
    const yar_mesh_light_desc* mesh_lights;
    uint32_t sphere_light_count;    /* sphere lights */
    const yar_sphere_light_desc* sphere_lights;
    const yar_environment_desc* environment;  /* NULL: no environment light */
    uint32_t texture_count;         /* image textures */
    const yar_texture_desc* textures;
    uint32_t texture_mip_count;
    const yar_texture_mip_desc* texture_mips;
    const float* texels;            /* RGB triples of every mip */
    uint64_t texel_count;           /* texels (RGB triples) behind `texels`; every mip must lie inside */
    uint32_t fourier_count;         /* pbrt3 fourier BSDF tables */
    const yar_fourier_desc* fourier_tables;
    uint64_t fourier_float_count;
    const float* fourier_floats;
    uint64_t fourier_uint_count;
    const uint32_t* fourier_uints;
} yar_flat_scene;

/* One ray of a batch: 32 bytes, two float4.  tmax plays the role of the
 * initial Intersection::t (src/ref/intersection.h:17-19) for closest hit and
 * of ray_tmax for any hit. */
typedef struct yar_ray {
    float origin[3];
    float tmax;
    float direction[3];
    float pad;
} yar_ray;

/* Closest-hit results, structure of arrays; any pointer may be NULL.
 * t = Intersection::t (tmax when there is no hit), prim = triangle index
 * within its mesh (0xffffffff when no hit), object = Scene_Object index,
 * bary = barycentrics y,z (x = 1 - y - z is not stored). */
typedef struct yar_hit_soa {
    float* t;
    uint32_t* prim;
    uint32_t* object;
    float* bary;        /* float2 per ray */
} yar_hit_soa;

typedef struct yar_gpu_options {
    int32_t device;                 /* CUDA device ordinal */
    uint32_t max_batch_rays;        /* capacity of the host-buffer staging area (0 = 16M) */
    int32_t traversal_kernel;       /* YAR_TRAVERSAL_*: 0 = chosen per scene by timing */
    uint32_t pipeline_chunk_rays;   /* host-buffer casts of two or more chunks of this many rays (0 = 4M,
                                       at most 32 chunks) overlap their copies with the traversal once
                                       the traversal kernel is chosen; UINT32_MAX: never */
} yar_gpu_options;

/* Traversal kernels (identical results, different speed): persistent warps
 * at high occupancy (PERSISTENT_64: a register cap for 8 blocks of 128
 * threads per SM, 64 registers, for closest-hit rays and for 12 blocks, 40
 * registers, for any-hit rays), persistent warps with up to 128 registers
 * (PERSISTENT_128), or one ray per thread.  With AUTO the first large enough
 * batch of each ray kind (and each render bounce) after a scene upload times
 * all three and keeps the fastest. */
#define YAR_TRAVERSAL_AUTO 0
#define YAR_TRAVERSAL_PERSISTENT_64 1
#define YAR_TRAVERSAL_PERSISTENT_128 2
#define YAR_TRAVERSAL_PER_RAY 3
#define YAR_TRAVERSAL_PER_RAY_VOTE 4  /* one ray per thread, the warp runs one traversal mode per iteration */

/* The traversal kernels chosen so far on the uploaded scene (YAR_TRAVERSAL_*,
 * 0 = not chosen yet): cast[0] closest-hit and cast[1] any-hit C-ABI casts;
 * render_closest[b] / render_any[b] the render's extend and shadow queues of
 * bounce b (the last entry covers deeper bounces). */
#define YAR_TRAVERSAL_BOUNCE_BUCKETS 5
int yar_gpu_traversal_kernels(yar_gpu_ctx* ctx, int32_t cast[2], int32_t render_closest[YAR_TRAVERSAL_BOUNCE_BUCKETS],
                              int32_t render_any[YAR_TRAVERSAL_BOUNCE_BUCKETS]);

typedef struct yar_render_stats {
    double variance;            /* render_scene's variance_estimate */
    float seconds;              /* render_scene's render_time */
    uint64_t paths;             /* camera paths traced */
    uint64_t rays_closest;      /* closest-hit rays (camera, continuation and MIS probe) */
    uint64_t rays_any;          /* any-hit shadow rays */
    uint32_t kernel_launches;
} yar_render_stats;

/* ---- context ---- */
int yar_gpu_create(yar_gpu_ctx** out, const yar_gpu_options* options);
void yar_gpu_destroy(yar_gpu_ctx* ctx);
const char* yar_gpu_last_error(const yar_gpu_ctx* ctx);
/* CUDA stream (cudaStream_t) the context launches on */
void* yar_gpu_stream(yar_gpu_ctx* ctx);
int yar_gpu_synchronize(yar_gpu_ctx* ctx);

/* ---- scene ---- */
int yar_gpu_upload_scene(yar_gpu_ctx* ctx, const yar_flat_scene* scene);

/* ---- ray casts (KdTree::intersect / intersect_any over the scene tree) ---- */
int yar_gpu_cast_closest(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t ray_count,
                         const yar_hit_soa* hits, int32_t buffers);
int yar_gpu_cast_any(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t ray_count,
                     uint8_t* occluded, int32_t buffers);
/* Same casts with per-kernel device time (CUDA events on the context stream,
 * milliseconds) written to *kernel_ms; buffers must be device memory. */
int yar_gpu_cast_closest_timed(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t ray_count,
                               const yar_hit_soa* hits, float* kernel_ms);
int yar_gpu_cast_any_timed(yar_gpu_ctx* ctx, const yar_ray* rays, uint32_t ray_count,
                           uint8_t* occluded, float* kernel_ms);

/* ---- render (render_scene) ----
 * rgb_out: host float3 image of render_region size (FP32 film resolve).
 * stats may be NULL. */
int yar_gpu_render(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats);

/* render_scene with Scene_Context::checkpoint_directory set
 * (src/ref/reference_renderer.cpp:180-324, :446-584): the directory holds the
 * reference's checkpoint files, so a render may be resumed by either renderer.
 * An empty or missing directory starts a checkpoint; otherwise its metadata
 * must name the same input_filename (the reference stores Scene::path), tile
 * count and samples per pixel, and its finished tiles are loaded instead of
 * rendered.  The others are rendered one row of tiles at a time, each tile
 * written (temporary file, then rename) as its row completes.  stats->seconds
 * includes the time of earlier sessions.  YAR_ERR_IO for a checkpoint that
 * does not match or a file that cannot be read or written. */
int yar_gpu_render_checkpoint(yar_gpu_ctx* ctx, const char* checkpoint_directory, const char* input_filename,
                              float* rgb_out, yar_render_stats* stats);

/* ---- render without allocation ----
 * No counterpart in the reference.  yar_gpu_render allocates its working
 * memory (path state, ray queues, per-sample film data) with cudaMalloc,
 * on its first call and whenever a call needs more.  Callers that must not allocate device memory at render time -
 * an application running under a fixed, pre-reserved memory budget, a host
 * that forbids allocation after start-up for latency reasons, or code whose
 * device allocator is owned by someone else - use this entry point instead:
 * it renders the path tracer (rendering_algorithm 1; direct-lighting scenes
 * and image textures are refused with YAR_ERR_UNSUPPORTED) exactly like
 * yar_gpu_render, draws past the sampler's dimension budget included, but
 * takes all working memory from
 * one static device array of YAR_GPU_STATIC_ARENA_BYTES (64 MiB) that is
 * linked into the library (every GPU that loads the library keeps it until
 * the process exits), and it calls no cudaMalloc, cudaFree or other
 * allocating routine.
 *   rgb_out_device: device memory of the context's device, float3 per pixel of
 *                   the render region (the caller allocates it).
 *   Renders whose film data and one chunk of paths do not fit in the array
 *   are rejected with YAR_ERR_CAPACITY (a 256x256 image at 16 samples per
 *   pixel fits).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls on a device share the one array and leave their data in it:
 * calls that overlap on the GPU (from different streams or contexts) race. */
#define YAR_GPU_STATIC_ARENA_BYTES (64u << 20)
int yar_gpu_render_static(yar_gpu_ctx* ctx, float* rgb_out_device, yar_render_stats* stats);

/* ---- batched render ----
 * No reference counterpart.  Renders `count` scenes, each exactly as
 * yar_gpu_render would (same per-pixel results), in one CUDA graph launch:
 * each scene's chunks and bounces run device-driven (queue lengths stay on
 * the device), the graph forks the scenes over concurrent streams, and an
 * autotuner first picks each scene's traversal kernel (timed on random rays)
 * and the stream count and paths in flight per stream (timed on the batch at
 * one sample per pixel).  rgb_out[i]: host float[w_i * h_i * 3]. */
typedef struct yar_batch_scene_stats {
    double variance;              /* render_scene's variance_estimate */
    float completion_seconds;     /* batch start to this scene's resolved film, GPU clock */
    uint64_t paths;               /* camera paths */
    uint32_t traversal_kernel[2]; /* YAR_TRAVERSAL_* used for closest-hit and any-hit rays */
} yar_batch_scene_stats;

typedef struct yar_batch_stats {
    float gpu_seconds;            /* makespan of the batch graph, GPU clock */
    uint64_t paths;               /* camera paths of all scenes */
    uint64_t rays_closest;        /* camera, continuation and MIS probe rays */
    uint64_t rays_any;            /* shadow rays */
    uint32_t branches;            /* autotuner: concurrent streams */
    uint32_t chunk_paths;         /* autotuner: paths in flight per stream */
    float upload_seconds;         /* scene uploads (host) */
    float tune_seconds;           /* autotuning (host wall time) */
    float capture_seconds;        /* graph capture and instantiation (host wall time) */
} yar_batch_stats;

int yar_gpu_render_batch(yar_gpu_ctx* ctx, const yar_flat_scene* const* scenes, uint32_t count,
                         float* const* rgb_out, yar_batch_scene_stats* scene_stats, yar_batch_stats* stats);

/* ---- guided render (config: the uploaded scene's camera, region, depth, RR, film clamp) ----
 * No reference counterpart.  Renders `passes` independent one-sample-per-
 * pixel passes of the path tracer and returns the per-pixel FP64 sum of the
 * sample radiance (clamped and scaled as the film does) and/or the mean.
 * With guide_fraction > 0 the continuation of each path vertex is drawn
 * from the learned proposal with that probability (one-sample MIS with the
 * BSDF, so the estimate stays unbiased); the first train_passes passes also
 * train the proposal online from their own path samples.  guide_fraction 0
 * is the plain path tracer (the baseline).  Requires a box filter of radius
 * <= 0.5 (each sample lands in its own pixel). */
typedef struct yar_guided_params {
    uint32_t passes;          /* samples per pixel, one independent pass each */
    uint32_t train_passes;    /* guided: the first passes also train the proposal */
    float guide_fraction;     /* probability of drawing a continuation from the proposal, [0, 1) */
    float learning_rate;      /* Adam step size */
    uint32_t train_steps;     /* optimizer steps (minibatches) per training pass */
    uint32_t stream_offset;   /* distinct values give statistically independent renders (< 4096) */
    float time_budget;        /* seconds; > 0 stops after the pass that reaches it */
    uint32_t keep_guide;      /* 1: start from the current network instead of re-initialising it */
    /* 0: the image is the mean of `passes` one-sample passes.  > 0: the
     * stratified form - the train_passes training passes (guided only), then
     * the image rendered with the scene's stratified pixel sampler at this
     * many samples per pixel (rounded up to nx x ny strata, nx = ceil(sqrt(n)),
     * ny = ceil(n / nx): a perfect square stays one, as RAY's --spp makes it),
     * continuations drawn from the trained proposal; `passes` and
     * `time_budget` are not used, radiance_sum receives image x spp. */
    uint32_t samples_per_pixel;
    /* stratified form: the proposal guides the continuations of the first
     * guide_bounces vertices of each path (0: every vertex); deeper vertices
     * sample the BSDF alone */
    uint32_t guide_bounces;
    /* stratified form: > 0 sets the strata columns nx (ny = ceil(n / nx))
     * instead of ceil(sqrt(n)); at most 4 x ny and at least ny / 4 */
    uint32_t strata_x;
} yar_guided_params;

typedef struct yar_guided_stats {
    uint32_t passes;          /* passes rendered */
    float seconds;            /* wall time of the passes, training included */
    float train_seconds;      /* of which record finalisation and optimizer steps */
    uint64_t rays;            /* closest-hit + any-hit rays traced */
    uint64_t train_samples;   /* training samples used */
    float loss;               /* loss of the last minibatch (mean over its samples) */
} yar_guided_stats;

/* radiance_sum: host double[w * h * 3] or NULL; rgb_out: host float[w * h * 3] or NULL */
int yar_gpu_guided_render(yar_gpu_ctx* ctx, const yar_guided_params* params, double* radiance_sum, float* rgb_out,
                          yar_guided_stats* stats);

/* ---- learned directional proposal: the network ----
 * No reference counterpart: the reference has no path guiding.  A BF16 MLP
 * (FP32 accumulation on the tensor cores) maps a shading point to a mixture
 * of 8 von Mises-Fisher lobes over world directions; the guided render
 * trains it online and samples path continuations from it.  These calls
 * expose the network itself (tests, custom training loops).
 *   parameters: YAR_GUIDE_PARAMS floats, four row-major [out][in] matrices
 *     W1 64x128, W2 64x64, W3 64x64, W4 64x64.  Input 127 and hidden unit 63
 *     are the constant 1 (bias columns); outputs 0..39 are 8 x (mean xyz,
 *     log kappa, logit).
 *   box: scene bounds (min xyz, max xyz), positions are normalised by it.
 *   queries (device, 16-byte aligned): 12 floats per row
 *     {pos xyz, normal xyz, wo xyz, 0, 0, 0}
 *   lobes (device): YAR_GUIDE_LOBE_FLOATS per row, 8 x {mean xyz, kappa, weight}
 *   samples (device): 16 floats per row {pos, normal, wo, dir xyz, weight, 0, 0, 0};
 *     loss = sum over rows of -(weight * weight_scale) * log q(dir) */
#define YAR_GUIDE_PARAMS 20480
#define YAR_GUIDE_LOBE_FLOATS 40
int yar_guide_set_params(yar_gpu_ctx* ctx, const float* params);
int yar_guide_get_params(yar_gpu_ctx* ctx, float* params);
int yar_guide_infer(yar_gpu_ctx* ctx, const float* queries, uint32_t n, const float box[6], float* lobes);

/* Diagnostic, no counterpart in the reference: runs the tensor-core kernels'
 * bounded mbarrier wait (`limit` polls, 1..2^24) on a barrier that nothing
 * arrives at.  Returns YAR_ERR_TIMEOUT once the wait gives up - the status the
 * network kernels report when a tensor-core wait runs out - and leaves the
 * context usable. */
int yar_gpu_wait_selftest(yar_gpu_ctx* ctx, uint32_t limit);
/* summed gradient of the loss (device, YAR_GUIDE_PARAMS floats); loss to the host */
int yar_guide_gradient(yar_gpu_ctx* ctx, const float* samples, uint32_t n, const float box[6], float weight_scale,
                       float* grad, float* loss);
/* one Adam step (beta 0.9 / 0.99) on the loss */
int yar_guide_train_step(yar_gpu_ctx* ctx, const float* samples, uint32_t n, const float box[6],
                         float weight_scale, float learning_rate, float* loss);

/* ---- host-side kd-tree builders (the reference's builder, same node stream) ----
 * The returned node array is owned by the library; release it with yar_free_nodes. */
int yar_build_mesh_kdtree(const float* vertices, uint32_t vertex_count,
                          const int32_t* indices, uint32_t triangle_count,
                          int32_t thread_count,
                          float bounds_out[6], yar_kd_node** nodes_out, uint32_t* node_count_out);
int yar_build_scene_kdtree(const float* object_bounds /* 6 floats per object, world space */,
                           uint32_t object_count,
                           float bounds_out[6], yar_kd_node** nodes_out, uint32_t* node_count_out);
void yar_free_nodes(yar_kd_node* nodes);

/* kd-tree cache files in the reference's format (KdTree::save / KdTree::load,
 * src/ref/kdtree.cpp:111-160): bounds, 64-bit geometry hash, node count,
 * nodes.  A file the reference wrote loads here and vice versa, so trees
 * built once (by either builder) need not be rebuilt.  The read node array
 * is released with yar_free_nodes; trailing bytes are an error. */
int yar_read_kdtree_cache(const char* path, float bounds_out[6], uint64_t* hash_out,
                          yar_kd_node** nodes_out, uint32_t* node_count_out);
int yar_write_kdtree_cache(const char* path, const float bounds[6], uint64_t hash,
                           const yar_kd_node* nodes, uint32_t node_count);

/* transform_bounding_box (src/lib/matrix.cpp:391-402) of a tree's bounds, for
 * the scene-tree primitive bounds (src/ref/kdtree_builder.cpp:445-452) */
void yar_transform_bounds(const float object_to_world[12], const float bounds_in[6], float bounds_out[6]);

#ifdef __cplusplus
}
#endif

#endif /* YAR_GPU_H */
