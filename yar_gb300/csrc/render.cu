// render.cu - the reference-order render behind yar_gpu_render (render_scene,
// src/ref/reference_renderer.cpp:479-584) and its allocation-free variant
// yar_gpu_render_static; the kernels are in wavefront.cuh.
#include "wavefront.cuh"

#include <filesystem>
#include <fstream>
#include <map>
#include <mutex>

namespace yar {

int render_upload(yar_gpu_ctx* ctx, const yar_flat_scene* scene) {
    Render_Scene& R = ctx->render;
    R.camera = scene->camera;
    R.config = scene->config;
    R.other_light_count = scene->other_light_count;
    // per-triangle shading records
    uint64_t total = 0;
    for (uint32_t m = 0; m < scene->mesh_count; m++) total += scene->meshes[m].triangle_count;
    R.triangle_total = (uint32_t)total;
    std::vector<float4> shading(4 * total);
    uint64_t g = 0;
    for (uint32_t m = 0; m < scene->mesh_count; m++) {
        const yar_mesh_desc& mesh = scene->meshes[m];
        uint32_t flags = (mesh.normals ? 1u : 0u) | (mesh.uvs ? 2u : 0u) |
                         (mesh.reverse_geometric_normal_orientation ? 4u : 0u);
        float fflags;
        memcpy(&fflags, &flags, 4);
        for (uint32_t t = 0; t < mesh.triangle_count; t++, g++) {
            float n[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, uv[3][2] = {{0, 0}, {0, 0}, {0, 0}};
            for (int k = 0; k < 3; k++) {
                const int32_t vi = mesh.indices[3 * (size_t)t + k];
                if (mesh.normals) memcpy(n[k], mesh.normals + 3 * (size_t)vi, 12);
                if (mesh.uvs) memcpy(uv[k], mesh.uvs + 2 * (size_t)vi, 8);
            }
            shading[4 * g + 0] = make_float4(n[0][0], n[0][1], n[0][2], uv[0][0]);
            shading[4 * g + 1] = make_float4(n[1][0], n[1][1], n[1][2], uv[0][1]);
            shading[4 * g + 2] = make_float4(n[2][0], n[2][1], n[2][2], uv[1][0]);
            shading[4 * g + 3] = make_float4(uv[1][1], uv[2][0], uv[2][1], fflags);
        }
    }
    std::vector<float4> obj(7 * (size_t)scene->object_count);
    for (uint32_t i = 0; i < scene->object_count; i++) {
        const yar_object_desc& o = scene->objects[i];
        const float* a = o.object_to_world;
        const float* b = o.object_to_world_normal;
        obj[7 * i + 0] = make_float4(a[0], a[1], a[2], a[3]);
        obj[7 * i + 1] = make_float4(a[4], a[5], a[6], a[7]);
        obj[7 * i + 2] = make_float4(a[8], a[9], a[10], a[11]);
        obj[7 * i + 3] = make_float4(b[0], b[1], b[2], b[3]);
        obj[7 * i + 4] = make_float4(b[4], b[5], b[6], b[7]);
        obj[7 * i + 5] = make_float4(b[8], b[9], b[10], b[11]);
        int32_t info[4] = {(int32_t)o.material_type, o.material_index, (int32_t)o.area_light_type, o.area_light_index};
        memcpy(&obj[7 * i + 6], info, 16);
    }
    std::vector<Material_Dev> mats(std::max<uint32_t>(1, scene->material_count));
    for (uint32_t i = 0; i < scene->material_count; i++) {
        const yar_material_desc& m = scene->materials[i];
        Material_Dev& d = mats[i];
        memset(&d, 0, sizeof(d));
        d.type = m.type == YAR_MATERIAL_PLASTIC && scene->config.pbrt3_scene ? kPbrt3Plastic : m.type;
        d.reflectance = Col{m.reflectance[0], m.reflectance[1], m.reflectance[2]};
        d.texture = m.reflectance_texture;
        d.texture_scale = make_float2(m.reflectance_uv_scale[0], m.reflectance_uv_scale[1]);
        d.texture2 = m.transmittance_texture;
        d.texture2_scale = make_float2(m.transmittance_uv_scale[0], m.transmittance_uv_scale[1]);
        d.bump = m.bump;
        d.bump_height = m.bump_height;
        d.bump_texture = m.bump == 2 ? m.bump_texture : 0u;
        d.bump_scale = make_float2(m.bump_uv_scale[0], m.bump_uv_scale[1]);
        if (m.type == YAR_MATERIAL_PBRT3_FOURIER && m.fourier_table >= 1 && m.fourier_table <= scene->fourier_count &&
            scene->fourier_tables) {  // the table's device addresses are set after its upload
            const yar_fourier_desc& t = scene->fourier_tables[m.fourier_table - 1];
            d.fourier_node_count = t.node_count;
            d.fourier_channels = t.channel_count;
        }
        d.transmittance = Col{m.transmittance[0], m.transmittance[1], m.transmittance[2]};
        d.eta_t = Col{m.eta[0], m.eta[1], m.eta[2]};
        d.k_t = Col{m.k[0], m.k[1], m.k[2]};
        d.eta_i_metal = m.eta_i;
        d.ior = m.index_of_refraction;
        d.alpha_x = roughness_to_alpha(scene->config, m.u_roughness, m.roughness_is_alpha);
        d.alpha_y = roughness_to_alpha(scene->config, m.v_roughness, m.roughness_is_alpha);
        d.alpha = d.alpha_x;
        d.delta = m.type == YAR_MATERIAL_PERFECT_REFLECTOR   ? kDeltaReflector
                  : m.type == YAR_MATERIAL_PERFECT_REFRACTOR ? kDeltaRefractor
                  : m.type == YAR_MATERIAL_GLASS && !(m.u_roughness > 0.f) ? kDeltaGlass
                                                                            : kDeltaNone;
        auto rgb = [](const float* v) { return Col{v[0], v[1], v[2]}; };
        auto clamp_unit = [](Col c) {  // ColorRGB::clamp_to_unit_range
            auto c1 = [](float v) { return v < 0.f ? 0.f : (1.f < v ? 1.f : v); };
            return Col{c1(c.r), c1(c.g), c1(c.b)};
        };
        if (m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) {  // Diffuse_Transmission_BSDF (bsdf.cpp:89-103)
            d.reflectance = clamp_unit(Col{m.diffuse[0] * m.reflectance[0], m.diffuse[1] * m.reflectance[1],
                                           m.diffuse[2] * m.reflectance[2]});
            d.transmittance = clamp_unit(Col{m.diffuse[0] * m.transmittance[0], m.diffuse[1] * m.transmittance[1],
                                             m.diffuse[2] * m.transmittance[2]});
            d.extra = rgb(m.diffuse);  // the scale, for textured reflectance and transmittance
        } else if (m.type == YAR_MATERIAL_PBRT3_TRANSLUCENT) {  // roughness always remapped
            d.extra = rgb(m.diffuse);
            d.specular = rgb(m.specular);
            d.alpha = roughness_to_alpha(scene->config, m.u_roughness, 0);
        } else if (m.type == YAR_MATERIAL_PBRT3_UBER) {  // roughness always remapped
            d.specular = rgb(m.specular);
            d.extra = rgb(m.opacity);
            d.delta_reflectance = rgb(m.delta_reflectance);
            d.alpha_x = roughness_to_alpha(scene->config, m.u_roughness, 0);
            d.alpha_y = roughness_to_alpha(scene->config, m.v_roughness, 0);
            d.uber_components = std::min<uint32_t>(m.component_count, 5) << 24;
            for (uint32_t k = 0; k < m.component_count && k < 5; k++) d.uber_components |= (m.components[k] & 7u) << (3 * k);
            d.delta = kDeltaUber;  // every sample picks a layer
        }
    }
    // BSDF::reflection_scattering / transmission_scattering of each material, then the
    // mixes (Mix_BSDF, Scaled_BSDF and get_mix_info's constants, bsdf.cpp:497-629)
    auto luminance = [](const float* c) { return 0.2126729f * c[0] + 0.7151522f * c[1] + 0.0721750f * c[2]; };
    for (uint32_t i = 0; i < scene->material_count; i++) {
        const yar_material_desc& m = scene->materials[i];
        const bool black_r = !(m.reflectance[0] != 0.f || m.reflectance[1] != 0.f || m.reflectance[2] != 0.f);
        const bool black_t = !(m.transmittance[0] != 0.f || m.transmittance[1] != 0.f || m.transmittance[2] != 0.f);
        uint32_t sc = 1u;
        if (m.type == YAR_MATERIAL_GLASS || m.type == YAR_MATERIAL_DIFFUSE_TRANSMISSION) sc = 3u;
        if (m.type == YAR_MATERIAL_PBRT3_TRANSLUCENT) sc = (black_r ? 0u : 1u) | (black_t ? 0u : 2u);
        if (m.type == YAR_MATERIAL_PERFECT_REFLECTOR || m.type == YAR_MATERIAL_PERFECT_REFRACTOR) sc = 0u;
        mats[i].scattering = sc;
    }
    for (uint32_t i = 0; i < scene->material_count; i++) {
        const yar_material_desc& m = scene->materials[i];
        if (m.type != YAR_MATERIAL_MIX) continue;
        Material_Dev& d = mats[i];
        const int32_t a = m.mix_materials[0], b = m.mix_materials[1];
        if (a < 0 || b < 0 || (uint32_t)a >= scene->material_count || (uint32_t)b >= scene->material_count)
            return fail(ctx, YAR_ERR_INVALID, "mix material " + std::to_string(i) + " has no valid sub-materials");
        d.mix_sub[0] = a;
        d.mix_sub[1] = b;
        const float lum = luminance(m.mix_amount);
        d.mix_lum = lum;
        d.mix_amount = 1.f < lum ? 1.f : lum;
        d.mix_coeff = Col{1.f - m.mix_amount[0], 1.f - m.mix_amount[1], 1.f - m.mix_amount[2]};
        const float coeff[3] = {d.mix_coeff.r, d.mix_coeff.g, d.mix_coeff.b};
        d.mix_p = 1.f - luminance(coeff);
        const bool has_a = mats[a].type != kPerfectReflector && mats[a].type != kPerfectRefractor;
        const bool has_b = mats[b].type != kPerfectReflector && mats[b].type != kPerfectRefractor;
        d.scattering = (has_a ? mats[a].scattering : 0u) | (has_b ? mats[b].scattering : 0u);
        d.delta = kDeltaMix;
    }
    // whether Shading_Context::initialize_scattering creates a BSDF (some layer is not delta)
    for (uint32_t i = 0; i < scene->material_count; i++) {
        const yar_material_desc& m = scene->materials[i];
        bool has = mats[i].delta == kDeltaNone || mats[i].delta == kDeltaMix;
        if (m.type == YAR_MATERIAL_PBRT3_UBER)
            for (uint32_t k = 0; k < m.component_count && k < 5; k++) has = has || m.components[k] < YAR_UBER_DELTA_REFLECTION;
        mats[i].has_bsdf = has ? 1u : 0u;
    }
    std::vector<Rect_Light_Dev> lights(std::max<uint32_t>(1, scene->rect_light_count));
    for (uint32_t i = 0; i < scene->rect_light_count; i++) {
        const yar_rect_light_desc& l = scene->rect_lights[i];
        const float* m = l.light_to_world;
        lights[i].r0 = make_float4(m[0], m[1], m[2], m[3]);
        lights[i].r1 = make_float4(m[4], m[5], m[6], m[7]);
        lights[i].r2 = make_float4(m[8], m[9], m[10], m[11]);
        lights[i].le = make_float4(l.emitted_radiance[0], l.emitted_radiance[1], l.emitted_radiance[2], l.size[0]);
        lights[i].sz = make_float4(l.size[1], 0.f, 0.f, 0.f);
    }
    // Probe culling per rectangular light (probe_may_reach): only when the
    // light frame is orthogonal with a unit normal and every vertex of the
    // light's objects lies on its plane and inside its rectangle (within 1e-3
    // of its larger side), so that a ray missing the widened rectangle misses
    // the light's triangles.
    for (uint32_t i = 0; i < scene->rect_light_count; i++) {
        const float* m = scene->rect_lights[i].light_to_world;
        const double X[3] = {m[0], m[4], m[8]}, Y[3] = {m[1], m[5], m[9]}, N[3] = {m[2], m[6], m[10]};
        const double C[3] = {m[3], m[7], m[11]};
        auto dot3d = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
        const double xx = dot3d(X, X), yy = dot3d(Y, Y), nn = dot3d(N, N);
        const double sx = scene->rect_lights[i].size[0], sy = scene->rect_lights[i].size[1];
        bool ok = xx > 0 && yy > 0 && std::fabs(nn - 1.0) <= 1e-3 && sx > 0 && sy > 0 &&
                  std::fabs(dot3d(X, Y)) <= 1e-6 * std::sqrt(xx * yy) &&
                  std::fabs(dot3d(X, N)) <= 1e-6 * std::sqrt(xx * nn) && std::fabs(dot3d(Y, N)) <= 1e-6 * std::sqrt(yy * nn);
        const double tol = 1e-3 * std::max(sx, sy);
        uint32_t objects_found = 0;
        for (uint32_t o = 0; ok && o < scene->object_count; o++) {
            const yar_object_desc& ob = scene->objects[o];
            if (ob.area_light_type != YAR_LIGHT_DIFFUSE_RECTANGULAR || ob.area_light_index != (int32_t)i) continue;
            if (ob.mesh_index < 0 || (uint32_t)ob.mesh_index >= scene->mesh_count) {
                ok = false;
                break;
            }
            objects_found++;
            const yar_mesh_desc& mesh = scene->meshes[ob.mesh_index];
            const float* w = ob.object_to_world;
            for (uint32_t v = 0; ok && v < mesh.vertex_count; v++) {
                const float* pv = mesh.vertices + 3 * (size_t)v;
                double P[3];
                for (int r = 0; r < 3; r++)
                    P[r] = w[4 * r] * pv[0] + w[4 * r + 1] * pv[1] + w[4 * r + 2] * pv[2] + w[4 * r + 3] - C[r];
                const double a = dot3d(P, X) / xx, b = dot3d(P, Y) / yy, h = dot3d(P, N) / std::sqrt(nn);
                ok = std::fabs(h) <= tol && std::fabs(a) <= 0.5 * sx + tol && std::fabs(b) <= 0.5 * sy + tol;
            }
        }
        if (ok && objects_found > 0)
            lights[i].sz = make_float4((float)sy, (float)(1.0 / xx), (float)(1.0 / yy), 1.f);
    }
    std::vector<Delta_Light_Dev> dlights(std::max<uint32_t>(1, scene->delta_light_count));
    for (uint32_t i = 0; i < scene->delta_light_count; i++) {
        const yar_delta_light_desc& l = scene->delta_lights[i];
        float type_bits;
        memcpy(&type_bits, &l.type, 4);
        dlights[i].a = make_float4(l.position[0], l.position[1], l.position[2], type_bits);
        dlights[i].b = make_float4(l.direction[0], l.direction[1], l.direction[2], std::cos(l.cone_angle));
        dlights[i].c = make_float4(l.intensity[0], l.intensity[1], l.intensity[2],
                                   std::cos(std::max(0.f, l.cone_angle - l.penumbra_angle)));
    }
    R.host_delta_lights.assign(scene->delta_lights, scene->delta_lights + scene->delta_light_count);
    // Triangle-mesh lights: init_triangle_mesh_light_samplers (src/ref/reference_renderer.cpp:131-151)
    // with Triangle_Mesh::get_area / get_triangle_area and Distribution_1D::initialize
    // (src/ref/sampling.cpp:149-166), in the reference's float order.
    std::vector<uint32_t> mesh_first(scene->mesh_count + 1, 0);
    for (uint32_t m = 0; m < scene->mesh_count; m++) mesh_first[m + 1] = mesh_first[m] + scene->meshes[m].triangle_count;
    std::vector<Mesh_Light_Dev> mlights(std::max<uint32_t>(1, scene->mesh_light_count));
    std::vector<float> cdf;
    for (uint32_t i = 0; i < scene->mesh_light_count; i++) {
        const yar_mesh_light_desc& l = scene->mesh_lights[i];
        if (l.triangle_mesh_index >= scene->mesh_count || scene->meshes[l.triangle_mesh_index].triangle_count == 0)
            return fail(ctx, YAR_ERR_INVALID, "triangle-mesh light " + std::to_string(i) + " has no valid mesh");
        const yar_mesh_desc& mesh = scene->meshes[l.triangle_mesh_index];
        auto area = [&](uint32_t t) {
            float p[3][3];
            for (int k = 0; k < 3; k++) memcpy(p[k], mesh.vertices + 3 * (size_t)mesh.indices[3 * (size_t)t + k], 12);
            const float e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
            const float e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
            const float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                e1[0] * e2[1] - e1[1] * e2[0]};
            return std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * 0.5f;
        };
        float mesh_area = 0.f;
        for (uint32_t t = 0; t < mesh.triangle_count; t++) mesh_area += area(t);
        const uint32_t offset = (uint32_t)cdf.size();
        float total = 0.f, sum = 0.f;
        for (uint32_t t = 0; t < mesh.triangle_count; t++) total += area(t);
        for (uint32_t t = 0; t < mesh.triangle_count; t++) {
            sum += area(t);
            cdf.push_back(sum / total);
        }
        mlights[i].le = make_float4(l.emitted_radiance[0], l.emitted_radiance[1], l.emitted_radiance[2], mesh_area);
        mlights[i].info = make_uint4(mesh_first[l.triangle_mesh_index], mesh.triangle_count, offset, 0u);
    }
    if (cdf.empty()) cdf.push_back(1.f);
    R.mesh_light_count = scene->mesh_light_count;
    std::vector<Sphere_Light_Dev> slights(std::max<uint32_t>(1, scene->sphere_light_count));
    for (uint32_t i = 0; i < scene->sphere_light_count; i++) {
        const yar_sphere_light_desc& l = scene->sphere_lights[i];
        slights[i].a = make_float4(l.position[0], l.position[1], l.position[2], l.radius);
        slights[i].le = make_float4(l.emitted_radiance[0], l.emitted_radiance[1], l.emitted_radiance[2], 0.f);
    }
    R.sphere_light_count = scene->sphere_light_count;
    R.host_sphere_lights.assign(scene->sphere_lights, scene->sphere_lights + scene->sphere_light_count);
    // Environment light: the map as float4 texels and its Distribution_2D, built as
    // initialize_from_latitude_longitude_radiance_map does (src/ref/sampling.cpp:185-259).
    R.has_environment = scene->environment != nullptr;
    R.texture_count = scene->texture_count;
    R.has_no_shadow_meshes = false;
    for (uint32_t m = 0; m < scene->mesh_count; m++)
        if (scene->meshes[m].visibility == YAR_VISIBLE_NO_SHADOWS) R.has_no_shadow_meshes = true;
    std::vector<float4> env_map(1, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> env_marginal(1, 1.f), env_cdfs(1, 1.f);
    if (R.has_environment) {
        const yar_environment_desc& e = *scene->environment;
        if (!e.radiance || e.width == 0 || e.height == 0)
            return fail(ctx, YAR_ERR_INVALID, "environment light without a map");
        R.environment = e;
        R.environment.radiance = nullptr;
        const int nx = (int)e.width, ny = (int)e.height;
        env_map.assign((size_t)nx * ny, make_float4(0.f, 0.f, 0.f, 0.f));
        for (size_t i = 0; i < env_map.size(); i++)
            env_map[i] = make_float4(e.radiance[3 * i], e.radiance[3 * i + 1], e.radiance[3 * i + 2], 0.f);
        auto nearest_lum = [&](float u, float v) {
            int x = (int)(u * (float)nx), y = (int)(v * (float)ny);
            x = x < 0 ? 0 : (nx - 1 < x ? nx - 1 : x);
            y = y < 0 ? 0 : (ny - 1 < y ? ny - 1 : y);
            const float4 t = env_map[(size_t)y * nx + x];
            return 0.2126729f * t.x + 0.7151522f * t.y + 0.0721750f * t.z;
        };
        std::vector<float> values((size_t)nx * ny), row_sums(ny);
        for (int y = 0; y < ny; y++) {
            const float sin_theta = std::sin((y + 0.5f) / (float)ny * 3.14159265f);
            const float v = (y + 0.5f) / (float)ny;
            for (int x = 0; x < nx; x++) values[(size_t)y * nx + x] = nearest_lum((x + 0.5f) / (float)nx, v) * sin_theta;
        }
        float total = 0.f;
        int last_nonzero = -1;
        for (int y = 0; y < ny; y++) {
            float row = 0.f;
            for (int x = 0; x < nx; x++) row += values[(size_t)y * nx + x];
            row_sums[y] = row;
            total += row;
            if (row != 0.f) last_nonzero = y;
        }
        if (last_nonzero < 0) return fail(ctx, YAR_ERR_UNSUPPORTED, "environment map is black");
        env_marginal.assign(ny, 1.f);
        for (int y = 0; y < last_nonzero; y++) env_marginal[y] = (y == 0 ? 0.f : env_marginal[y - 1]) + row_sums[y] / total;
        env_cdfs.assign((size_t)nx * ny, 0.f);
        for (int y = 0; y < ny; y++) {
            float* cdf = env_cdfs.data() + (size_t)y * nx;
            if (row_sums[y] == 0.f) continue;
            for (int x = 0; x < nx - 1; x++) cdf[x] = (x == 0 ? 0.f : cdf[x - 1]) + values[(size_t)y * nx + x] / row_sums[y];
            cdf[nx - 1] = 1.f;
        }
    }
    R.host_materials.assign(scene->materials, scene->materials + scene->material_count);
    R.host_fourier_tables.clear();
    if (scene->fourier_tables)
        R.host_fourier_tables.assign(scene->fourier_tables, scene->fourier_tables + scene->fourier_count);
    R.host_rect_lights.assign(scene->rect_lights, scene->rect_lights + scene->rect_light_count);
    R.host_object_info.resize(4 * (size_t)scene->object_count);
    for (uint32_t i = 0; i < scene->object_count; i++) {
        const yar_object_desc& o = scene->objects[i];
        R.host_object_info[4 * i + 0] = (int32_t)o.material_type;
        R.host_object_info[4 * i + 1] = o.material_index;
        R.host_object_info[4 * i + 2] = (int32_t)o.area_light_type;
        R.host_object_info[4 * i + 3] = o.area_light_index;
    }
    int rc;
    auto up = [&](Device_Buffer& b, const void* src, size_t bytes) {
        int r = device_alloc(ctx, b, bytes);
        if (r != YAR_OK) return r;
        cudaError_t e = cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
        return e == cudaSuccess ? YAR_OK : cuda_fail(ctx, e, "render upload");
    };
    if ((rc = up(R.shading, shading.data(), shading.size() * sizeof(float4))) != YAR_OK) return rc;
    if ((rc = up(R.object_info, obj.data(), obj.size() * sizeof(float4))) != YAR_OK) return rc;
    // pbrt3 fourier tables: every read the evaluation makes stays inside them
    // (one or three channels, series inside the coefficients, the last node at
    // least 1 so that the node search of a clamped cosine ends inside)
    if (scene->fourier_count) {
        if (!scene->fourier_tables || !scene->fourier_floats || !scene->fourier_uints)
            return fail(ctx, YAR_ERR_INVALID, "fourier tables without data");
        for (uint32_t i = 0; i < scene->fourier_count; i++) {
            const yar_fourier_desc& t = scene->fourier_tables[i];
            const uint64_t pairs = (uint64_t)t.node_count * t.node_count;
            bool ok = t.node_count > 0 && t.node_count <= 65536 && (t.channel_count == 1 || t.channel_count == 3) &&
                      t.nodes + t.node_count <= scene->fourier_float_count &&
                      t.coeffs + t.coeff_count <= scene->fourier_float_count &&
                      t.series + 2 * pairs <= scene->fourier_uint_count;
            if (ok) ok = scene->fourier_floats[t.nodes + t.node_count - 1] >= 1.f;
            for (uint64_t k = 0; ok && k < pairs; k++) {
                const uint64_t off = scene->fourier_uints[t.series + 2 * k];
                const uint64_t cnt = scene->fourier_uints[t.series + 2 * k + 1];
                ok = off + cnt * t.channel_count <= t.coeff_count;
            }
            if (!ok) return fail(ctx, YAR_ERR_INVALID, "fourier table " + std::to_string(i) + " is malformed");
        }
        if ((rc = up(R.fourier_floats, scene->fourier_floats, scene->fourier_float_count * sizeof(float))) != YAR_OK)
            return rc;
        if ((rc = up(R.fourier_uints, scene->fourier_uints, scene->fourier_uint_count * sizeof(uint32_t))) != YAR_OK)
            return rc;
        const float* ff = reinterpret_cast<const float*>(R.fourier_floats.ptr);
        const uint32_t* fu = reinterpret_cast<const uint32_t*>(R.fourier_uints.ptr);
        for (uint32_t i = 0; i < scene->material_count; i++) {
            const yar_material_desc& m = scene->materials[i];
            if (m.type != YAR_MATERIAL_PBRT3_FOURIER || m.fourier_table == 0 || m.fourier_table > scene->fourier_count)
                continue;
            const yar_fourier_desc& t = scene->fourier_tables[m.fourier_table - 1];
            mats[i].fourier_nodes = ff + t.nodes;
            mats[i].fourier_coeffs = ff + t.coeffs;
            mats[i].fourier_series = fu + t.series;
        }
    }
    if ((rc = up(R.materials, mats.data(), mats.size() * sizeof(Material_Dev))) != YAR_OK) return rc;
    if ((rc = up(R.rect_lights, lights.data(), lights.size() * sizeof(Rect_Light_Dev))) != YAR_OK) return rc;
    if ((rc = up(R.delta_lights, dlights.data(), dlights.size() * sizeof(Delta_Light_Dev))) != YAR_OK) return rc;
    if ((rc = up(R.mesh_lights, mlights.data(), mlights.size() * sizeof(Mesh_Light_Dev))) != YAR_OK) return rc;
    if ((rc = up(R.mesh_cdf, cdf.data(), cdf.size() * sizeof(float))) != YAR_OK) return rc;
    if ((rc = up(R.sphere_lights, slights.data(), slights.size() * sizeof(Sphere_Light_Dev))) != YAR_OK) return rc;
    if ((rc = up(R.env_map, env_map.data(), env_map.size() * sizeof(float4))) != YAR_OK) return rc;
    if ((rc = up(R.env_marginal, env_marginal.data(), env_marginal.size() * sizeof(float))) != YAR_OK) return rc;
    if ((rc = up(R.env_cdfs, env_cdfs.data(), env_cdfs.size() * sizeof(float))) != YAR_OK) return rc;
    {   // image textures: texels as float4, per-mip and per-texture records, EWA weights
        std::vector<float4> texels(1, make_float4(0.f, 0.f, 0.f, 0.f));
        std::vector<uint4> mips(1, make_uint4(1, 1, 0, 0));
        std::vector<uint2> texs(1, make_uint2(0, 1));
        if (scene->texture_count) {
            uint64_t total = 0;
            for (uint32_t i = 0; i < scene->texture_mip_count; i++) {
                const yar_texture_mip_desc& m = scene->texture_mips[i];
                if (m.width == 0 || m.height == 0 || (m.width & (m.width - 1)) || (m.height & (m.height - 1)))
                    return fail(ctx, YAR_ERR_INVALID, "texture mips must have power-of-two sizes");
                if (m.texel_offset > scene->texel_count ||
                    (uint64_t)m.width * m.height > scene->texel_count - m.texel_offset)
                    return fail(ctx, YAR_ERR_INVALID, "texture mip outside the texel array");
                total = std::max<uint64_t>(total, m.texel_offset + (uint64_t)m.width * m.height);
            }
            if (total >= (1ull << 32)) return fail(ctx, YAR_ERR_CAPACITY, "more than 2^32 texels");
            if (!scene->texels) return fail(ctx, YAR_ERR_INVALID, "textures without texels");
            texels.assign(total, make_float4(0.f, 0.f, 0.f, 0.f));
            for (uint64_t i = 0; i < total; i++)
                texels[i] = make_float4(scene->texels[3 * i], scene->texels[3 * i + 1], scene->texels[3 * i + 2], 0.f);
            mips.resize(scene->texture_mip_count);
            for (uint32_t i = 0; i < scene->texture_mip_count; i++) {
                const yar_texture_mip_desc& m = scene->texture_mips[i];
                mips[i] = make_uint4(m.width, m.height, (uint32_t)m.texel_offset, 0u);
            }
            texs.resize(scene->texture_count);
            for (uint32_t i = 0; i < scene->texture_count; i++) {
                const yar_texture_desc& t = scene->textures[i];
                if (t.mip_count == 0 || (uint64_t)t.first_mip + t.mip_count > scene->texture_mip_count)
                    return fail(ctx, YAR_ERR_INVALID, "texture with invalid mips");
                texs[i] = make_uint2(t.first_mip, t.mip_count);
            }
            // The EWA footprint walks integer texel coordinates held in floats:
            // refuse uv ranges whose texel coordinates reach 2^22 (a bump map's
            // finite-difference lookups step past the uv by the footprint, which
            // only grazing hits make large; there the reference's own float
            // counters stop advancing, and the device's loops stay bounded).
            for (uint32_t o = 0; o < scene->object_count; o++) {
                const yar_object_desc& ob = scene->objects[o];
                if (ob.material_index < 0 || (uint32_t)ob.material_index >= scene->material_count) continue;
                const yar_material_desc& md = scene->materials[ob.material_index];
                const yar_mesh_desc& mesh = scene->meshes[ob.mesh_index];
                if (!mesh.uvs) continue;
                const uint32_t slot_texture[3] = {md.reflectance_texture, md.transmittance_texture,
                                                  md.bump == 2 ? md.bump_texture : 0u};
                const float* slot_scale[3] = {md.reflectance_uv_scale, md.transmittance_uv_scale, md.bump_uv_scale};
                float uv_max = -1.f;
                for (int k = 0; k < 3; k++) {
                    if (!slot_texture[k] || slot_texture[k] > scene->texture_count) continue;
                    if (uv_max < 0.f) {
                        uv_max = 0.f;
                        for (uint64_t j = 0; j < 2ull * mesh.vertex_count; j++)
                            uv_max = std::max(uv_max, std::fabs(mesh.uvs[j]));
                    }
                    const yar_texture_desc& t = scene->textures[slot_texture[k] - 1];
                    const yar_texture_mip_desc& top = scene->texture_mips[t.first_mip];
                    const double reach = (double)uv_max *
                                         std::max(std::fabs(slot_scale[k][0]), std::fabs(slot_scale[k][1])) *
                                         std::max(top.width, top.height);
                    if (!(reach < (double)(1 << 22)))
                        return fail(ctx, YAR_ERR_UNSUPPORTED, "texture coordinates of object " + std::to_string(o) +
                                                                  " reach 2^22 texels");
                }
            }
        }
        // do_EWA's weights exp(-2 x), x = i / 255 (src/ref/image_texture.cpp:503-512), correctly rounded
        std::vector<float> w(256);
        for (int i = 0; i < 256; i++) w[i] = (float)std::exp((double)(-2.f * ((float)i / (float)(256 - 1))));
        if ((rc = up(R.texels, texels.data(), texels.size() * sizeof(float4))) != YAR_OK) return rc;
        if ((rc = up(R.texture_mips, mips.data(), mips.size() * sizeof(uint4))) != YAR_OK) return rc;
        if ((rc = up(R.textures, texs.data(), texs.size() * sizeof(uint2))) != YAR_OK) return rc;
        if ((rc = up(R.ewa_weights, w.data(), w.size() * sizeof(float))) != YAR_OK) return rc;
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render upload");
    return YAR_OK;
}

void render_release(yar_gpu_ctx* ctx) {
    Render_Scene& R = ctx->render;
    for (Device_Buffer* b : {&R.shading, &R.materials, &R.rect_lights, &R.delta_lights, &R.mesh_lights, &R.mesh_cdf,
                             &R.sphere_lights, &R.env_map, &R.env_marginal, &R.env_cdfs, &R.texels,
                             &R.texture_mips, &R.textures, &R.ewa_weights, &R.fourier_floats, &R.fourier_uints, &R.object_info,
                             &R.object_to_world, &R.object_to_world_normal})
        device_free(*b);
    for (Device_Buffer& b : ctx->render_scratch) device_free(b);
    ctx->render_scratch.clear();
    for (Device_Buffer& b : ctx->guided_scratch) device_free(b);
    ctx->guided_scratch.clear();
    device_free(ctx->guide_queries);
    device_free(ctx->guide_lobes);
}

// Per-tile film data of a render (checkpoint bands): each tile's variance
// accumulator and its Film_Pixel array (color sum, weight) over its pixel bounds.
struct Tile_Output {
    std::vector<double> tile_variance;
    std::vector<uint32_t> offset;  // per tile, into pixels
    std::vector<float4> pixels;
};

int render_run_params(yar_gpu_ctx* ctx, const Render_Params& p, float* rgb_out, yar_render_stats* stats,
                      Tile_Output* tiles_out, const Guide_Render_Hook* guide = nullptr);

int render_run(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats) {
    if (!rgb_out) return fail(ctx, YAR_ERR_INVALID, "null image buffer");
    if (ctx->render.config.rendering_algorithm == 0) return render_direct(ctx, rgb_out, stats);
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    return render_run_params(ctx, p, rgb_out, stats, nullptr);
}

// The render of render_run over the sample region of p.  With tiles_out, the
// image is not resolved: the tiles' film data come back instead.
int render_run_params(yar_gpu_ctx* ctx, const Render_Params& p_in, float* rgb_out, yar_render_stats* stats,
                      Tile_Output* tiles_out, const Guide_Render_Hook* guide) {
    cudaSetDevice(ctx->device);
    // Draws past the sampler budget follow the reference's per-pixel stream
    // (exact tail) for the reference's own streams.
    Render_Params p = p_in;
    p.exact_tail = (p.stream_hi == 0 && p.n1d > 0) ? 1 : 0;
    Render_Params p_wave = p;
    p_wave.exact_tail = 2;
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t pixels = (uint64_t)p.sw * p.sh;
    const uint64_t samples = pixels * p.spp;
    const uint64_t budget = guide && guide->chunk_paths ? guide->chunk_paths : kChunkSampleBudget;
    const uint64_t chunk_pixels = std::max<uint64_t>(1, std::min<uint64_t>(pixels, budget / p.spp));
    const uint64_t cap = chunk_pixels * p.spp;  // paths per chunk

    // scratch: everything sized by the largest chunk; a buffer of the last
    // call is kept when it is large enough (cudaMalloc and cudaFree synchronise)
    std::vector<Device_Buffer>& B = ctx->render_scratch;
    if (B.size() != 43) {
        for (Device_Buffer& b : B) device_free(b);
        B.assign(43, Device_Buffer{});
    }
    int rc = YAR_OK;
    auto alloc = [&](int i, size_t bytes) {
        if (rc == YAR_OK && !(B[i].ptr && B[i].bytes >= bytes)) rc = device_alloc(ctx, B[i], bytes);
    };
    alloc(0, samples * sizeof(float4));                    // radiance
    alloc(1, samples * sizeof(float2));                    // image-plane samples
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
    alloc(26, 8 * sizeof(uint32_t));                       // counters
    alloc(27, pixels * sizeof(double));                    // pixel variance
    alloc(28, (size_t)p.tiles_x * p.tiles_y * sizeof(double));
    alloc(29, (size_t)p.rw * p.rh * 3 * sizeof(float));    // rgb
    if (p.exact_tail) {
        alloc(30, cap * sizeof(uint32_t));                 // rng draws past the budget
        alloc(31, cap * 2 * sizeof(float4));               // deferred extend rays
        alloc(32, cap * sizeof(uint32_t));                 // deferred slots per pixel, in sample order
        alloc(33, chunk_pixels * sizeof(uint32_t));        // deferred count per pixel
        alloc(34, chunk_pixels * sizeof(uint32_t));        // stream position per pixel
        alloc(35, 2 * sizeof(uint32_t));                   // largest count, stray-draw flag
    }
    alloc(36, 2 * sizeof(unsigned long long));             // closest and any rays (device-driven bounces)
    alloc(37, cap * sizeof(uint8_t));                      // shading class per extend-queue entry
    alloc(38, cap * sizeof(uint32_t));                     // shading order of the extend queue
    alloc(39, 2 * kShadeClasses * sizeof(uint32_t));       // class sizes and cursors
    alloc(40, cap * sizeof(uint16_t));                     // extend-queue sort keys
    alloc(41, kRayBins * sizeof(uint32_t));                // their histogram, then the bins' cursors
    if (p.spec_diffs) alloc(42, cap * 3 * sizeof(float4));  // delta rays' specular differential rays
    if (rc != YAR_OK) return rc;

    Path_State ps{dptr<float4>(B[4]), dptr<float4>(B[5]), dptr<uint32_t>(B[6]), dptr<uint4>(B[7]),
                  dptr<float4>(B[8]), dptr<float4>(B[9]), dptr<float4>(B[10]), dptr<float4>(B[11]),
                  dptr<float4>(B[12]), dptr<uint8_t>(B[13]), dptr<float4>(B[14]), dptr<uint2>(B[15])};
    ps.rng_draws = dptr<uint32_t>(B[30]);
    ps.deferred = dptr<float4>(B[31]);
    ps.image_samples = dptr<float2>(B[1]);
    ps.diff = dptr<float4>(B[42]);
    Queues q{};
    q.ext_rays[0] = dptr<float4>(B[16]);
    q.ext_rays[1] = dptr<float4>(B[17]);
    q.ext_slot[0] = dptr<uint32_t>(B[18]);
    q.ext_slot[1] = dptr<uint32_t>(B[19]);
    q.ext_hit4 = dptr<float4>(B[20]);
    q.ext_hit2 = dptr<uint2>(B[21]);
    q.shd_rays = dptr<float4>(B[22]);
    q.shd_slot = dptr<uint32_t>(B[23]);
    q.prb_rays = dptr<float4>(B[24]);
    q.prb_slot = dptr<uint32_t>(B[25]);
    q.counters = dptr<uint32_t>(B[26]);
    Scene_Dev S = scene_dev(ctx->ds, ctx->render);
    float4* radiance = dptr<float4>(B[0]);
    float2* image_samples = dptr<float2>(B[1]);

    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemsetAsync(q.counters, 0, 8 * sizeof(uint32_t), st);
    uint64_t rays_closest = 0, rays_any = 0;
    uint32_t launches = 0;
    // Bounces are driven from the device once a render of this scene has tuned
    // the traversal kernels with host-read queue lengths (the guided render's
    // hook reads them too): no host round trip until the render ends, or per
    // chunk with the exact tail (its wave count).
    const bool device_driven = !guide && ctx->render_tuned;
    unsigned long long* rays_dev = dptr<unsigned long long>(B[36]);
    if (device_driven && e == cudaSuccess) e = cudaMemsetAsync(rays_dev, 0, 2 * sizeof(unsigned long long), st);
    // The shading order of the extend queue (material classes together), when
    // the scene's objects use more than one of the classes diffuse, metal and
    // other: qo is q with the order, for the shade kernel.  On C3 (Lambertian
    // and GGX objects) the render went from 1.555 to 1.307 s; on C1 (diffuse
    // only) ordering cost 5% and is skipped.
    bool mixed = false;
    {
        uint32_t seen = 0;
        const std::vector<int32_t>& oi = ctx->render.host_object_info;
        for (size_t o = 0; o + 3 < oi.size(); o += 4) {
            if ((uint32_t)oi[o + 2] != YAR_LIGHT_NULL || (uint32_t)oi[o] == YAR_MATERIAL_NULL) continue;
            const uint32_t m = (uint32_t)oi[o];
            seen |= m == YAR_MATERIAL_DIFFUSE ? 1u : (m == YAR_MATERIAL_METAL ? 2u : 4u);
        }
        mixed = (seen & (seen - 1)) != 0;
    }
    uint8_t* shade_keys = dptr<uint8_t>(B[37]);
    uint32_t* shade_bins = dptr<uint32_t>(B[39]);
    Queues qo = q;
    qo.order = mixed ? dptr<uint32_t>(B[38]) : nullptr;
    auto order_queue = [&](const Queues& qq, uint32_t max_count, int grid) {
        if (!mixed) return;
        cudaMemsetAsync(shade_bins, 0, 2 * kShadeClasses * sizeof(uint32_t), st);
        shade_bin_kernel<<<grid, kBlock, 0, st>>>(S, qq, max_count, shade_keys, shade_bins);
        shade_order_kernel<<<grid, kBlock, 0, st>>>(qq, max_count, shade_keys, shade_bins,
                                                    const_cast<uint32_t*>(qo.order));
    };
    // The rays of bounces after the camera's, sorted by direction octant and
    // origin cell into the other extend buffer (the traversal then reads
    // that one), in scenes of at most kSortRaysMaxTriangles triangles: on C1
    // (36 triangles) the render went from 5.50 to 5.32 ms; on C3 (4.1M
    // triangles, a kd-tree larger than L2) the sort cost more than it saved
    // (1.323-1.345 s against 1.311 s).
    Ray_Grid grid_box;
    for (int k = 0; k < 3; k++) {
        const float lo = ctx->ds.scene_bounds[k], ext = ctx->ds.scene_bounds[3 + k] - lo;
        grid_box.lo[k] = lo;
        grid_box.scale[k] = ext > 0.f ? 8.f / ext : 0.f;
    }
    constexpr uint64_t kSortRaysMaxTriangles = 1u << 20;
    const bool sort_rays = ctx->tris.bytes / (3 * sizeof(float4)) <= kSortRaysMaxTriangles;
    uint16_t* ray_keys = dptr<uint16_t>(B[40]);
    uint32_t* ray_hist = dptr<uint32_t>(B[41]);
    auto sort_queue = [&](int from, const uint32_t* count_dev, uint32_t count, uint32_t max_count) {
        cudaMemsetAsync(ray_hist, 0, kRayBins * sizeof(uint32_t), st);
        const int g = std::min(grid_for(max_count), 152 * 2);
        ray_hist_kernel<<<g, 256, 0, st>>>(grid_box, q.ext_rays[from], count_dev, count, ray_keys, ray_hist);
        ray_scan_kernel<<<1, 1024, 0, st>>>(ray_hist);
        ray_scatter_kernel<<<grid_for(max_count), kBlock, 0, st>>>(q.ext_rays[from], q.ext_slot[from],
                                                                    q.ext_rays[from ^ 1], q.ext_slot[from ^ 1],
                                                                    ray_keys, ray_hist, count_dev, count);
    };
    // The bounce loop over extend queue 0 of `count` paths; bounce0 picks the
    // traversal kernels.  Sets e; returns a YAR_ERR_* for a traversal overflow.
    auto run_bounces = [&](const Render_Params& pp, uint32_t count, int bounce0) -> int {
        int cur = 0;
        for (int it = 0; count > 0 && it <= p.max_bounces + 1; it++) {
            const int bounce = bounce0 + it;
            if (sort_rays && it > 0) {
                sort_queue(cur, nullptr, count, count);
                cur ^= 1;
                launches += 3;
            }
            e = trace_extend(ctx, q, cur, count, bounce, st);
            if (e != cudaSuccess) break;
            cudaMemsetAsync(q.counters, 0, 3 * sizeof(uint32_t), st);
            order_queue(q, count, grid_for(count));
            if (guide && guide->before_shade && (guide->max_bounce <= 0 || bounce < guide->max_bounce)) {
                e = guide->before_shade(guide->user, q.ext_rays[cur], q.ext_hit4, q.ext_hit2, count, st);
                if (e != cudaSuccess) break;
                Guide_Shade gs;
                gs.lobes = guide->lobes;
                gs.queries = guide->queries;
                gs.alpha = guide->alpha;
                launch_shade<true>(pp, grid_for(count), st, S, cur, count, dptr<float>(B[2]), dptr<float2>(B[3]), ps,
                                   qo, gs);
                launches += 2;
            } else {
                launch_shade<false>(pp, grid_for(count), st, S, cur, count, dptr<float>(B[2]), dptr<float2>(B[3]), ps,
                                    qo, Guide_Shade{});
            }
            e = trace_light_queues(ctx, q, ps, count, bounce, st);
            if (e != cudaSuccess) break;
            connect_kernel<<<grid_for(count), kBlock, 0, st>>>(pp, S, q.ext_slot[cur], count, ps, nullptr);
            launches += mixed ? 7 : 5;
            uint32_t h[4];
            e = cudaMemcpyAsync(h, q.counters, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (h[3]) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
            rays_closest += count + h[2];
            rays_any += h[1];
            count = h[0];
            cur ^= 1;
        }
        return YAR_OK;
    };
    // The same bounces with the queue lengths on the device: every iteration
    // runs (the kernels exit on an empty queue); first_paths = 0 takes the
    // first count from counters[0] (a tail wave's queue).
    auto run_bounces_device = [&](const Render_Params& pp, uint32_t first_paths, uint32_t max_paths, int bounce0) {
        Queues qd = qo;
        qd.ext_count = q.counters + 7;
        const int grid = grid_for(max_paths);
        int cur = 0;
        for (int it = 0; it <= p.max_bounces + 1 && e == cudaSuccess; it++) {
            const int bounce = bounce0 + it;
            bounce_begin_kernel<<<1, 1, 0, st>>>(q.counters, it == 0 ? first_paths : 0u, rays_dev);
            if (sort_rays && it > 0) {
                sort_queue(cur, q.counters + 7, 0u, max_paths);
                cur ^= 1;
                launches += 3;
            }
            Cast_Args a;
            a.rays = q.ext_rays[cur];
            a.count = q.counters + 7;
            a.n_max = max_paths;
            a.next_ray = q.counters + 4;
            a.err = reinterpret_cast<int*>(q.counters + 3);
            a.hit4 = q.ext_hit4;
            a.hit2 = q.ext_hit2;
            e = launch_extend(ctx->ds, a, render_choice(ctx, 0, bounce), st);
            if (e != cudaSuccess) break;
            order_queue(qd, max_paths, grid);
            launch_shade<false>(pp, grid, st, S, cur, max_paths, dptr<float>(B[2]), dptr<float2>(B[3]), ps, qd,
                                Guide_Shade{});
            Cast_Args sh;
            sh.rays = q.shd_rays;
            sh.count = q.counters + 1;
            sh.n_max = max_paths;
            sh.perm = q.shd_slot;
            sh.next_ray = q.counters + 5;
            sh.err = reinterpret_cast<int*>(q.counters + 3);
            sh.occluded = ps.occluded;
            e = launch_shadow(ctx->ds, sh, render_choice(ctx, 1, bounce), st);
            if (e != cudaSuccess) break;
            Cast_Args pr;
            pr.rays = q.prb_rays;
            pr.count = q.counters + 2;
            pr.n_max = max_paths;
            pr.perm = q.prb_slot;
            pr.next_ray = q.counters + 6;
            pr.err = reinterpret_cast<int*>(q.counters + 3);
            pr.hit4 = ps.probe_hit4;
            pr.hit2 = ps.probe_hit2;
            e = launch_extend(ctx->ds, pr, render_choice(ctx, 0, bounce), st);
            if (e != cudaSuccess) break;
            connect_kernel<<<grid, kBlock, 0, st>>>(pp, S, q.ext_slot[cur], max_paths, ps, nullptr, q.counters + 7);
            launches += mixed ? 8 : 6;
            cur ^= 1;
        }
        bounce_begin_kernel<<<1, 1, 0, st>>>(q.counters, 0u, rays_dev);  // adds the last bounce's rays
        launches++;
        if (e == cudaSuccess) e = cudaGetLastError();
    };
    for (uint64_t first = 0; first < pixels && e == cudaSuccess; first += chunk_pixels) {
        const uint32_t cp = (uint32_t)std::min<uint64_t>(chunk_pixels, pixels - first);
        const uint32_t paths = cp * (uint32_t)p.spp;
        ps.chunk_first = (uint32_t)first;
        launch_generate(p, (uint32_t)first, cp, dptr<float>(B[2]), dptr<float>(B[3]), image_samples, ps, q, st);
        launches++;
        if (device_driven) {
            run_bounces_device(p, paths, paths, 0);
        } else if (int rc1 = run_bounces(p, paths, 0)) {
            return rc1;
        }
        if (e != cudaSuccess) break;
        if (p.exact_tail) {
            uint32_t* list = dptr<uint32_t>(B[32]);
            uint32_t* deferred_count = dptr<uint32_t>(B[33]);
            uint32_t* stream_pos = dptr<uint32_t>(B[34]);
            uint32_t* tail = dptr<uint32_t>(B[35]);
            cudaMemsetAsync(tail, 0, 2 * sizeof(uint32_t), st);
            tail_rank_kernel<<<grid_for(cp), kBlock, 0, st>>>(p, cp, ps, list, deferred_count, stream_pos, tail);
            launches++;
            uint32_t ht[2];
            e = cudaMemcpyAsync(ht, tail, sizeof(ht), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (ht[1]) return fail(ctx, YAR_ERR_INVALID, "a path drew past the sampler budget before its deferral");
            for (uint32_t wave = 0; wave < ht[0] && e == cudaSuccess; wave++) {
                cudaMemsetAsync(q.counters, 0, sizeof(uint32_t), st);
                tail_wave_kernel<<<grid_for(cp), kBlock, 0, st>>>(p_wave, (uint32_t)first, cp, wave, ps, q, list,
                                                                  deferred_count, stream_pos);
                launches++;
                if (device_driven) {  // at most one deferred sample per pixel and wave
                    run_bounces_device(p_wave, 0u, cp, yar_gpu_ctx::kBounceBuckets - 1);
                    continue;
                }
                uint32_t n = 0;
                e = cudaMemcpyAsync(&n, q.counters, sizeof(n), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) break;
                if (int rc1 = run_bounces(p_wave, n, yar_gpu_ctx::kBounceBuckets - 1)) return rc1;
            }
            if (e != cudaSuccess) break;
        }
        finish_chunk_kernel<<<grid_for(paths), kBlock, 0, st>>>(paths, first * p.spp, ps, radiance);
        launches++;
    }
    if (e == cudaSuccess) {
        samples_kernel<<<(uint32_t)((pixels + kBlock - 1) / kBlock), kBlock, 0, st>>>(p, radiance, dptr<double>(B[27]));
        // the tile sums (one sequential FP64 chain per 64 x 64 tile, the
        // reference's order) run on a second stream beside the film
        if (!ctx->aux_stream) e = cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess && !ctx->aux_fork) e = cudaEventCreateWithFlags(&ctx->aux_fork, cudaEventDisableTiming);
        if (e == cudaSuccess && !ctx->aux_join) e = cudaEventCreateWithFlags(&ctx->aux_join, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->aux_fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->aux_stream, ctx->aux_fork, 0);
        if (e == cudaSuccess)
            tile_variance_kernel<<<p.tiles_x * p.tiles_y, kTileVarThreads, 0, ctx->aux_stream>>>(
                p, dptr<double>(B[27]), dptr<double>(B[28]));
        launches += 2;
        if (e == cudaSuccess && !tiles_out) {
            film_kernel<<<(uint32_t)(((uint64_t)p.rw * p.rh + kBlock - 1) / kBlock), kBlock, 0, st>>>(
                p, radiance, image_samples, dptr<float>(B[29]));
            launches++;
        }
        if (e == cudaSuccess) e = cudaEventRecord(ctx->aux_join, ctx->aux_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->aux_join, 0);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    std::vector<double> tile_var((size_t)p.tiles_x * p.tiles_y);
    if (e == cudaSuccess && tiles_out) {
        // per-tile Film_Pixel arrays: offsets from the tiles' pixel bounds (Film::get_tile_bounds)
        const int n_tiles = p.tiles_x * p.tiles_y;
        tiles_out->offset.assign(n_tiles + 1, 0);
        uint32_t max_area = 0;
        for (int t = 0; t < n_tiles; t++) {
            int b[4];
            host_tile_pixel_bounds(p, t, b);
            const uint32_t area = (uint32_t)std::max(0, b[2] - b[0]) * (uint32_t)std::max(0, b[3] - b[1]);
            tiles_out->offset[t + 1] = tiles_out->offset[t] + area;
            max_area = std::max(max_area, area);
        }
        Device_Buffer offs, pix;
        int rc2 = device_alloc(ctx, offs, tiles_out->offset.size() * sizeof(uint32_t));
        if (rc2 == YAR_OK) rc2 = device_alloc(ctx, pix, std::max<size_t>(1, tiles_out->offset[n_tiles]) * sizeof(float4));
        if (rc2 != YAR_OK) {
            device_free(offs);
            device_free(pix);
            return rc2;
        }
        tiles_out->pixels.resize(tiles_out->offset[n_tiles]);
        e = cudaMemcpyAsync(offs.ptr, tiles_out->offset.data(), tiles_out->offset.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && max_area > 0) {
            tile_film_kernel<<<dim3((max_area + kBlock - 1) / kBlock, (unsigned)n_tiles), kBlock, 0, st>>>(
                p, radiance, image_samples, dptr<uint32_t>(offs), dptr<float4>(pix));
            launches++;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && !tiles_out->pixels.empty())
            e = cudaMemcpyAsync(tiles_out->pixels.data(), pix.ptr, tiles_out->pixels.size() * sizeof(float4),
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        device_free(offs);
        device_free(pix);
    }
    if (e == cudaSuccess && !tiles_out)
        e = cudaMemcpyAsync(rgb_out, B[29].ptr, (size_t)p.rw * p.rh * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tile_var.data(), B[28].ptr, tile_var.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    uint32_t err_word = 0;
    unsigned long long rays_h[2] = {0, 0};
    if (device_driven && e == cudaSuccess)
        e = cudaMemcpyAsync(&err_word, q.counters + 3, sizeof(err_word), cudaMemcpyDeviceToHost, st);
    if (device_driven && e == cudaSuccess) e = cudaMemcpyAsync(rays_h, rays_dev, sizeof(rays_h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
    if (err_word) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
    if (device_driven) {
        rays_closest = rays_h[0];
        rays_any = rays_h[1];
    } else if (!guide) {
        finish_render_tuning(ctx);
        ctx->render_tuned = true;
    }
    if (tiles_out) tiles_out->tile_variance = tile_var;
    const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    if (stats) {
        double acc = 0.0;
        int64_t count = 0;
        for (int t = 0; t < p.tiles_x * p.tiles_y; t++) {
            acc += tile_var[t];
            const int tx = t % p.tiles_x, ty = t / p.tiles_x;
            const int w = std::min(kTile, p.sw - tx * kTile), h = std::min(kTile, p.sh - ty * kTile);
            count += (int64_t)w * h;
        }
        stats->variance = p.spp > 1 ? acc / (double)count : 0.0;
        stats->seconds = (float)seconds;
        stats->paths = samples;
        stats->rays_closest = rays_closest;
        stats->rays_any = rays_any;
        stats->kernel_launches = launches;
    }
    return YAR_OK;
}

int render_guided_stratified(yar_gpu_ctx* ctx, int nx, int ny, uint32_t stream_hi, const Guide_Render_Hook& hook,
                             float* rgb_out, yar_render_stats* stats) {
    if (!rgb_out || nx < 1 || nx > 256 || ny < 1 || ny > 256 || stream_hi == 0)
        return fail(ctx, YAR_ERR_INVALID, "guided stratified render: arguments");
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    p.nx = nx;
    p.ny = ny;
    p.spp = nx * ny;
    p.stream_hi = stream_hi;  // own pixel streams: draws past the budget from one pcg stream per sample
    if (hook.chunk_paths < (uint64_t)p.spp) return fail(ctx, YAR_ERR_CAPACITY, "guided stratified render: chunk");
    return render_run_params(ctx, p, rgb_out, stats, nullptr, &hook);
}

// ---------------------------------------------------------------- render without allocation
// yar_gpu_render_static: the same kernels as render_run, with every working
// buffer carved out of one static device array instead of cudaMalloc'ed.
// Rendering is chunked by the space left after the per-sample film data, so
// the result is the same as render_run's (per-path results do not depend on
// the chunking).
namespace {

static __device__ __align__(256) unsigned char g_static_arena[YAR_GPU_STATIC_ARENA_BYTES];

std::mutex g_arena_mutex;
unsigned char* g_arena_address[64] = {};  // device address of g_static_arena per device ordinal

struct Arena {
    unsigned char* base;
    size_t size, used;
    template <class T>
    T* take(size_t count) {
        used = (used + 255) & ~(size_t)255;
        const size_t bytes = count * sizeof(T);
        if (bytes > size || used > size - bytes) return nullptr;
        T* p = reinterpret_cast<T*>(base + used);
        used += bytes;
        return p;
    }
};

} // namespace

int render_run_static(yar_gpu_ctx* ctx, float* rgb_out_device, yar_render_stats* stats) {
    if (!rgb_out_device) return fail(ctx, YAR_ERR_INVALID, "null image buffer");
    if (ctx->render.config.rendering_algorithm == 0)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "the static render runs the path tracer only (rendering_algorithm 1)");
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    // draws past the sampler budget from the pixel's own stream, as render_run_params
    p.exact_tail = (p.stream_hi == 0 && p.n1d > 0) ? 1 : 0;
    Render_Params p_wave = p;
    p_wave.exact_tail = 2;
    if (p.textured) return fail(ctx, YAR_ERR_UNSUPPORTED, "the static render does not evaluate image textures or bump maps");

    cudaSetDevice(ctx->device);
    if (ctx->device < 0 || ctx->device >= 64) return fail(ctx, YAR_ERR_INVALID, "device ordinal above 63");
    unsigned char* arena_base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_arena_mutex);
        if (!g_arena_address[ctx->device]) {
            void* addr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&addr, g_static_arena);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(static render arena)");
            g_arena_address[ctx->device] = static_cast<unsigned char*>(addr);
        }
        arena_base = g_arena_address[ctx->device];
    }
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t pixels = (uint64_t)p.sw * p.sh;
    const uint64_t samples = pixels * p.spp;
    const uint64_t tiles = (uint64_t)p.tiles_x * p.tiles_y;

    // film data for the whole image first, then as many paths per chunk as fit
    Arena A{arena_base, YAR_GPU_STATIC_ARENA_BYTES, 0};
    float4* radiance = A.take<float4>(samples);
    float2* image_samples = A.take<float2>(samples);
    double* pixel_variance = A.take<double>(pixels);
    double* tile_variance = A.take<double>(tiles);
    double* variance_total = A.take<double>(1);
    uint32_t* counters = A.take<uint32_t>(8);
    uint32_t* tail = A.take<uint32_t>(2);
    const int kChunkBuffers = 29;
    // per path: sample tables, path state (157 B), queues (168 B) and, for the
    // exact tail, the draw count, the deferred ray and the per-pixel list (40 B)
    // plus two words per pixel
    const size_t per_path = 4 * (size_t)std::max(1, p.n1d) + 8 * (size_t)std::max(1, p.n2d) + 157 + 168 +
                            (p.exact_tail ? 40 + (8 + p.spp - 1) / p.spp : 0);
    const size_t left = (radiance && image_samples && pixel_variance && tile_variance && variance_total && counters &&
                         tail && A.size > A.used + 256 * kChunkBuffers)
                            ? A.size - A.used - 256 * kChunkBuffers
                            : 0;
    const uint64_t chunk_pixels = std::min<uint64_t>(pixels, left / per_path / p.spp);
    if (chunk_pixels == 0)
        return fail(ctx, YAR_ERR_CAPACITY,
                    "render of " + std::to_string(samples) + " samples does not fit the " +
                        std::to_string(YAR_GPU_STATIC_ARENA_BYTES >> 20) + " MiB static arena");
    const uint64_t cap = chunk_pixels * p.spp;
    float* s1d = A.take<float>(cap * std::max(1, p.n1d));
    float2* s2d = A.take<float2>(cap * std::max(1, p.n2d));
    Path_State ps{A.take<float4>(cap), A.take<float4>(cap), A.take<uint32_t>(cap), A.take<uint4>(cap),
                  A.take<float4>(cap), A.take<float4>(cap), A.take<float4>(cap), A.take<float4>(cap),
                  A.take<float4>(cap), A.take<uint8_t>(cap), A.take<float4>(cap), A.take<uint2>(cap)};
    Queues q{};
    q.ext_rays[0] = A.take<float4>(2 * cap);
    q.ext_rays[1] = A.take<float4>(2 * cap);
    q.ext_slot[0] = A.take<uint32_t>(cap);
    q.ext_slot[1] = A.take<uint32_t>(cap);
    q.ext_hit4 = A.take<float4>(cap);
    q.ext_hit2 = A.take<uint2>(cap);
    q.shd_rays = A.take<float4>(2 * cap);
    q.shd_slot = A.take<uint32_t>(cap);
    q.prb_rays = A.take<float4>(2 * cap);
    q.prb_slot = A.take<uint32_t>(cap);
    q.counters = counters;
    uint32_t *list = nullptr, *deferred_count = nullptr, *stream_pos = nullptr;
    if (p.exact_tail) {
        ps.rng_draws = A.take<uint32_t>(cap);
        ps.deferred = A.take<float4>(2 * cap);
        list = A.take<uint32_t>(cap);
        deferred_count = A.take<uint32_t>(chunk_pixels);
        stream_pos = A.take<uint32_t>(chunk_pixels);
        if (!ps.rng_draws || !ps.deferred || !list || !deferred_count || !stream_pos)
            return fail(ctx, YAR_ERR_CAPACITY, "static arena layout overflow");
    }
    ps.image_samples = image_samples;
    if (!s1d || !s2d || !ps.probe_hit2 || !q.prb_slot)
        return fail(ctx, YAR_ERR_CAPACITY, "static arena layout overflow");
    Scene_Dev S = scene_dev(ctx->ds, ctx->render);

    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemsetAsync(q.counters, 0, 8 * sizeof(uint32_t), st);  // the arena keeps the last call's data
    uint64_t rays_closest = 0, rays_any = 0;
    uint32_t launches = 0;
    auto run_bounces = [&](const Render_Params& pp, uint32_t count, int bounce0) -> int {
        int cur = 0;
        for (int it = 0; count > 0 && it <= p.max_bounces + 1; it++) {
            const int bounce = bounce0 + it;
            e = trace_extend(ctx, q, cur, count, bounce, st);
            if (e != cudaSuccess) break;
            cudaMemsetAsync(q.counters, 0, 3 * sizeof(uint32_t), st);
            launch_shade<false>(pp, grid_for(count), st, S, cur, count, s1d, s2d, ps, q, Guide_Shade{});
            e = trace_light_queues(ctx, q, ps, count, bounce, st);
            if (e != cudaSuccess) break;
            connect_kernel<<<grid_for(count), kBlock, 0, st>>>(pp, S, q.ext_slot[cur], count, ps, nullptr);
            launches += 5;
            uint32_t h[4];
            e = cudaMemcpyAsync(h, q.counters, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (h[3]) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
            rays_closest += count + h[2];
            rays_any += h[1];
            count = h[0];
            cur ^= 1;
        }
        return YAR_OK;
    };
    for (uint64_t first = 0; first < pixels && e == cudaSuccess; first += chunk_pixels) {
        const uint32_t cp = (uint32_t)std::min<uint64_t>(chunk_pixels, pixels - first);
        const uint32_t paths = cp * (uint32_t)p.spp;
        ps.chunk_first = (uint32_t)first;
        launch_generate(p, (uint32_t)first, cp, s1d, reinterpret_cast<float*>(s2d), image_samples, ps, q, st);
        launches++;
        if (int rc1 = run_bounces(p, paths, 0)) return rc1;
        if (e != cudaSuccess) break;
        if (p.exact_tail) {  // the waves of deferred samples, as render_run_params runs them
            cudaMemsetAsync(tail, 0, 2 * sizeof(uint32_t), st);
            tail_rank_kernel<<<grid_for(cp), kBlock, 0, st>>>(p, cp, ps, list, deferred_count, stream_pos, tail);
            launches++;
            uint32_t ht[2];
            e = cudaMemcpyAsync(ht, tail, sizeof(ht), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (ht[1]) return fail(ctx, YAR_ERR_INVALID, "a path drew past the sampler budget before its deferral");
            for (uint32_t wave = 0; wave < ht[0] && e == cudaSuccess; wave++) {
                cudaMemsetAsync(q.counters, 0, sizeof(uint32_t), st);
                tail_wave_kernel<<<grid_for(cp), kBlock, 0, st>>>(p_wave, (uint32_t)first, cp, wave, ps, q, list,
                                                                  deferred_count, stream_pos);
                launches++;
                uint32_t n = 0;
                e = cudaMemcpyAsync(&n, q.counters, sizeof(n), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) break;
                if (int rc1 = run_bounces(p_wave, n, yar_gpu_ctx::kBounceBuckets - 1)) return rc1;
            }
            if (e != cudaSuccess) break;
        }
        finish_chunk_kernel<<<grid_for(paths), kBlock, 0, st>>>(paths, first * p.spp, ps, radiance);
        launches++;
    }
    double variance = 0.0;
    if (e == cudaSuccess) {
        samples_kernel<<<(uint32_t)((pixels + kBlock - 1) / kBlock), kBlock, 0, st>>>(p, radiance, pixel_variance);
        tile_variance_kernel<<<(uint32_t)tiles, kTileVarThreads, 0, st>>>(p, pixel_variance, tile_variance);
        variance_total_kernel<<<1, 1, 0, st>>>(p, tile_variance, variance_total);
        film_kernel<<<(uint32_t)(((uint64_t)p.rw * p.rh + kBlock - 1) / kBlock), kBlock, 0, st>>>(
            p, radiance, image_samples, rgb_out_device);
        launches += 4;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&variance, variance_total, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "static render");
    if (stats) {
        stats->variance = variance;
        stats->seconds = (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->paths = samples;
        stats->rays_closest = rays_closest;
        stats->rays_any = rays_any;
        stats->kernel_launches = launches;
    }
    return YAR_OK;
}

// ---------------------------------------------------------------- checkpointed render
// render_scene with a checkpoint directory (src/ref/reference_renderer.cpp:180-324,
// :446-476, :479-584), in the reference's file format: a "checkpoint" metadata
// file (input file name, tile count, samples per pixel) and one "tile_NNNN" file
// per finished tile: render time (float), variance accumulator (double), pixel
// bounds (4 x int32), Film_Pixel[area] (color sum rgb, weight sum).  Tiles
// already in the directory are loaded; the others are rendered one row of tiles
// at a time and written as soon as their row is done (a temporary file renamed
// into place); the image merges all tiles in index order, as Film::merge_tile
// and Film::get_image do.
namespace {
namespace fs = std::filesystem;

std::string format_tile_index(int tile_index) {  // reference_renderer.cpp:153-158
    std::string s = std::to_string(tile_index);
    s.insert(0, s.length() <= 4 ? 4 - s.length() : 0, '0');
    return s;
}

struct Checkpoint_Tile {
    bool present = false;
    double variance = 0.0;
    int bounds[4] = {0, 0, 0, 0};
    std::vector<float4> pixels;  // color sum rgb, weight sum
};

bool write_tile_file(const fs::path& dir, int tile_index, float time, const Checkpoint_Tile& t, std::string& err) {
    const fs::path temp = dir / ("temp_tile_" + format_tile_index(tile_index));
    const fs::path final_path = dir / ("tile_" + format_tile_index(tile_index));
    {
        std::ofstream f(temp, std::ofstream::out | std::ofstream::binary);
        if (!f) {
            err = "failed to create file: " + temp.string();
            return false;
        }
        f.write(reinterpret_cast<const char*>(&time), sizeof(float));
        f.write(reinterpret_cast<const char*>(&t.variance), sizeof(double));
        f.write(reinterpret_cast<const char*>(t.bounds), 4 * sizeof(int32_t));
        f.write(reinterpret_cast<const char*>(t.pixels.data()), (std::streamsize)(t.pixels.size() * sizeof(float4)));
        if (!f) {
            err = "failed to write to file: " + temp.string();
            return false;
        }
    }
    std::error_code ec;
    if (fs::exists(final_path, ec)) {
        err = "tile file already exists: " + final_path.string();
        return false;
    }
    fs::rename(temp, final_path, ec);
    if (ec) {
        err = "failed to rename temp file to: " + final_path.string();
        return false;
    }
    return true;
}

// start_or_resume_checkpoint: creates the directory and its metadata, or checks
// the metadata and loads the finished tiles.  Returns an empty string or the error.
std::string start_or_resume(const fs::path& dir, const std::string& input_filename, int tile_count, int spp,
                            std::vector<Checkpoint_Tile>& tiles, float* previous_time) {
    std::error_code ec;
    const fs::path meta = dir / "checkpoint";
    *previous_time = 0.f;
    if (!fs::exists(dir, ec) && !fs::create_directories(dir, ec))
        return "failed to create checkpoint directory: " + dir.string();
    if (fs::is_empty(dir, ec)) {
        std::ofstream f(meta, std::ofstream::out);
        if (!f) return "failed to create checkpoint file: " + meta.string();
        f << "input_filename " << input_filename << "\n";
        f << "total_tile_count " << tile_count << "\n";
        f << "samples_per_pixer " << spp << "\n";  // the reference's spelling
        return "";
    }
    if (!fs::exists(meta, ec)) return dir.string() + " is not a checkpoint directory: 'checkpoint' file is missing";
    std::ifstream f(meta);
    std::string tag, stored_name, stored_tiles, stored_spp;
    f >> tag >> stored_name >> tag >> stored_tiles >> tag >> stored_spp;
    if (!f) return "failed to read all the required fields from the metadata file: " + meta.string();
    if (stored_name != input_filename) return "can not resume rendering because input_filename is changed";
    if (stored_tiles != std::to_string(tile_count))
        return "can not resume rendering because total_tile_count is changed";
    if (stored_spp != std::to_string(spp)) return "can not resume rendering because samples_per_pixer is changed";
    for (const fs::directory_entry& entry : fs::directory_iterator(dir, ec)) {
        const std::string name = entry.path().stem().string();
        if (name.rfind("tile_", 0) != 0) continue;
        char* end = nullptr;
        const long index = std::strtol(name.c_str() + 5, &end, 10);
        if (!end || *end != '\0' || index < 0 || index >= tile_count) return "unexpected tile file: " + name;
        std::ifstream tf(entry.path(), std::ifstream::in | std::ifstream::binary);
        std::vector<char> content((std::istreambuf_iterator<char>(tf)), std::istreambuf_iterator<char>());
        Checkpoint_Tile& t = tiles[index];
        float time = 0.f;
        if (content.size() < 28) return "truncated tile file: " + name;
        memcpy(&time, content.data(), 4);
        memcpy(&t.variance, content.data() + 4, 8);
        memcpy(t.bounds, content.data() + 12, 16);
        const int64_t area = (int64_t)std::max(0, t.bounds[2] - t.bounds[0]) * std::max(0, t.bounds[3] - t.bounds[1]);
        if ((int64_t)content.size() != 28 + 16 * area) return "tile file of the wrong size: " + name;
        t.pixels.resize((size_t)area);
        memcpy(t.pixels.data(), content.data() + 28, (size_t)area * 16);
        t.present = true;
        *previous_time = std::max(*previous_time, time);
    }
    return "";
}

} // namespace

int render_checkpoint(yar_gpu_ctx* ctx, const char* directory, const char* input_filename, float* rgb_out,
                      yar_render_stats* stats) {
    if (!rgb_out || !directory || !input_filename) return fail(ctx, YAR_ERR_INVALID, "null argument");
    if (ctx->render.config.rendering_algorithm == 0)
        return fail(ctx, YAR_ERR_UNSUPPORTED, "checkpointed renders run the path tracer only (rendering_algorithm 1)");
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    const auto t_start = std::chrono::steady_clock::now();
    const int tile_count = p.tiles_x * p.tiles_y;
    std::vector<Checkpoint_Tile> tiles(tile_count);
    float previous_time = 0.f;
    const std::string err = start_or_resume(fs::path(directory), input_filename, tile_count, p.spp, tiles,
                                            &previous_time);
    if (!err.empty()) return fail(ctx, YAR_ERR_IO, "checkpoint: " + err);
    yar_render_stats total{};
    for (int ty = 0; ty < p.tiles_y; ty++) {
        bool needed = false;
        for (int tx = 0; tx < p.tiles_x; tx++) needed = needed || !tiles[ty * p.tiles_x + tx].present;
        if (!needed) continue;
        // one row of tiles: the render over its sample rows
        Render_Params band = p;
        band.sy0 = p.sy0 + ty * kTile;
        band.sh = std::min(kTile, p.sh - ty * kTile);
        band.tiles_y = 1;
        Tile_Output out;
        yar_render_stats bs{};
        int rc = render_run_params(ctx, band, nullptr, &bs, &out);
        if (rc != YAR_OK) return rc;
        total.paths += bs.paths;
        total.rays_closest += bs.rays_closest;
        total.rays_any += bs.rays_any;
        total.kernel_launches += bs.kernel_launches;
        const float now = previous_time +
                          (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        for (int tx = 0; tx < p.tiles_x; tx++) {
            Checkpoint_Tile& t = tiles[ty * p.tiles_x + tx];
            if (t.present) continue;
            host_tile_pixel_bounds(p, ty * p.tiles_x + tx, t.bounds);
            t.variance = out.tile_variance[tx];
            t.pixels.assign(out.pixels.begin() + out.offset[tx], out.pixels.begin() + out.offset[tx + 1]);
            t.present = true;
            std::string werr;
            if (!write_tile_file(fs::path(directory), ty * p.tiles_x + tx, now, t, werr))
                return fail(ctx, YAR_ERR_IO, "checkpoint: " + werr);
        }
    }
    // Film::merge_tile in tile order, then Film::get_image (box filter)
    std::vector<float4> film((size_t)p.rw * p.rh, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int t = 0; t < tile_count; t++) {
        const Checkpoint_Tile& tile = tiles[t];
        const int w = tile.bounds[2] - tile.bounds[0];
        for (int y = tile.bounds[1]; y < tile.bounds[3]; y++)
            for (int x = tile.bounds[0]; x < tile.bounds[2]; x++) {
                const float4 c = tile.pixels[(size_t)(y - tile.bounds[1]) * w + (x - tile.bounds[0])];
                float4& f = film[(size_t)(y - p.ry0) * p.rw + (x - p.rx0)];
                f.x += c.x;
                f.y += c.y;
                f.z += c.z;
                f.w += c.w;
            }
    }
    for (size_t i = 0; i < film.size(); i++) {
        const float4 f = film[i];
        float cr = 0.f, cg = 0.f, cb = 0.f;
        if (f.w != 0.f) {
            const float inv = 1.f / f.w;
            cr = f.x * inv;
            cg = f.y * inv;
            cb = f.z * inv;
        }
        rgb_out[3 * i + 0] = std::max(0.f, cr);
        rgb_out[3 * i + 1] = std::max(0.f, cg);
        rgb_out[3 * i + 2] = std::max(0.f, cb);
    }
    if (stats) {
        double acc = 0.0;
        int64_t count = 0;
        for (int t = 0; t < tile_count; t++) {
            acc += tiles[t].variance;
            const int tx = t % p.tiles_x, ty = t / p.tiles_x;
            count += (int64_t)std::min(kTile, p.sw - tx * kTile) * std::min(kTile, p.sh - ty * kTile);
        }
        *stats = total;
        stats->variance = p.spp > 1 ? acc / (double)count : 0.0;
        stats->seconds = previous_time +
                         (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
    return YAR_OK;
}

} // namespace yar

extern "C" int yar_gpu_render_checkpoint(yar_gpu_ctx* ctx, const char* checkpoint_directory,
                                         const char* input_filename, float* rgb_out, yar_render_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return yar::fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    return yar::render_checkpoint(ctx, checkpoint_directory, input_filename, rgb_out, stats);
}

extern "C" int yar_gpu_render_static(yar_gpu_ctx* ctx, float* rgb_out_device, yar_render_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return yar::fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    return yar::render_run_static(ctx, rgb_out_device, stats);
}

extern "C" int yar_gpu_render(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats) {
    if (!ctx) return YAR_ERR_INVALID;
    if (!ctx->has_scene) return yar::fail(ctx, YAR_ERR_NO_SCENE, "no scene uploaded");
    return yar::render_run(ctx, rgb_out, stats);
}
