// ref_flatten.hpp - the reference-side adapter of the C ABI: flatten() turns
// a reference Scene + Scene_Context (the reference's pbrt-v3 loader and
// kd-tree builder, as init_scene_context left them) into the flat scene
// (include/yar_gpu.h) that yar_gpu_upload_scene consumes.  Compiled against
// the reference's own headers by oracle/build_ref.sh, into the reference
// harness (yar_ref) and into the drop-in render_scene_gpu (yar_ref_gpu).
#pragma once

#include "lib/common.h"
#include "lib/scene.h"
#include "lib/scene_object.h"
#include "lib/triangle_mesh.h"
#include "ref/camera.h"
#include "ref/scene_context.h"

#include "yfs.hpp"

namespace {

void matrix_to_floats(const Matrix3x4& m, float out[12]) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) out[r * 4 + c] = m.a[r][c];
}

Matrix3x4 floats_to_matrix(const float in[12]) {
    Matrix3x4 m;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) m.a[r][c] = in[r * 4 + c];
    return m;
}

// Parameters of the material being flattened that a texture gives and the
// library does not evaluate (counted into yar_material_desc::other_textured_parameters).
static uint32_t g_textured_parameters = 0;

bool constant_rgb(const Parameter& p, float out[3]) {
    if (p.eval_mode != EvaluationMode::value || !p.value.is_constant) {
        if (p.eval_mode != EvaluationMode::none) g_textured_parameters++;
        return false;
    }
    out[0] = p.value.constant.r;
    out[1] = p.value.constant.g;
    out[2] = p.value.constant.b;
    return true;
}

bool constant_float(const Parameter& p, float* out) {
    float c[3];
    if (!constant_rgb(p, c)) return false;
    *out = c[0];
    return true;
}

// An RGB parameter: its constant, or (value mode, texture leaf) its texture
// and uv scale; any other form is counted as not evaluated.
void constant_or_texture(const RGB_Parameter& p, float out[3], uint32_t* texture, float uv_scale[2]) {
    if (p.eval_mode == EvaluationMode::value && !p.value.is_constant) {
        *texture = (uint32_t)p.value.texture.texture_index + 1u;
        uv_scale[0] = p.value.texture.u_scale;
        uv_scale[1] = p.value.texture.v_scale;
        return;
    }
    constant_rgb(p, out);
}

// The bump map of a material (Shading_Context::apply_bump_map runs in create_bsdf
// and, for the delta-capable materials, in check_for_delta_scattering_event).
void flatten_bump(const Float_Parameter& bump_map, yar_material_desc& d) {
    if (bump_map.eval_mode == EvaluationMode::none) return;
    if (bump_map.eval_mode == EvaluationMode::value) {
        if (bump_map.value.is_constant) {
            d.bump = 1;
            d.bump_height = bump_map.value.constant.r;
        } else {
            d.bump = 2;
            d.bump_texture = (uint32_t)bump_map.value.texture.texture_index + 1u;
            d.bump_uv_scale[0] = bump_map.value.texture.u_scale;
            d.bump_uv_scale[1] = bump_map.value.texture.v_scale;
        }
        return;
    }
    g_textured_parameters++;
}

void push_material(yfs::Scene& out, yar_material_desc d) {
    d.other_textured_parameters = g_textured_parameters;
    g_textured_parameters = 0;
    out.materials.push_back(d);
}

// The C-ABI adapter: reference Scene/Scene_Context -> flat scene.
yfs::Scene flatten(const Scene& scene, const Scene_Context& ctx) {
    yfs::Scene out;
    const auto& meshes = scene.geometries.triangle_meshes;
    for (size_t i = 0; i < meshes.size(); i++) {
        const Triangle_Mesh& m = meshes[i];
        yfs::Mesh fm;
        fm.vertices.resize(m.vertices.size() * 3);
        memcpy(fm.vertices.data(), m.vertices.data(), fm.vertices.size() * 4);
        fm.normals.resize(m.normals.size() * 3);
        if (!m.normals.empty()) memcpy(fm.normals.data(), m.normals.data(), fm.normals.size() * 4);
        fm.uvs.resize(m.uvs.size() * 2);
        if (!m.uvs.empty()) memcpy(fm.uvs.data(), m.uvs.data(), fm.uvs.size() * 4);
        fm.indices = m.indices;
        fm.reverse_orientation = m.reverse_geometric_normal_orientation ? 1 : 0;
        fm.visibility = (int32_t)m.visibility;
        fm.alpha_texture = m.alpha_texture_index >= 0 ? (uint32_t)m.alpha_texture_index + 1u : 0u;
        const KdTree& t = ctx.kdtree_data.geometry_kdtrees[i];
        memcpy(fm.bounds, &t.bounds.min_p.x, 12);
        memcpy(fm.bounds + 3, &t.bounds.max_p.x, 12);
        fm.nodes.resize(t.nodes.size());
        memcpy(fm.nodes.data(), t.nodes.data(), t.nodes.size() * 8);
        out.meshes.push_back(std::move(fm));
    }
    // materials: diffuse, metal, glass, plastic, coated diffuse, perfect reflector, perfect refractor,
    // diffuse transmission, pbrt3 translucent, pbrt3 uber, pbrt3 fourier, mix flattened in that order
    std::vector<int> diffuse_index, metal_index, glass_index;
    for (const Diffuse_Material& m : ctx.materials.diffuse) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_DIFFUSE;
        constant_or_texture(m.reflectance, d.reflectance, &d.reflectance_texture, d.reflectance_uv_scale);
        diffuse_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (const Metal_Material& m : ctx.materials.metal) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_METAL;
        constant_float(m.u_roughness, &d.u_roughness);
        constant_float(m.v_roughness, &d.v_roughness);
        constant_float(m.eta_i, &d.eta_i);
        constant_rgb(m.eta, d.eta);
        constant_rgb(m.k, d.k);
        d.roughness_is_alpha = m.roughness_is_alpha ? 1 : 0;
        metal_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (const Glass_Material& m : ctx.materials.glass) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_GLASS;
        constant_or_texture(m.reflectance, d.reflectance, &d.reflectance_texture, d.reflectance_uv_scale);
        constant_or_texture(m.transmittance, d.transmittance, &d.transmittance_texture, d.transmittance_uv_scale);
        constant_float(m.index_of_refraction, &d.index_of_refraction);
        constant_float(m.roughness, &d.u_roughness);
        d.v_roughness = d.u_roughness;
        d.roughness_is_alpha = m.roughness_is_alpha ? 1 : 0;
        glass_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    // plastic and coated diffuse: reflectance = diffuse reflectance, transmittance = r0
    std::vector<int> plastic_index, coated_index;
    for (const Plastic_Material& m : ctx.materials.plastic) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_PLASTIC;
        constant_or_texture(m.diffuse_reflectance, d.reflectance, &d.reflectance_texture, d.reflectance_uv_scale);
        float r0 = 0.f;
        constant_float(m.r0, &r0);
        d.transmittance[0] = d.transmittance[1] = d.transmittance[2] = r0;
        constant_float(m.roughness, &d.u_roughness);
        d.v_roughness = d.u_roughness;
        d.roughness_is_alpha = m.roughness_is_alpha ? 1 : 0;
        plastic_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (const Coated_Diffuse_Material& m : ctx.materials.coated_diffuse) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_COATED_DIFFUSE;
        constant_or_texture(m.diffuse_reflectance, d.reflectance, &d.reflectance_texture, d.reflectance_uv_scale);
        constant_rgb(m.r0, d.transmittance);
        constant_float(m.u_roughness, &d.u_roughness);
        constant_float(m.v_roughness, &d.v_roughness);
        d.roughness_is_alpha = m.roughness_is_alpha ? 1 : 0;
        coated_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    std::vector<int> reflector_index, refractor_index;
    for (const Perfect_Reflector_Material& m : ctx.materials.perfect_reflector) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);  // applied in check_for_delta_scattering_event
        d.type = YAR_MATERIAL_PERFECT_REFLECTOR;
        constant_rgb(m.reflectance, d.reflectance);
        reflector_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (const Perfect_Refractor_Material& m : ctx.materials.perfect_refractor) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);  // applied in check_for_delta_scattering_event
        d.type = YAR_MATERIAL_PERFECT_REFRACTOR;
        constant_float(m.index_of_refraction, &d.index_of_refraction);
        refractor_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    // diffuse transmission: reflectance, transmittance, diffuse = scale
    std::vector<int> transmission_index, translucent_index, uber_index, mix_index;
    for (const Diffuse_Transmission_Material& m : ctx.materials.diffuse_transmission) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_DIFFUSE_TRANSMISSION;
        constant_or_texture(m.reflectance, d.reflectance, &d.reflectance_texture, d.reflectance_uv_scale);
        constant_or_texture(m.transmittance, d.transmittance, &d.transmittance_texture, d.transmittance_uv_scale);
        constant_rgb(m.scale, d.diffuse);
        transmission_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (const Pbrt3_Translucent_Material& m : ctx.materials.pbrt3_translucent) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_PBRT3_TRANSLUCENT;
        constant_rgb(m.reflectance, d.reflectance);
        constant_rgb(m.transmittance, d.transmittance);
        constant_rgb(m.diffuse, d.diffuse);
        constant_rgb(m.specular, d.specular);
        constant_float(m.roughness, &d.u_roughness);
        d.v_roughness = d.u_roughness;
        translucent_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    // pbrt3 uber: reflectance = Kd, transmittance = Kt
    for (const Pbrt3_Uber_Material& m : ctx.materials.pbrt3_uber) {
        yar_material_desc d{};
        flatten_bump(m.bump_map, d);
        d.type = YAR_MATERIAL_PBRT3_UBER;
        constant_rgb(m.diffuse_reflectance, d.reflectance);
        constant_rgb(m.specular_reflectance, d.specular);
        constant_rgb(m.delta_reflectance, d.delta_reflectance);
        constant_rgb(m.delta_transmission, d.transmittance);
        constant_rgb(m.opacity, d.opacity);
        constant_float(m.u_roughness, &d.u_roughness);
        constant_float(m.v_roughness, &d.v_roughness);
        constant_float(m.index_of_refraction, &d.index_of_refraction);
        d.component_count = m.component_count;
        for (int k = 0; k < m.component_count; k++) d.components[k] = (uint32_t)m.components[k];
        uber_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    // pbrt3 fourier: the table as Pbrt3_Fourier_Material::load_bsdf_file read it
    std::vector<int> fourier_index;
    for (const Pbrt3_Fourier_Material& m : ctx.materials.pbrt3_fourier) {
        yar_material_desc d{};
        d.type = YAR_MATERIAL_PBRT3_FOURIER;
        yar_fourier_desc t{};
        t.node_count = (uint32_t)m.zenith_angle_discretization.size();
        t.channel_count = m.channel_count;
        t.max_order = m.max_order;
        t.eta = m.eta;
        t.nodes = out.fourier_floats.size();
        out.fourier_floats.insert(out.fourier_floats.end(), m.zenith_angle_discretization.begin(),
                                  m.zenith_angle_discretization.end());
        t.coeffs = out.fourier_floats.size();
        t.coeff_count = m.coeffs.size();
        out.fourier_floats.insert(out.fourier_floats.end(), m.coeffs.begin(), m.coeffs.end());
        t.series = out.fourier_uints.size();
        for (size_t k = 0; k < m.coeff_offset.size(); k++) {
            out.fourier_uints.push_back(m.coeff_offset[k]);
            out.fourier_uints.push_back(m.coeff_count[k]);
        }
        out.fourier_tables.push_back(t);
        d.fourier_table = (uint32_t)out.fourier_tables.size();
        fourier_index.push_back((int)out.materials.size());
        push_material(out, d);
    }
    for (size_t i = 0; i < ctx.materials.mix.size(); i++) {
        mix_index.push_back((int)out.materials.size() + (int)i);
    }
    auto flat_index = [&](Material_Handle h) -> int {
        switch (h.type) {
        case Material_Type::diffuse: return diffuse_index[h.index];
        case Material_Type::metal: return metal_index[h.index];
        case Material_Type::glass: return glass_index[h.index];
        case Material_Type::plastic: return plastic_index[h.index];
        case Material_Type::coated_diffuse: return coated_index[h.index];
        case Material_Type::perfect_reflector: return reflector_index[h.index];
        case Material_Type::perfect_refractor: return refractor_index[h.index];
        case Material_Type::diffuse_transmission: return transmission_index[h.index];
        case Material_Type::pbrt3_translucent: return translucent_index[h.index];
        case Material_Type::pbrt3_uber: return uber_index[h.index];
        case Material_Type::pbrt3_fourier: return fourier_index[h.index];
        case Material_Type::mix: return mix_index[h.index];
        default: return -1;
        }
    };
    // mix: the two materials by flat index, mix_amount
    for (const Mix_Material& m : ctx.materials.mix) {
        yar_material_desc d{};
        d.type = YAR_MATERIAL_MIX;
        d.mix_materials[0] = flat_index(m.material1);
        d.mix_materials[1] = flat_index(m.material2);
        constant_rgb(m.mix_amount, d.mix_amount);
        push_material(out, d);
    }
    for (const Scene_Object& o : scene.objects) {
        yar_object_desc d{};
        d.mesh_index = o.geometry.index;
        d.material_type = (uint32_t)o.material.type;
        d.material_index = o.material.type == Material_Type::null_material ? -1 : flat_index(o.material);
        if (o.material.type != Material_Type::null_material && d.material_index < 0)
            fprintf(stderr, "warning: material type %u not flattened\n", (unsigned)o.material.type);
        d.area_light_type = (uint32_t)o.area_light.type;
        d.area_light_index = o.area_light.index;
        matrix_to_floats(o.object_to_world_transform, d.object_to_world);
        matrix_to_floats(o.world_to_object_transform, d.world_to_object);
        matrix_to_floats(o.object_to_world_normal_transform, d.object_to_world_normal);
        out.objects.push_back(d);
    }
    const KdTree& st = ctx.kdtree_data.scene_kdtree;
    memcpy(out.scene_bounds, &st.bounds.min_p.x, 12);
    memcpy(out.scene_bounds + 3, &st.bounds.max_p.x, 12);
    out.scene_nodes.resize(st.nodes.size());
    memcpy(out.scene_nodes.data(), st.nodes.data(), st.nodes.size() * 8);

    for (const Diffuse_Rectangular_Light& l : ctx.lights.diffuse_rectangular_lights) {
        yar_rect_light_desc d{};
        matrix_to_floats(l.light_to_world_transform, d.light_to_world);
        d.emitted_radiance[0] = l.emitted_radiance.r;
        d.emitted_radiance[1] = l.emitted_radiance.g;
        d.emitted_radiance[2] = l.emitted_radiance.b;
        d.size[0] = l.size.x;
        d.size[1] = l.size.y;
        d.sample_count = l.sample_count;
        out.rect_lights.push_back(d);
    }
    // point, spot, directional lights in the reference's selection order
    for (const Point_Light& l : ctx.lights.point_lights) {
        yar_delta_light_desc d{};
        d.type = YAR_LIGHT_POINT;
        memcpy(d.position, &l.position.x, 12);
        memcpy(d.intensity, &l.intensity.r, 12);
        out.delta_lights.push_back(d);
    }
    for (const Spot_Light& l : ctx.lights.spot_lights) {
        yar_delta_light_desc d{};
        d.type = YAR_LIGHT_SPOT;
        memcpy(d.position, &l.position.x, 12);
        memcpy(d.direction, &l.direction.x, 12);
        memcpy(d.intensity, &l.intensity.r, 12);
        d.cone_angle = l.cone_angle;
        d.penumbra_angle = l.penumbra_angle;
        out.delta_lights.push_back(d);
    }
    for (const Directional_Light& l : ctx.lights.directional_lights) {
        yar_delta_light_desc d{};
        d.type = YAR_LIGHT_DIRECTIONAL;
        memcpy(d.direction, &l.direction.x, 12);
        memcpy(d.intensity, &l.irradiance.r, 12);
        out.delta_lights.push_back(d);
    }
    for (const Diffuse_Triangle_Mesh_Light& l : ctx.lights.diffuse_triangle_mesh_lights) {
        yar_mesh_light_desc d{};
        matrix_to_floats(l.light_to_world_transform, d.light_to_world);
        memcpy(d.emitted_radiance, &l.emitted_radiance.r, 12);
        d.triangle_mesh_index = l.triangle_mesh_index;
        out.mesh_lights.push_back(d);
    }
    for (const Diffuse_Sphere_Light& l : ctx.lights.diffuse_sphere_lights) {
        yar_sphere_light_desc d{};
        memcpy(d.position, &l.position.x, 12);
        memcpy(d.emitted_radiance, &l.emitted_radiance.r, 12);
        d.radius = l.radius;
        d.sample_count = l.sample_count;
        out.sphere_lights.push_back(d);
    }
    if (ctx.lights.has_environment_light) {
        const Environment_Light& l = ctx.lights.environment_light;
        const Image& map = ctx.textures[l.environment_map_index].get_mips()[0];
        out.has_environment = true;
        matrix_to_floats(l.light_to_world, out.environment.light_to_world);
        matrix_to_floats(l.world_to_light, out.environment.world_to_light);
        memcpy(out.environment.scale, &l.scale.r, 12);
        out.environment.sample_count = l.sample_count;
        out.environment.width = (uint32_t)map.width;
        out.environment.height = (uint32_t)map.height;
        out.environment_radiance.resize(3 * map.data.size());
        memcpy(out.environment_radiance.data(), map.data.data(), out.environment_radiance.size() * sizeof(float));
    }
    // image textures, when a flattened material or a mesh's alpha test reads
    // one: every texture of the scene context (indices stay the reference's),
    // each with its mip chain
    bool textured = false;
    for (const yar_material_desc& d : out.materials)
        textured = textured || d.reflectance_texture != 0 || d.transmittance_texture != 0 || d.bump_texture != 0;
    for (const yfs::Mesh& fm : out.meshes) textured = textured || fm.alpha_texture != 0;
    for (size_t ti = 0; textured && ti < ctx.textures.size(); ti++) {
        const std::vector<Image>& mips = ctx.textures[ti].get_mips();
        yar_texture_desc td{};
        td.first_mip = (uint32_t)out.texture_mips.size();
        td.mip_count = (uint32_t)mips.size();
        for (const Image& im : mips) {
            yar_texture_mip_desc md{};
            md.width = (uint32_t)im.width;
            md.height = (uint32_t)im.height;
            md.texel_offset = out.texels.size() / 3;
            out.texture_mips.push_back(md);
            const size_t at = out.texels.size();
            out.texels.resize(at + 3 * im.data.size());
            memcpy(out.texels.data() + at, im.data.data(), 3 * im.data.size() * sizeof(float));
        }
        out.textures.push_back(td);
    }
    out.other_light_count = (uint32_t)(ctx.lights.total_light_count - (int)ctx.lights.diffuse_rectangular_lights.size() -
                                       (int)out.delta_lights.size() - (int)out.mesh_lights.size() -
                                       (int)out.sphere_lights.size() - (out.has_environment ? 1 : 0));

    // Camera fields exactly as Camera::Camera computes them (src/ref/camera.cpp:5-14).
    const Matrix3x4& pose = scene.view_points[0];
    matrix_to_floats(pose, out.camera.camera_to_world);
    Vector2 extent = Vector2(scene.film_resolution);
    out.camera.image_extent[0] = extent.x;
    out.camera.image_extent[1] = extent.y;
    float tan_fovy_over_2 = std::tan(radians(scene.camera_fov_y / 2.f));
    out.camera.vert_half_dist = tan_fovy_over_2;
    out.camera.horz_half_dist = (extent.x / extent.y) * tan_fovy_over_2;
    out.camera.z_is_up = scene.z_is_up ? 1 : 0;

    const Raytracer_Config& rc = ctx.raytracer_config;
    yar_render_config& c = out.config;
    c.render_region[0] = ctx.render_region.p0.x;
    c.render_region[1] = ctx.render_region.p0.y;
    c.render_region[2] = ctx.render_region.p1.x;
    c.render_region[3] = ctx.render_region.p1.y;
    c.rendering_algorithm = (int32_t)rc.rendering_algorithm;
    c.max_light_bounces = rc.max_light_bounces;
    c.russian_roulette_threshold = rc.russian_roulette_threshold;
    c.russian_roulette_bounce_count_threshold = rc.russian_roulette_bounce_count_threshold;
    c.pixel_filter_type = (int32_t)rc.pixel_filter_type;
    c.pixel_filter_radius = rc.pixel_filter_radius;
    c.pixel_filter_alpha = rc.pixel_filter_alpha;
    c.x_pixel_sample_count = rc.x_pixel_sample_count;
    c.y_pixel_sample_count = rc.y_pixel_sample_count;
    c.film_radiance_scale = rc.film_radiance_scale;
    c.max_rgb_component_value_of_film_sample = rc.max_rgb_component_value_of_film_sample;
    c.pbrt3_scene = ctx.pbrt3_scene ? 1 : 0;
    c.rng_seed_offset = ctx.rng_seed_offset;
    return out;
}

} // namespace
