// yfs.hpp - "flat scene" file: a serialised yar_flat_scene (include/yar_gpu.h).
//
// The file carries exactly what the device path consumes: meshes with their
// kd-trees (node words bit for bit as KdTree::save writes them,
// src/ref/kdtree.cpp:137-160), scene objects, the scene kd-tree, constant
// materials, rectangular lights, point/spot/directional, triangle-mesh,
// sphere and environment lights, image textures and pbrt3 fourier BSDF
// tables (optional chunks), camera
// and Raytracer_Config.  It is produced
// by the host scene loader of this library and by the reference-side adapter
// that flattens a reference Scene_Context, so both sides can be compared on
// identical bytes.
//
// Layout: "YFS1" u32 version, then chunks {char tag[4]; u32 zero; u64 size;
// payload}.  All scalar fields are 4-byte little-endian values.
#pragma once

#include "yar_gpu.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace yfs {

constexpr uint32_t kMaterialRecordV1 = 72;  // yar_material_desc up to roughness_is_alpha

struct Mesh {
    std::vector<float> vertices;   // 3 per vertex
    std::vector<float> normals;    // empty or 3 per vertex
    std::vector<float> uvs;        // empty or 2 per vertex
    std::vector<int32_t> indices;  // 3 per triangle
    int32_t reverse_orientation = 0;
    int32_t visibility = YAR_VISIBLE;
    float bounds[6] = {0, 0, 0, 0, 0, 0};
    std::vector<yar_kd_node> nodes;
    uint32_t alpha_texture = 0;  // 0 none, else 1 + texture index
};

struct Scene {
    std::vector<Mesh> meshes;
    std::vector<yar_object_desc> objects;
    float scene_bounds[6] = {0, 0, 0, 0, 0, 0};
    std::vector<yar_kd_node> scene_nodes;
    std::vector<yar_material_desc> materials;
    std::vector<yar_rect_light_desc> rect_lights;
    std::vector<yar_delta_light_desc> delta_lights;
    std::vector<yar_mesh_light_desc> mesh_lights;
    std::vector<yar_sphere_light_desc> sphere_lights;
    bool has_environment = false;
    yar_environment_desc environment{};   // radiance points into environment_radiance
    std::vector<float> environment_radiance;
    std::vector<yar_texture_desc> textures;
    std::vector<yar_texture_mip_desc> texture_mips;
    std::vector<float> texels;           // RGB triples
    std::vector<yar_fourier_desc> fourier_tables;
    std::vector<float> fourier_floats;
    std::vector<uint32_t> fourier_uints;
    uint32_t other_light_count = 0;
    yar_camera_desc camera{};
    yar_render_config config{};

    // Views for the C ABI; valid while this object is alive and unmodified.
    std::vector<yar_mesh_desc> mesh_views;
    yar_flat_scene view() {
        mesh_views.resize(meshes.size());
        for (size_t i = 0; i < meshes.size(); i++) {
            const Mesh& m = meshes[i];
            yar_mesh_desc& d = mesh_views[i];
            d.vertices = m.vertices.data();
            d.normals = m.normals.empty() ? nullptr : m.normals.data();
            d.uvs = m.uvs.empty() ? nullptr : m.uvs.data();
            d.indices = m.indices.data();
            d.vertex_count = (uint32_t)(m.vertices.size() / 3);
            d.triangle_count = (uint32_t)(m.indices.size() / 3);
            d.reverse_geometric_normal_orientation = m.reverse_orientation;
            d.visibility = m.visibility;
            memcpy(d.kdtree.bounds_min, m.bounds, 3 * sizeof(float));
            memcpy(d.kdtree.bounds_max, m.bounds + 3, 3 * sizeof(float));
            d.kdtree.nodes = m.nodes.data();
            d.kdtree.node_count = (uint32_t)m.nodes.size();
            d.alpha_texture = m.alpha_texture;
        }
        yar_flat_scene s{};
        s.mesh_count = (uint32_t)meshes.size();
        s.meshes = mesh_views.data();
        s.object_count = (uint32_t)objects.size();
        s.objects = objects.data();
        memcpy(s.scene_kdtree.bounds_min, scene_bounds, 3 * sizeof(float));
        memcpy(s.scene_kdtree.bounds_max, scene_bounds + 3, 3 * sizeof(float));
        s.scene_kdtree.nodes = scene_nodes.data();
        s.scene_kdtree.node_count = (uint32_t)scene_nodes.size();
        s.material_count = (uint32_t)materials.size();
        s.materials = materials.data();
        s.rect_light_count = (uint32_t)rect_lights.size();
        s.rect_lights = rect_lights.data();
        s.other_light_count = other_light_count;
        s.camera = camera;
        s.config = config;
        s.delta_light_count = (uint32_t)delta_lights.size();
        s.delta_lights = delta_lights.empty() ? nullptr : delta_lights.data();
        s.mesh_light_count = (uint32_t)mesh_lights.size();
        s.mesh_lights = mesh_lights.empty() ? nullptr : mesh_lights.data();
        s.sphere_light_count = (uint32_t)sphere_lights.size();
        s.sphere_lights = sphere_lights.empty() ? nullptr : sphere_lights.data();
        environment.radiance = environment_radiance.data();
        s.environment = has_environment ? &environment : nullptr;
        s.texture_count = (uint32_t)textures.size();
        s.textures = textures.empty() ? nullptr : textures.data();
        s.texture_mip_count = (uint32_t)texture_mips.size();
        s.texture_mips = texture_mips.empty() ? nullptr : texture_mips.data();
        s.texels = texels.empty() ? nullptr : texels.data();
        s.texel_count = texels.size() / 3;
        s.fourier_count = (uint32_t)fourier_tables.size();
        s.fourier_tables = fourier_tables.empty() ? nullptr : fourier_tables.data();
        s.fourier_float_count = fourier_floats.size();
        s.fourier_floats = fourier_floats.empty() ? nullptr : fourier_floats.data();
        s.fourier_uint_count = fourier_uints.size();
        s.fourier_uints = fourier_uints.empty() ? nullptr : fourier_uints.data();
        return s;
    }
};

namespace detail {
struct Writer {
    FILE* f;
    bool ok = true;
    void raw(const void* p, size_t n) { if (n && fwrite(p, 1, n, f) != n) ok = false; }
    template <class T> void pod(const T& v) { raw(&v, sizeof(T)); }
    void chunk(const char tag[4], const std::vector<uint8_t>& payload) {
        raw(tag, 4);
        uint32_t zero = 0;
        pod(zero);
        uint64_t size = payload.size();
        pod(size);
        raw(payload.data(), payload.size());
    }
};
struct Buf {
    std::vector<uint8_t> b;
    void raw(const void* p, size_t n) {
        const uint8_t* s = (const uint8_t*)p;
        b.insert(b.end(), s, s + n);
    }
    template <class T> void pod(const T& v) { raw(&v, sizeof(T)); }
};
struct Reader {
    const uint8_t* p;
    const uint8_t* end;
    bool ok = true;
    void raw(void* dst, size_t n) {
        if ((size_t)(end - p) < n) { ok = false; return; }
        memcpy(dst, p, n);
        p += n;
    }
    template <class T> T pod() { T v{}; raw(&v, sizeof(T)); return v; }
};
} // namespace detail

inline bool write(const std::string& path, const Scene& s) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    detail::Writer w{f};
    w.raw("YFS1", 4);
    uint32_t version = 1;
    w.pod(version);
    {
        detail::Buf b;
        b.pod(s.config);
        b.pod(s.camera);
        b.pod(s.other_light_count);
        w.chunk("CONF", b.b);
    }
    for (const Mesh& m : s.meshes) {
        detail::Buf b;
        uint32_t vc = (uint32_t)(m.vertices.size() / 3), tc = (uint32_t)(m.indices.size() / 3);
        uint32_t flags = (m.normals.empty() ? 0u : 1u) | (m.uvs.empty() ? 0u : 2u) | (m.alpha_texture ? 4u : 0u);
        uint32_t nc = (uint32_t)m.nodes.size();
        b.pod(vc); b.pod(tc); b.pod(flags); b.pod(m.reverse_orientation); b.pod(m.visibility); b.pod(nc);
        b.raw(m.bounds, sizeof(m.bounds));
        b.raw(m.vertices.data(), m.vertices.size() * 4);
        b.raw(m.indices.data(), m.indices.size() * 4);
        if (flags & 1) b.raw(m.normals.data(), m.normals.size() * 4);
        if (flags & 2) b.raw(m.uvs.data(), m.uvs.size() * 4);
        b.raw(m.nodes.data(), m.nodes.size() * sizeof(yar_kd_node));
        if (flags & 4) b.pod(m.alpha_texture);
        w.chunk("MESH", b.b);
    }
    {
        detail::Buf b;
        uint32_t n = (uint32_t)s.objects.size();
        b.pod(n);
        b.raw(s.objects.data(), n * sizeof(yar_object_desc));
        w.chunk("OBJS", b.b);
    }
    {
        detail::Buf b;
        uint32_t n = (uint32_t)s.scene_nodes.size();
        b.raw(s.scene_bounds, sizeof(s.scene_bounds));
        b.pod(n);
        b.raw(s.scene_nodes.data(), n * sizeof(yar_kd_node));
        w.chunk("SKDT", b.b);
    }
    {   // MAT2: record size first, so the records can grow
        detail::Buf b;
        uint32_t n = (uint32_t)s.materials.size(), record = (uint32_t)sizeof(yar_material_desc);
        b.pod(n);
        b.pod(record);
        b.raw(s.materials.data(), n * sizeof(yar_material_desc));
        w.chunk("MAT2", b.b);
    }
    {
        detail::Buf b;
        uint32_t n = (uint32_t)s.rect_lights.size();
        b.pod(n);
        b.raw(s.rect_lights.data(), n * sizeof(yar_rect_light_desc));
        w.chunk("RLIT", b.b);
    }
    if (!s.delta_lights.empty()) {
        detail::Buf b;
        uint32_t n = (uint32_t)s.delta_lights.size();
        b.pod(n);
        b.raw(s.delta_lights.data(), n * sizeof(yar_delta_light_desc));
        w.chunk("DLIT", b.b);
    }
    if (!s.mesh_lights.empty()) {
        detail::Buf b;
        uint32_t n = (uint32_t)s.mesh_lights.size();
        b.pod(n);
        b.raw(s.mesh_lights.data(), n * sizeof(yar_mesh_light_desc));
        w.chunk("MLIT", b.b);
    }
    if (!s.sphere_lights.empty()) {
        detail::Buf b;
        uint32_t n = (uint32_t)s.sphere_lights.size();
        b.pod(n);
        b.raw(s.sphere_lights.data(), n * sizeof(yar_sphere_light_desc));
        w.chunk("SPHL", b.b);
    }
    if (s.has_environment) {
        detail::Buf b;
        yar_environment_desc e = s.environment;
        e.radiance = nullptr;
        b.pod(e);
        b.raw(s.environment_radiance.data(), s.environment_radiance.size() * sizeof(float));
        w.chunk("ENVM", b.b);
    }
    if (!s.textures.empty()) {  // TEXS: counts, texture records, mip records, texels
        detail::Buf b;
        const uint32_t nt = (uint32_t)s.textures.size(), nm = (uint32_t)s.texture_mips.size();
        const uint64_t nx = s.texels.size() / 3;
        b.pod(nt);
        b.pod(nm);
        b.pod(nx);
        b.raw(s.textures.data(), nt * sizeof(yar_texture_desc));
        b.raw(s.texture_mips.data(), nm * sizeof(yar_texture_mip_desc));
        b.raw(s.texels.data(), s.texels.size() * sizeof(float));
        w.chunk("TEXS", b.b);
    }
    if (!s.fourier_tables.empty()) {  // FOUR: counts, table records, floats, uints
        detail::Buf b;
        const uint32_t nt = (uint32_t)s.fourier_tables.size();
        const uint64_t nf = s.fourier_floats.size(), nu = s.fourier_uints.size();
        b.pod(nt);
        b.pod(nf);
        b.pod(nu);
        b.raw(s.fourier_tables.data(), nt * sizeof(yar_fourier_desc));
        b.raw(s.fourier_floats.data(), nf * sizeof(float));
        b.raw(s.fourier_uints.data(), nu * sizeof(uint32_t));
        w.chunk("FOUR", b.b);
    }
    bool ok = w.ok;
    if (fclose(f) != 0) ok = false;
    return ok;
}

inline bool read(const std::string& path, Scene& s, std::string* err = nullptr) {
    auto fail = [&](const char* m) { if (err) *err = m; return false; };
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return fail("cannot open file");
    std::vector<uint8_t> data;
    {
        if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return fail("seek failed"); }
        long size = ftell(f);
        if (size < 0) { fclose(f); return fail("tell failed"); }
        fseek(f, 0, SEEK_SET);
        data.resize((size_t)size);
        size_t got = data.empty() ? 0 : fread(data.data(), 1, data.size(), f);
        fclose(f);
        if (got != data.size()) return fail("short read");
    }
    detail::Reader r{data.data(), data.data() + data.size()};
    char magic[4];
    r.raw(magic, 4);
    uint32_t version = r.pod<uint32_t>();
    if (!r.ok || memcmp(magic, "YFS1", 4) != 0 || version != 1) return fail("not a YFS1 file");
    s = Scene{};
    while (r.ok && r.p < r.end) {
        char tag[4];
        r.raw(tag, 4);
        r.pod<uint32_t>();
        uint64_t size = r.pod<uint64_t>();
        if (!r.ok || (uint64_t)(r.end - r.p) < size) return fail("truncated chunk");
        detail::Reader c{r.p, r.p + size};
        r.p += size;
        if (!memcmp(tag, "CONF", 4)) {
            s.config = c.pod<yar_render_config>();
            s.camera = c.pod<yar_camera_desc>();
            s.other_light_count = c.pod<uint32_t>();
        } else if (!memcmp(tag, "MESH", 4)) {
            Mesh m;
            uint32_t vc = c.pod<uint32_t>(), tc = c.pod<uint32_t>(), flags = c.pod<uint32_t>();
            m.reverse_orientation = c.pod<int32_t>();
            m.visibility = c.pod<int32_t>();
            uint32_t nc = c.pod<uint32_t>();
            c.raw(m.bounds, sizeof(m.bounds));
            if (!c.ok || (uint64_t)vc * 12 + (uint64_t)tc * 12 + (uint64_t)nc * 8 > size) return fail("bad mesh chunk");
            m.vertices.resize((size_t)vc * 3);
            c.raw(m.vertices.data(), m.vertices.size() * 4);
            m.indices.resize((size_t)tc * 3);
            c.raw(m.indices.data(), m.indices.size() * 4);
            if (flags & 1) { m.normals.resize((size_t)vc * 3); c.raw(m.normals.data(), m.normals.size() * 4); }
            if (flags & 2) { m.uvs.resize((size_t)vc * 2); c.raw(m.uvs.data(), m.uvs.size() * 4); }
            m.nodes.resize(nc);
            c.raw(m.nodes.data(), nc * sizeof(yar_kd_node));
            if (flags & 4) m.alpha_texture = c.pod<uint32_t>();
            if (!c.ok) return fail("truncated mesh chunk");
            s.meshes.push_back(std::move(m));
        } else if (!memcmp(tag, "OBJS", 4)) {
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * sizeof(yar_object_desc) > size) return fail("bad object chunk");
            s.objects.resize(n);
            c.raw(s.objects.data(), n * sizeof(yar_object_desc));
        } else if (!memcmp(tag, "SKDT", 4)) {
            c.raw(s.scene_bounds, sizeof(s.scene_bounds));
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * 8 > size) return fail("bad scene tree chunk");
            s.scene_nodes.resize(n);
            c.raw(s.scene_nodes.data(), n * sizeof(yar_kd_node));
        } else if (!memcmp(tag, "MATS", 4) || !memcmp(tag, "MAT2", 4)) {
            // MATS: the first records, without the layered-material fields (72 bytes)
            uint32_t n = c.pod<uint32_t>();
            const uint32_t record = !memcmp(tag, "MATS", 4) ? kMaterialRecordV1 : c.pod<uint32_t>();
            if (record < kMaterialRecordV1 || (uint64_t)n * record > size) return fail("bad material chunk");
            s.materials.assign(n, yar_material_desc{});
            for (uint32_t i = 0; i < n && c.ok; i++) {
                const size_t keep = record < sizeof(yar_material_desc) ? record : sizeof(yar_material_desc);
                c.raw(&s.materials[i], keep);
                if (record > keep) c.p += record - keep;
            }
        } else if (!memcmp(tag, "RLIT", 4)) {
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * sizeof(yar_rect_light_desc) > size) return fail("bad light chunk");
            s.rect_lights.resize(n);
            c.raw(s.rect_lights.data(), n * sizeof(yar_rect_light_desc));
        } else if (!memcmp(tag, "DLIT", 4)) {
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * sizeof(yar_delta_light_desc) > size) return fail("bad delta light chunk");
            s.delta_lights.resize(n);
            c.raw(s.delta_lights.data(), n * sizeof(yar_delta_light_desc));
        } else if (!memcmp(tag, "MLIT", 4)) {
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * sizeof(yar_mesh_light_desc) > size) return fail("bad mesh light chunk");
            s.mesh_lights.resize(n);
            c.raw(s.mesh_lights.data(), n * sizeof(yar_mesh_light_desc));
        } else if (!memcmp(tag, "SPHL", 4)) {
            uint32_t n = c.pod<uint32_t>();
            if ((uint64_t)n * sizeof(yar_sphere_light_desc) > size) return fail("bad sphere light chunk");
            s.sphere_lights.resize(n);
            c.raw(s.sphere_lights.data(), n * sizeof(yar_sphere_light_desc));
        } else if (!memcmp(tag, "TEXS", 4)) {
            const uint32_t nt = c.pod<uint32_t>(), nm = c.pod<uint32_t>();
            const uint64_t nx = c.pod<uint64_t>();
            // each count is checked against the chunk size before it is multiplied
            if (!c.ok || nt > size / sizeof(yar_texture_desc) || nm > size / sizeof(yar_texture_mip_desc) ||
                nx > size / 12 ||
                (uint64_t)nt * sizeof(yar_texture_desc) + (uint64_t)nm * sizeof(yar_texture_mip_desc) + nx * 12 > size)
                return fail("bad texture chunk");
            s.textures.resize(nt);
            c.raw(s.textures.data(), nt * sizeof(yar_texture_desc));
            s.texture_mips.resize(nm);
            c.raw(s.texture_mips.data(), nm * sizeof(yar_texture_mip_desc));
            s.texels.resize(nx * 3);
            c.raw(s.texels.data(), s.texels.size() * sizeof(float));
        } else if (!memcmp(tag, "FOUR", 4)) {
            const uint32_t nt = c.pod<uint32_t>();
            const uint64_t nf = c.pod<uint64_t>(), nu = c.pod<uint64_t>();
            if (!c.ok || nt > size / sizeof(yar_fourier_desc) || nf > size / 4 || nu > size / 4 ||
                (uint64_t)nt * sizeof(yar_fourier_desc) + (nf + nu) * 4 > size)
                return fail("bad fourier chunk");
            s.fourier_tables.resize(nt);
            c.raw(s.fourier_tables.data(), nt * sizeof(yar_fourier_desc));
            s.fourier_floats.resize(nf);
            c.raw(s.fourier_floats.data(), nf * sizeof(float));
            s.fourier_uints.resize(nu);
            c.raw(s.fourier_uints.data(), nu * sizeof(uint32_t));
        } else if (!memcmp(tag, "ENVM", 4)) {
            s.environment = c.pod<yar_environment_desc>();
            const uint64_t count = 3ull * s.environment.width * s.environment.height;
            if (!c.ok || count * sizeof(float) > size) return fail("bad environment chunk");
            s.environment_radiance.resize(count);
            c.raw(s.environment_radiance.data(), count * sizeof(float));
            s.environment.radiance = nullptr;
            s.has_environment = true;
        }
        if (!c.ok) return fail("truncated chunk payload");
    }
    if (!r.ok) return fail("truncated file");
    return true;
}

} // namespace yfs
