// shade.cuh - device restatement of the shading side of the reference path:
// shading context (src/ref/shading_context.cpp), Diffuse/Metal/Rough_Glass
// BSDFs (src/ref/bsdf.cpp), microfacet and Fresnel math (src/ref/scattering.cpp),
// sampling (src/ref/sampling.cpp), ray-origin offsetting (src/lib/math.cpp).
//
// Every expression keeps the reference's operand order; the translation unit
// is compiled with -fmad=false and IEEE division/sqrt, so all of it rounds
// like the reference except sin/cos: those are evaluated in double precision
// and rounded once to float, which gives the correctly rounded float result
// (what glibc's sinf/cosf return for all but a vanishing fraction of inputs).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace yar {

struct V3 {
    float x, y, z;
};
struct Col {
    float r, g, b;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 mul(V3 v, float t) { return v3(v.x * t, v.y * t, v.z * t); }   // Vector3 * float
__device__ __forceinline__ V3 divs(V3 v, float t) { return v3(v.x / t, v.y / t, v.z / t); }  // Vector3 / float
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len2(V3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
__device__ __forceinline__ float len(V3 v) { return sqrtf(len2(v)); }
__device__ __forceinline__ V3 normalized(V3 v) { return divs(v, len(v)); }

__device__ __forceinline__ Col col(float r, float g, float b) { return Col{r, g, b}; }
__device__ __forceinline__ Col operator+(Col a, Col b) { return col(a.r + b.r, a.g + b.g, a.b + b.b); }
__device__ __forceinline__ Col operator-(Col a, Col b) { return col(a.r - b.r, a.g - b.g, a.b - b.b); }
__device__ __forceinline__ Col operator*(Col a, Col b) { return col(a.r * b.r, a.g * b.g, a.b * b.b); }
__device__ __forceinline__ Col operator/(Col a, Col b) { return col(a.r / b.r, a.g / b.g, a.b / b.b); }
__device__ __forceinline__ Col mul(Col c, float k) { return col(c.r * k, c.g * k, c.b * k); }  // ColorRGB * float
__device__ __forceinline__ Col csqrt(Col c) { return col(sqrtf(c.r), sqrtf(c.g), sqrtf(c.b)); }
__device__ __forceinline__ bool black(Col c) { return c.r == 0.f && c.g == 0.f && c.b == 0.f; }
__device__ __forceinline__ float max_std(float a, float b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ float min_std(float a, float b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ float max_component(Col c) { return max_std(c.r, max_std(c.g, c.b)); }
__device__ __forceinline__ float clamp1(float x) { return x < -1.f ? -1.f : (x > 1.f ? 1.f : x); }

__device__ __forceinline__ float sin_f(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float cos_f(float x) { return (float)cos((double)x); }

constexpr float kPi = 3.14159265f;  // src/lib/math.h:7

// transform_point / transform_vector (src/lib/matrix.cpp:368-382)
__device__ __forceinline__ V3 xform_point(const float4& r0, const float4& r1, const float4& r2, V3 p) {
    return v3(r0.x * p.x + r0.y * p.y + r0.z * p.z + r0.w, r1.x * p.x + r1.y * p.y + r1.z * p.z + r1.w,
              r2.x * p.x + r2.y * p.y + r2.z * p.z + r2.w);
}
__device__ __forceinline__ V3 xform_vector(const float4& r0, const float4& r1, const float4& r2, V3 v) {
    return v3(r0.x * v.x + r0.y * v.y + r0.z * v.z, r1.x * v.x + r1.y * v.y + r1.z * v.z,
              r2.x * v.x + r2.y * v.y + r2.z * v.z);
}

// barycentric_interpolate (src/lib/math.h:146-153)
__device__ __forceinline__ V3 bary(V3 p0, V3 p1, V3 p2, float b0, float b1, float b2) {
    return (mul(p0, b0) + mul(p1, b1)) + mul(p2, b2);
}

// coordinate_system_from_vector (src/lib/math.cpp:21-25), first axis only
__device__ __forceinline__ V3 coordinate_axis(V3 v) {
    V3 v1 = (fabsf(v.x) > fabsf(v.y)) ? v3(-v.z, 0.f, v.x) : v3(0.f, -v.z, v.y);
    return divs(v1, len(v1));
}

__device__ __forceinline__ V3 reflect(V3 w, V3 n) { return mul(n, 2.f * dot(w, n)) - w; }

__device__ __forceinline__ bool refract(V3 wi, V3 n, float eta, V3& wt) {
    const float cos_i = dot(wi, n);
    const float sin_t2 = eta * eta * max_std(0.f, 1.f - cos_i * cos_i);
    if (sin_t2 >= 1.f) return false;
    const float cos_t = sqrtf(1.f - sin_t2);
    wt = mul(wi, -eta) + mul(n, eta * cos_i - cos_t);
    return true;
}

// offset_ray_origin_in_both_directions (src/lib/math.cpp:81-120)
__device__ __forceinline__ void offset_axis(float p, float n, float& pos, float& neg) {
    const int di = (int)(256.f * n);
    const int i1 = __float_as_int(p) - di, i2 = __float_as_int(p) + di;
    pos = __int_as_float(p < 0 ? i1 : i2);
    neg = __int_as_float(p < 0 ? i2 : i1);
    if (fabsf(p) < 1.0f / 32.0f) {
        const float d = (1.0f / 65536.0f) * n;
        pos = p + d;
        neg = p - d;
    }
}

struct Shading {
    V3 wo, position, ng, n, dpdu_shading;
    V3 origin_pos, origin_neg;
    bool flipped;
};

__device__ __forceinline__ V3 origin_for_direction(const Shading& sc, V3 dir) {
    return dot(dir, sc.ng) > 0.f ? sc.origin_pos : sc.origin_neg;
}
__device__ __forceinline__ V3 origin_for_point(const Shading& sc, V3 point) {
    return origin_for_direction(sc, point - sc.position);
}

// adjust_shading_normal (src/ref/shading_context.cpp:17-63)
__device__ __forceinline__ V3 adjust_shading_normal(V3 wo, V3 ng, V3 n) {
    const V3 R = reflect(wo, n);
    const float a = dot(R, ng);
    if (a >= 0.f) return n;
    if (dot(wo, ng) < 0.0017453f) return ng;
    const float b = dot(n, ng);
    V3 tangent;
    if (b > 1e-4f) {
        tangent = R + mul(n, fabsf(a) / b);
        tangent = divs(tangent, len(tangent));
    } else {
        tangent = n;
    }
    tangent = tangent + mul(ng, 1e-4f);
    return normalized(wo + tangent);
}

// ---------------------------------------------------------------- BSDFs
// The reference's Material_Type values, and kPbrt3Plastic: plastic in a pbrt-v3
// scene, which the reference shades with Pbrt3_Plastic_BRDF (src/ref/bsdf.cpp:656-667).
enum : uint32_t {
    kPerfectReflector = 0,
    kPerfectRefractor = 1,
    kDiffuse = 2,
    kMetal = 4,
    kDiffuseTransmission = 3,
    kPlastic = 5,
    kCoatedDiffuse = 6,
    kGlass = 7,
    kMix = 8,
    kUber = 9,
    kTranslucent = 10,
    kFourier = 11,
    kPbrt3Plastic = 0x105,
    kScaled = 0x108  // a mix with a pure delta material: the other one's BSDF, scaled
};

// How a material scatters without a BSDF: not at all (kDeltaNone), as a
// mirror, a perfect refractor, or smooth glass (glass of roughness 0).
enum : uint32_t { kDeltaNone = 0, kDeltaReflector = 1, kDeltaRefractor = 2, kDeltaGlass = 3, kDeltaUber = 4, kDeltaMix = 5 };

// Material constants as the BSDF constructors evaluate them (src/ref/bsdf.cpp:60-66,
// :146-158, :205-213, :268-294, :427-438); alpha values are computed on the host
// with the reference's roughness remapping.  Plastic and coated diffuse keep
// their diffuse reflectance in `reflectance` and their r0 in `transmittance`;
// diffuse transmission keeps its scale in `extra` (for textured slots).
struct Material_Dev {
    uint32_t type;
    float alpha_x, alpha_y, alpha;
    Col reflectance, transmittance;
    Col eta_t, k_t;
    float eta_i_metal, ior;
    uint32_t delta;  // kDelta*
    uint32_t uber_components;  // pbrt3 uber: component kinds, 3 bits each, count in bits 24..27
    Col specular;     // pbrt3 uber, pbrt3 translucent: Ks
    Col extra;        // pbrt3 uber: opacity; pbrt3 translucent: Kd
    Col delta_reflectance;  // pbrt3 uber: Kr
    uint32_t scattering;    // bit 0 reflection, bit 1 transmission (BSDF::reflection/transmission_scattering)
    int32_t mix_sub[2];     // mix: the two materials
    float mix_amount;       // mix: min(luminance(amount), 1), the layer choice
    float mix_p;            // mix: 1 - luminance(White - amount) (Mix_BSDF::p_coeff)
    float mix_lum;          // mix: luminance(amount), unclamped (the Scaled_BSDF factor)
    Col mix_coeff;          // mix: White - amount
    uint32_t has_bsdf;      // initialize_scattering creates a BSDF: some layer is not delta
    uint32_t texture;       // 1 + the reflectance's texture (0: the constant); diffuse, plastic,
                            // coated diffuse, glass, diffuse transmission
    float2 texture_scale;   // its uv scale
    uint32_t texture2;      // 1 + the transmittance's texture; glass, diffuse transmission
    float2 texture2_scale;
    uint32_t bump;          // bump map: 0 none, 1 constant height, 2 texture (its luminance)
    float bump_height;      // bump 1: the height
    uint32_t bump_texture;  // bump 2: 1 + the texture
    float2 bump_scale;      // bump 2: its uv scale
    // pbrt3 fourier: the table (device pointers), its node count and channels
    const float* fourier_nodes;
    const float* fourier_coeffs;
    const uint32_t* fourier_series;  // (offset, length) per node pair
    uint32_t fourier_node_count, fourier_channels;
};

struct Bsdf {
    uint32_t type;
    V3 n, t, bt;
    bool reflection, transmission;
    bool flipped;  // the shading normal was flipped towards wo (Pbrt3_Plastic_BRDF's IOR choice)
    Col reflectance, transmittance, eta_t, k_t;
    Col specular, extra;  // pbrt3 uber: Ks, opacity; pbrt3 translucent: Ks, Kd
    const Material_Dev* sub[2];  // mix: the two materials; scaled: sub[0]
    Col mix_coeff;
    float mix_p;
    float alpha_x, alpha_y, alpha, eta_i_metal, eta_o, eta_i;
};

__device__ __forceinline__ V3 local_to_world(const Bsdf& f, V3 l) {
    return v3(f.t.x * l.x + f.bt.x * l.y + f.n.x * l.z, f.t.y * l.x + f.bt.y * l.y + f.n.y * l.z,
              f.t.z * l.x + f.bt.z * l.y + f.n.z * l.z);
}
__device__ __forceinline__ V3 world_to_local(const Bsdf& f, V3 w) { return v3(dot(w, f.t), dot(w, f.bt), dot(w, f.n)); }

// The material part of a BSDF (its frame and flip stay): the constructors of
// src/ref/bsdf.cpp and bsdf_pbrt.cpp with constant parameters.
__device__ __forceinline__ void set_material(Bsdf& f, const Material_Dev& m) {
    f.type = m.type;
    f.reflection = (m.scattering & 1u) != 0;
    f.transmission = (m.scattering & 2u) != 0;
    f.specular = m.specular;
    f.extra = m.extra;
    f.reflectance = m.reflectance;
    f.transmittance = m.transmittance;
    f.eta_t = m.eta_t;
    f.k_t = m.k_t;
    f.alpha_x = m.alpha_x;
    f.alpha_y = m.alpha_y;
    f.alpha = m.alpha;
    f.eta_i_metal = m.eta_i_metal;
    const bool enter = !f.flipped;
    f.eta_o = enter ? 1.f : m.ior;
    f.eta_i = enter ? m.ior : 1.f;
    if (m.type == kTranslucent) {  // Pbrt3_Translucent_BSDF: the fixed 1.0 / 1.5 pair
        f.eta_o = enter ? 1.f : 1.5f;
        f.eta_i = enter ? 1.5f : 1.f;
    } else if (m.type == kUber) {  // Pbrt3_Uber_BRDF's relative IOR (bsdf_pbrt.cpp:14-32)
        f.eta_i = enter ? m.ior : 1.f / m.ior;
    } else if (m.type == kFourier) {  // the table, read through the material
        f.sub[0] = &m;
    }
}

// create_bsdf (src/ref/bsdf.cpp:631-714): the frame from the shading normal and
// dpdu, then the material.  A mix (create_mix_bsdf, :599-629) keeps its two
// materials and builds their BSDFs when it is evaluated or sampled.
__device__ __forceinline__ void make_bsdf(const Shading& sc, const Material_Dev& m, const Material_Dev* materials,
                                          Bsdf& f) {
    f.n = sc.n;
    f.bt = normalized(cross(sc.n, sc.dpdu_shading));
    f.t = cross(f.bt, sc.n);
    f.flipped = sc.flipped;
    set_material(f, m);
    if (m.type == kMix) {
        const Material_Dev& m1 = materials[m.mix_sub[0]];
        const Material_Dev& m2 = materials[m.mix_sub[1]];
        const bool has1 = m1.type != kPerfectReflector && m1.type != kPerfectRefractor;
        const bool has2 = m2.type != kPerfectReflector && m2.type != kPerfectRefractor;
        f.type = has1 && has2 ? kMix : kScaled;
        f.sub[0] = has1 ? &m1 : &m2;
        f.sub[1] = &m2;
        f.mix_coeff = m.mix_coeff;
        f.mix_p = has1 && has2 ? m.mix_p : (has1 ? m.mix_lum : 1.f - m.mix_lum);
        f.reflection = (m.scattering & 1u) != 0;
        f.transmission = (m.scattering & 2u) != 0;
    }
}

__device__ __forceinline__ V3 sample_hemisphere_cosine(float u0, float u1) {
    const float z = sqrtf(1.f - u0);
    const float r = sqrtf(u0);
    const float phi = 2.f * kPi * u1;
    return v3(r * cos_f(phi), r * sin_f(phi), z);
}

__device__ __forceinline__ float dielectric_fresnel(float cos_i, float eta) {
    cos_i = min_std(fabsf(cos_i), 1.f);
    const float sin_i = sqrtf(1.f - cos_i * cos_i);
    const float sin_t = (1.f / eta) * sin_i;
    if (sin_t >= 1.f) return 1.f;
    const float cos_t = sqrtf(1.f - sin_t * sin_t);
    const float Rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float Rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (Rp * Rp + Rs * Rs);
}

// check_for_delta_scattering_event with get_perfect_reflector_info,
// get_perfect_refractor_info and get_glass_info (src/ref/delta_scattering.cpp:27-97,
// :252-324) and get_pbrt_uber_info (:102-150), constant parameters, no
// nested dielectrics.  Returns 0 (no delta event), 1 (dir and atten set) or
// 2: a perfect refractor at total internal reflection, where the reference
// has no direction (an assertion) and the path ends.  bsdf_prob is 1 - the
// delta layers' selection probability; kind the event's
// Delta_Scattering_Type: 0 reflection, etaI_over_etaT (> 0) transmission, -1
// passthrough.
__device__ __forceinline__ int delta_scattering(const Shading& sc, const Material_Dev& m,
                                                const Material_Dev* materials, float& u, V3& dir, Col& atten,
                                                float& bsdf_prob, float& kind) {
    atten = col(1.f, 1.f, 1.f);
    kind = 0.f;
    const bool enter = !sc.flipped;
    if (m.delta == kDeltaMix) {
        // get_mix_info (delta_scattering.cpp:154-189) for sub-materials that are pure
        // delta or have no delta event
        const Material_Dev& m1 = materials[m.mix_sub[0]];
        const Material_Dev& m2 = materials[m.mix_sub[1]];
        const bool has1 = m1.type != kPerfectReflector && m1.type != kPerfectRefractor;
        const bool has2 = m2.type != kPerfectReflector && m2.type != kPerfectRefractor;
        const bool first = u < m.mix_amount;
        u = first ? u / m.mix_amount : (u - m.mix_amount) / (1.f - m.mix_amount);
        const Material_Dev& pick = first ? m1 : m2;
        int event = 0;
        float prob = 0.f;
        if (pick.type == kPerfectReflector) {
            dir = reflect(sc.wo, sc.n);
            atten = pick.reflectance;
            event = 1;
            prob = 1.f;
        } else if (pick.type == kPerfectRefractor) {
            kind = enter ? 1.f / pick.ior : pick.ior;
            event = refract(sc.wo, sc.n, kind, dir) ? 1 : 2;
            prob = 1.f;
        }
        if (has1 && has2) prob *= first ? m.mix_amount : 1.f - m.mix_amount;
        else prob = has1 ? 1.f - m.mix_amount : m.mix_amount;
        bsdf_prob = 1.f - prob;
        return event;
    }
    if (m.delta == kDeltaUber) {
        // get_pbrt_uber_info (delta_scattering.cpp:102-150): u picks a layer and is
        // re-normalised for the BSDF; delta reflection and opacity are delta events
        const uint32_t count = (m.uber_components >> 24) & 0xfu;
        const float fp = u * (float)count;
        const int k = (int)fp;
        const uint32_t comp = (m.uber_components >> (3 * k)) & 7u;
        const float r = fp - (float)k;
        u = r < 0.f ? 0.f : (__uint_as_float(0x3f7fffffu) < r ? __uint_as_float(0x3f7fffffu) : r);
        float delta_terms = 0.f;
        for (uint32_t c = 0; c < count; c++)
            if (((m.uber_components >> (3 * c)) & 7u) >= YAR_UBER_DELTA_REFLECTION) delta_terms += 1.f;
        bsdf_prob = 1.f - delta_terms / (float)count;
        if (comp == YAR_UBER_DELTA_REFLECTION) {
            const float fresnel = dielectric_fresnel(dot(sc.n, sc.wo), enter ? m.ior : 1.f / m.ior);
            atten = mul(m.delta_reflectance, (float)count * fresnel);
            dir = reflect(sc.wo, sc.n);
            return 1;
        }
        if (comp == YAR_UBER_OPACITY) {
            atten = mul(col(1.f, 1.f, 1.f) - m.extra, (float)count);
            dir = -sc.wo;
            kind = -1.f;
            return 1;
        }
        return 0;
    }
    bsdf_prob = 0.f;
    if (m.delta == kDeltaReflector) {
        dir = reflect(sc.wo, sc.n);
        atten = m.reflectance;
        return 1;
    }
    if (m.delta == kDeltaRefractor) {
        kind = enter ? 1.f / m.ior : m.ior;
        return refract(sc.wo, sc.n, kind, dir) ? 1 : 2;
    }
    const float eta_t_over_i = enter ? m.ior : 1.f / m.ior;
    const float fresnel = dielectric_fresnel(dot(sc.n, sc.wo), eta_t_over_i);
    if (u < fresnel) {
        dir = reflect(sc.wo, sc.n);
        atten = m.reflectance;
        return 1;
    }
    const float eta = 1.f / eta_t_over_i;
    atten = mul(m.transmittance, eta * eta);
    kind = eta;
    return refract(sc.wo, sc.n, eta, dir) ? 1 : 2;
}

__device__ __forceinline__ float one_minus_eps_min_s(float v) {  // std::min(v, One_Minus_Epsilon)
    const float ome = __uint_as_float(0x3f7fffffu);
    return v < ome ? v : ome;
}

// schlick_fresnel (src/ref/scattering.cpp:10-15)
__device__ __forceinline__ Col schlick_fresnel(Col r0, float cos_i) {
    const float k = 1.f - fabsf(cos_i);
    const float k5 = (k * k) * (k * k) * k;
    return r0 + mul(col(1.f, 1.f, 1.f) - r0, k5);
}

__device__ __forceinline__ Col conductor_fresnel(float cos_i, float eta_i, Col eta_t, Col k_t) {
    cos_i = fabsf(clamp1(cos_i));
    const float c2 = cos_i * cos_i;
    const float s2 = 1.f - c2;
    const Col eta = mul(eta_t, 1.f / eta_i);
    const Col k = mul(k_t, 1.f / eta_i);
    const Col eta2 = eta * eta;
    const Col k2 = k * k;
    const Col t0 = (eta2 - k2) - col(s2, s2, s2);
    const Col a2b2 = csqrt(t0 * t0 + mul(eta2, 4.f) * k2);
    const Col t1 = a2b2 + col(c2, c2, c2);
    const Col a = csqrt(mul(a2b2 + t0, 0.5f));
    const Col t2 = mul(a, 2.f * cos_i);
    const Col Rs = (t1 - t2) / (t1 + t2);
    const float s4 = s2 * s2;
    const Col t3 = mul(a2b2, c2) + col(s4, s4, s4);
    const Col t4 = mul(t2, s2);
    const Col Rp = (Rs * (t3 - t4)) / (t3 + t4);
    return mul(Rp + Rs, 0.5f);
}

__device__ __forceinline__ float ggx_D(V3 wh, V3 n, float alpha) {
    const float c = dot(wh, n);
    if (c <= 0.f) return 0.f;
    const float c2 = c * c;
    const float a2 = alpha * alpha;
    const float k = c2 * (a2 - 1) + 1;
    return a2 / (kPi * k * k);
}
__device__ __forceinline__ float ggx_D_aniso(V3 wh, float ax, float ay) {
    const float c = clamp1(wh.z);
    const float c2 = c * c;
    const float s2 = 1.f - c2;
    const float s2inv = 1.f / s2;
    const float cos2_phi = (s2 == 0.f) ? 1.f : (wh.x * wh.x) * s2inv;
    const float sin2_phi = (s2 == 0.f) ? 0.f : (wh.y * wh.y) * s2inv;
    const float k = c2 + s2 * (cos2_phi / (ax * ax) + sin2_phi / (ay * ay));
    return 1.f / (kPi * ax * ay * k * k);
}
__device__ __forceinline__ float ggx_lambda(V3 v, V3 n, float alpha) {
    const float c = dot(v, n);
    const float c2 = c * c;
    const float tan2 = max_std(0.f, (1.f - c2) / c2);
    return 0.5f * (-1.f + sqrtf(1.f + alpha * alpha * tan2));
}
__device__ __forceinline__ float ggx_lambda_aniso(V3 v, float ax, float ay) {
    const float c = clamp1(v.z);
    const float c2 = c * c;
    const float s2 = 1.f - c2;
    const float tan2 = s2 / c2;
    const float s2inv = 1.f / s2;
    const float cos2_phi = (s2 == 0.f) ? 1.f : (v.x * v.x) * s2inv;
    const float sin2_phi = (s2 == 0.f) ? 0.f : (v.y * v.y) * s2inv;
    const float alpha2 = cos2_phi * ax * ax + sin2_phi * ay * ay;
    return 0.5f * (-1.f + sqrtf(1.f + alpha2 * tan2));
}
__device__ __forceinline__ float ggx_G(V3 wi, V3 wo, V3 n, float a) {
    return 1.f / (1.f + ggx_lambda(wi, n, a) + ggx_lambda(wo, n, a));
}
__device__ __forceinline__ float ggx_G1(V3 v, V3 n, float a) { return 1.f / (1.f + ggx_lambda(v, n, a)); }
__device__ __forceinline__ float ggx_G_aniso(V3 wi, V3 wo, float ax, float ay) {
    return 1.f / (1.f + ggx_lambda_aniso(wi, ax, ay) + ggx_lambda_aniso(wo, ax, ay));
}
__device__ __forceinline__ float ggx_G1_aniso(V3 v, float ax, float ay) {
    return 1.f / (1.f + ggx_lambda_aniso(v, ax, ay));
}

// GGX_sample_visible_microfacet_normal (src/ref/sampling.cpp:310-335)
__device__ __forceinline__ V3 ggx_sample_vndf(float u0, float u1, V3 wo, float ax, float ay) {
    const V3 N = normalized(v3(ax * wo.x, ay * wo.y, wo.z));
    const float len_sq = N.x * N.x + N.y * N.y;
    const V3 T1 = len_sq > 0.f ? divs(v3(-N.y, N.x, 0.f), sqrtf(len_sq)) : v3(1.f, 0.f, 0.f);
    const V3 T2 = cross(N, T1);
    const float r = sqrtf(u0);
    const float phi = 2.f * kPi * u1;
    const float t1 = r * cos_f(phi);
    float t2 = r * sin_f(phi);
    const float s = 0.5f * (1.f + N.z);
    t2 = (1.f - s) * sqrtf(1.f - t1 * t1) + s * t2;
    const V3 nh = (mul(T1, t1) + mul(T2, t2)) + mul(N, sqrtf(max_std(0.f, 1.f - t1 * t1 - t2 * t2)));
    return normalized(v3(ax * nh.x, ay * nh.y, max_std(1e-6f, nh.z)));
}
__device__ __forceinline__ float vndf_pdf(V3 wo, V3 wh, V3 n, float alpha) {
    const float G1 = ggx_G1(wo, n, alpha);
    const float D = ggx_D(wh, n, alpha);
    return G1 * D * max_std(0.f, dot(wo, wh)) / dot(wo, n);
}
__device__ __forceinline__ float vndf_pdf_aniso(V3 wo, V3 wh, float ax, float ay) {
    const float G1 = ggx_G1_aniso(wo, ax, ay);
    const float D = ggx_D_aniso(wh, ax, ay);
    return G1 * D * max_std(0.f, dot(wo, wh)) / wo.z;
}
__device__ __forceinline__ V3 refraction_half(float eta_o, V3 wo, float eta_i, V3 wi, V3 n) {
    V3 wh = -normalized(mul(wo, eta_o) + mul(wi, eta_i));
    if (dot(wh, n) < 0.f) wh = -wh;
    return wh;
}
__device__ __forceinline__ float glass_reflection_probability(const Bsdf& f, float fresnel) {
    const float max_r = max_component(f.reflectance), max_t = max_component(f.transmittance);
    const float ratio = max_r / (max_r + max_t);
    const float r = fresnel * ratio;
    const float t = (1.f - fresnel) * (1 - ratio);
    return ((r + t) == 0) ? 0.f : r / (r + t);
}

__device__ __forceinline__ float pow5(float v) { return (v * v) * (v * v) * v; }

// The FULL forms (every material, mixes included) are called out of line:
// inlined at each of the shade kernels' call sites they multiplied the
// kernels' code and took the device compiler minutes per kernel.  The
// FULL = false forms (diffuse, metal, rough glass) stay inlined.
template <bool FULL> __device__ __forceinline__ Col leaf_evaluate_body(const Bsdf& f, V3 wo, V3 wi);
template <bool FULL> __device__ __forceinline__ float leaf_pdf_body(const Bsdf& f, V3 wo, V3 wi);
template <bool FULL>
__device__ __forceinline__ Col leaf_sample_body(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                                float& pdf);
static __device__ __noinline__ Col leaf_evaluate_full(const Bsdf& f, V3 wo, V3 wi) { return leaf_evaluate_body<true>(f, wo, wi); }
static __device__ __noinline__ float leaf_pdf_full(const Bsdf& f, V3 wo, V3 wi) { return leaf_pdf_body<true>(f, wo, wi); }
static __device__ __noinline__ Col leaf_sample_full(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                             float& pdf) {
    return leaf_sample_body<true>(f, u0, u1, u_scatter, wo, wi, pdf);
}
template <bool FULL = true>
__device__ __forceinline__ Col leaf_evaluate(const Bsdf& f, V3 wo, V3 wi) {
    if constexpr (FULL) return leaf_evaluate_full(f, wo, wi);
    else return leaf_evaluate_body<false>(f, wo, wi);
}
template <bool FULL = true>
__device__ __forceinline__ float leaf_pdf(const Bsdf& f, V3 wo, V3 wi) {
    if constexpr (FULL) return leaf_pdf_full(f, wo, wi);
    else return leaf_pdf_body<false>(f, wo, wi);
}
template <bool FULL = true>
__device__ __forceinline__ Col leaf_sample(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                           float& pdf) {
    if constexpr (FULL) return leaf_sample_full(f, u0, u1, u_scatter, wo, wi, pdf);
    else return leaf_sample_body<false>(f, u0, u1, u_scatter, wo, wi, pdf);
}

// FULL = false compiles out the plastic and coated-diffuse branches, for
// scenes that only use the diffuse, metal and rough-glass BSDFs.
// cos_delta_phi (src/lib/math.h:87-104): the cosine of the azimuth between a
// and b in the tangent plane (1 for a direction along the normal).
__device__ __forceinline__ float cos_delta_phi(V3 a, V3 b, V3 t1, V3 t2) {
    const float ax = dot(a, t1), ay = dot(a, t2), bx = dot(b, t1), by = dot(b, t2);
    const float a_len_sq = ax * ax + ay * ay, b_len_sq = bx * bx + by * by;
    if (a_len_sq == 0.f || b_len_sq == 0.f) return 1.f;
    const float cosine = (ax * bx + ay * by) / sqrtf(a_len_sq * b_len_sq);
    return cosine < -1.f ? -1.f : (1.f < cosine ? 1.f : cosine);
}

// The first zenith node not below c (std::lower_bound over increasing nodes;
// the last node is at least 1, so a clamped cosine always finds one).
__device__ __forceinline__ uint32_t fourier_node(const float* nodes, uint32_t count, float c) {
    uint32_t lo = 0, n = count;
    while (n > 0) {
        const uint32_t half = n / 2;
        if (__ldg(nodes + lo + half) < c) {
            lo += half + 1;
            n -= half + 1;
        } else {
            n = half;
        }
    }
    return lo;
}

// Pbrt3_Fourier_BSDF::evaluate (src/ref/bsdf_pbrt.cpp:305-358): the nearest
// node pair's Fourier series in the azimuth (no interpolation), divided by
// |cos_i|; three channels store Y, R, B.  acos and cos rounded correctly.
static __device__ __noinline__ Col fourier_evaluate(const Bsdf& f, V3 wo, V3 wi) {
    const Material_Dev& m = *f.sub[0];
    const V3 nwi = -wi;
    float cos_i = dot(f.n, nwi);
    cos_i = cos_i < -1.f ? -1.f : (1.f < cos_i ? 1.f : cos_i);
    float cos_o = dot(f.n, wo);
    cos_o = cos_o < -1.f ? -1.f : (1.f < cos_o ? 1.f : cos_o);
    const uint32_t nc = m.fourier_node_count;
    const uint32_t index = fourier_node(m.fourier_nodes, nc, cos_o) * nc + fourier_node(m.fourier_nodes, nc, cos_i);
    const float* coeffs = m.fourier_coeffs + __ldg(m.fourier_series + 2 * (size_t)index);
    const uint32_t count = __ldg(m.fourier_series + 2 * (size_t)index + 1);
    const float phi = (float)acos((double)cos_delta_phi(wo, nwi, f.t, f.bt));
    const float scale = cos_i != 0.f ? 1.f / fabsf(cos_i) : 0.f;
    if (m.fourier_channels == 1) {
        float y = 0.f;
        for (uint32_t i = 0; i < count; i++) y += __ldg(coeffs + i) * cos_f((float)i * phi);
        const float v = y * scale;
        return col(v, v, v);
    }
    float y = 0.f, r = 0.f, b = 0.f;
    for (uint32_t i = 0; i < count; i++) {
        const float c = cos_f((float)i * phi);
        y += __ldg(coeffs + i) * c;
        r += __ldg(coeffs + i + count) * c;
        b += __ldg(coeffs + i + 2 * count) * c;
    }
    const float g = 1.398304f * y - 0.297381f * r - 0.100923f * b;  // get_green_from_YRB, src/lib/color.cpp:26-29
    return col(r * scale, g * scale, b * scale);
}

template <bool FULL>
__device__ __forceinline__ Col leaf_evaluate_body(const Bsdf& f, V3 wo, V3 wi) {
    if (f.type == kDiffuse) return mul(f.reflectance, 1.f / kPi);
    if (FULL && f.type == kFourier) return fourier_evaluate(f, wo, wi);
    if (FULL && (f.type == kPlastic || f.type == kPbrt3Plastic)) {
        // Plastic_BRDF::evaluate (src/ref/bsdf.cpp:215-234); Pbrt3_Plastic_BRDF::evaluate
        // (src/ref/bsdf_pbrt.cpp:264-290) with pbrt-v3's swapped 1.0 / 1.5 IOR pair
        const V3 wh = normalized(wo + wi);
        const float cos_i = dot(wi, wh);
        Col F;
        if (f.type == kPbrt3Plastic) {
            const V3 original_n = f.flipped ? -f.n : f.n;
            const float fr = dielectric_fresnel(cos_i, dot(original_n, wi) < 0.f ? 1.5f / 1.f : 1.f / 1.5f);
            F = col(fr, fr, fr);
        } else {
            F = schlick_fresnel(col(0.04f, 0.04f, 0.04f), cos_i);
        }
        const float G = ggx_G(wi, wo, f.n, f.alpha);
        const float D = ggx_D(wh, f.n, f.alpha);
        const Col base = mul(F, (G * D) / (4.f * dot(wo, f.n) * dot(wi, f.n)));
        return mul(f.reflectance, 1.f / kPi) + mul(base, f.transmittance.r);
    }
    if (FULL && f.type == kDiffuseTransmission) {  // Diffuse_Transmission_BSDF::evaluate (bsdf.cpp:105-112)
        const bool same = dot(wo, f.n) * dot(wi, f.n) > 0.f;
        return mul(same ? f.reflectance : f.transmittance, 1.f / kPi);
    }
    if (FULL && f.type == kUber) {  // Pbrt3_Uber_BRDF::evaluate (bsdf_pbrt.cpp:34-52)
        const Col diffuse = mul(f.reflectance, 1.f / kPi) * f.extra;
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        const float F = dielectric_fresnel(dot(wi_l, wh_l), f.eta_i);
        const float G = ggx_G_aniso(wi_l, wo_l, f.alpha_x, f.alpha_y);
        const float D = ggx_D_aniso(wh_l, f.alpha_x, f.alpha_y);
        const float m = (F * G * D) / (4.f * wo_l.z * wi_l.z);
        return diffuse + mul(f.specular * f.extra, m);
    }
    if (FULL && f.type == kTranslucent) {  // Pbrt3_Translucent_BSDF::evaluate (bsdf_pbrt.cpp:117-158)
        if (dot(wo, f.n) * dot(wi, f.n) > 0.f) {
            const Col diffuse = mul(f.extra, 1.f / kPi) * f.reflectance;
            const V3 wh = normalized(wo + wi);
            const float F = dielectric_fresnel(dot(wi, wh), f.eta_i / f.eta_o);
            const float G = ggx_G(wi, wo, f.n, f.alpha);
            const float D = ggx_D(wh, f.n, f.alpha);
            const float base = (F * G * D) / (4.f * dot(wo, f.n) * dot(wi, f.n));
            return diffuse + mul(f.specular * f.reflectance, base);
        }
        const Col diffuse = mul(f.extra, 1.f / kPi) * f.transmittance;
        Col specular = col(0.f, 0.f, 0.f);
        const V3 wh = refraction_half(f.eta_o, wo, f.eta_i, wi, f.n);
        const float wo_wh = dot(wo, wh), wi_wh = dot(wi, wh);
        if (wo_wh * wi_wh <= 0.f) {
            const float F = dielectric_fresnel(wi_wh, f.eta_o / f.eta_i);
            if (F < 1.f) {
                const float G = ggx_G(wi, wo, f.n, f.alpha);
                const float D = ggx_D(wh, f.n, f.alpha);
                const float wo_n = dot(wo, f.n), wi_n = dot(wi, f.n);
                const float k = fabsf((wo_wh * wi_wh) / (wo_n * wi_n));
                const float k2 = f.eta_o * wo_wh + f.eta_i * wi_wh;
                const float base = (f.eta_o * f.eta_o * k * G * D * (1.f - F)) / (k2 * k2);
                specular = mul(f.specular * f.transmittance, base);
            }
        }
        return diffuse + specular;
    }
    if (FULL && f.type == kCoatedDiffuse) {
        // Ashikhmin_Shirley_Phong_BRDF::evaluate (src/ref/bsdf.cpp:440-460)
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        const float cos_i = dot(wi_l, wh_l);
        const Col F = schlick_fresnel(f.transmittance, cos_i);
        const float D = ggx_D_aniso(wh_l, f.alpha_x, f.alpha_y);
        const Col specular = mul(F, D / (4.f * cos_i * max_std(wo_l.z, wi_l.z)));
        const Col diffuse = mul(f.reflectance * (col(1.f, 1.f, 1.f) - f.transmittance),
                                28.f / (23.f * kPi) * (1.f - pow5(1.f - 0.5f * wi_l.z)) *
                                    (1.f - pow5(1.f - 0.5f * wo_l.z)));
        return diffuse + specular;
    }
    if (f.type == kMetal) {
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        const float cos_i = dot(wi_l, wh_l);
        const Col F = conductor_fresnel(cos_i, f.eta_i_metal, f.eta_t, f.k_t);
        const float G = ggx_G_aniso(wi_l, wo_l, f.alpha_x, f.alpha_y);
        const float D = ggx_D_aniso(wh_l, f.alpha_x, f.alpha_y);
        return mul(F, (G * D) / (4.f * wo_l.z * wi_l.z));
    }
    const bool same = dot(wo, f.n) * dot(wi, f.n) > 0.f;
    if (same) {
        const V3 wh = normalized(wo + wi);
        const float cos_i = dot(wi, wh);
        const float F = dielectric_fresnel(cos_i, f.eta_i / f.eta_o);
        const float G = ggx_G(wi, wo, f.n, f.alpha);
        const float D = ggx_D(wh, f.n, f.alpha);
        const float base = (F * G * D) / (4.f * dot(wo, f.n) * dot(wi, f.n));
        return mul(f.reflectance, base);
    }
    const V3 wh = refraction_half(f.eta_o, wo, f.eta_i, wi, f.n);
    const float wo_wh = dot(wo, wh), wi_wh = dot(wi, wh);
    if (wo_wh * wi_wh > 0.f) return col(0.f, 0.f, 0.f);
    const float cos_i = dot(wi, wh);
    const float F = dielectric_fresnel(cos_i, f.eta_o / f.eta_i);
    if (F == 1.f) return col(0.f, 0.f, 0.f);
    const float G = ggx_G(wi, wo, f.n, f.alpha);
    const float D = ggx_D(wh, f.n, f.alpha);
    const float wo_n = dot(wo, f.n), wi_n = dot(wi, f.n);
    const float k = fabsf((wo_wh * wi_wh) / (wo_n * wi_n));
    const float k2 = f.eta_o * wo_wh + f.eta_i * wi_wh;
    const float base = (f.eta_o * f.eta_o * k * G * D * (1.f - F)) / (k2 * k2);
    return mul(f.transmittance, base);
}

template <bool FULL>
__device__ __forceinline__ float leaf_pdf_body(const Bsdf& f, V3 wo, V3 wi) {
    // Pbrt3_Fourier_BSDF::pdf (src/ref/bsdf_pbrt.cpp:368-372): cosine-weighted as diffuse
    if (f.type == kDiffuse || (FULL && f.type == kFourier)) return dot(f.n, wi) / kPi;
    if (FULL && (f.type == kPlastic || f.type == kPbrt3Plastic)) {  // Plastic_BRDF::pdf (src/ref/bsdf.cpp:253-263)
        const float diffuse_pdf = dot(f.n, wi) / kPi;
        const V3 wh = normalized(wo + wi);
        const float spec_pdf = vndf_pdf(wo, wh, f.n, f.alpha) / (4 * dot(wh, wo));
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (FULL && f.type == kDiffuseTransmission) {  // Diffuse_Transmission_BSDF::pdf (bsdf.cpp:128-141)
        const float max_r = max_component(f.reflectance), max_t = max_component(f.transmittance);
        const float pdf = fabsf(dot(f.n, wi)) * (1.f / kPi);
        return dot(wo, f.n) * dot(wi, f.n) > 0.f ? (max_r / (max_r + max_t)) * pdf : (max_t / (max_r + max_t)) * pdf;
    }
    if (FULL && f.type == kUber) {  // Pbrt3_Uber_BRDF::pdf (bsdf_pbrt.cpp:74-87)
        const float diffuse_pdf = dot(f.n, wi) / kPi;
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        const float spec_pdf = vndf_pdf_aniso(wo_l, wh_l, f.alpha_x, f.alpha_y) / (4 * dot(wh_l, wo_l));
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (FULL && f.type == kTranslucent) {  // Pbrt3_Translucent_BSDF::pdf (bsdf_pbrt.cpp:211-250)
        const float max_r = max_component(f.reflectance), max_t = max_component(f.transmittance);
        const float rp = max_r / (max_r + max_t);
        if (dot(wo, f.n) * dot(wi, f.n) > 0.f) {
            const float diffuse_pdf = dot(wi, f.n) * (1.f / kPi);
            const V3 wh = normalized(wo + wi);
            const float spec_pdf = vndf_pdf(wo, wh, f.n, f.alpha) / (4 * dot(wh, wo));
            return rp * 0.5f * (diffuse_pdf + spec_pdf);
        }
        const float diffuse_pdf = -dot(wi, f.n) * (1.f / kPi);
        float spec_pdf = 0.f;
        const V3 wh = refraction_half(f.eta_o, wo, f.eta_i, wi, f.n);
        if (dot(wo, wh) * dot(wi, wh) <= 0.f) {
            const float wh_pdf = vndf_pdf(wo, wh, f.n, f.alpha);
            const float denom = f.eta_o * dot(wo, wh) + f.eta_i * dot(wi, wh);
            const float dwh = f.eta_i * f.eta_i * fabsf(dot(wi, wh)) / (denom * denom);
            spec_pdf = wh_pdf * dwh;
        }
        return (1.f - rp) * 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (FULL && f.type == kCoatedDiffuse) {  // Ashikhmin_Shirley_Phong_BRDF::pdf (src/ref/bsdf.cpp:480-492)
        const float diffuse_pdf = dot(f.n, wi) / kPi;
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        const float spec_pdf = vndf_pdf_aniso(wo_l, wh_l, f.alpha_x, f.alpha_y) / (4 * dot(wh_l, wo_l));
        return 0.5f * (diffuse_pdf + spec_pdf);
    }
    if (f.type == kMetal) {
        const V3 wo_l = world_to_local(f, wo), wi_l = world_to_local(f, wi);
        const V3 wh_l = normalized(wo_l + wi_l);
        return vndf_pdf_aniso(wo_l, wh_l, f.alpha_x, f.alpha_y) / (4 * dot(wh_l, wo_l));
    }
    const bool same = dot(wo, f.n) * dot(wi, f.n) > 0.f;
    if (same) {
        const V3 wh = normalized(wo + wi);
        const float rp = vndf_pdf(wo, wh, f.n, f.alpha) / (4 * dot(wh, wo));
        const float cos_i = dot(wi, wh);
        const float fr = dielectric_fresnel(cos_i, f.eta_i / f.eta_o);
        return rp * glass_reflection_probability(f, fr);
    }
    const V3 wh = refraction_half(f.eta_o, wo, f.eta_i, wi, f.n);
    const float wo_wh = dot(wo, wh), wi_wh = dot(wi, wh);
    if (wo_wh * wi_wh > 0.f) return 0.f;
    const float fr = dielectric_fresnel(dot(wo, wh), f.eta_i / f.eta_o);
    const float rprob = glass_reflection_probability(f, fr);
    const float wh_pdf = vndf_pdf(wo, wh, f.n, f.alpha);
    const float denom = f.eta_o * dot(wo, wh) + f.eta_i * dot(wi, wh);
    const float dwh = f.eta_i * f.eta_i * fabsf(dot(wi, wh)) / (denom * denom);
    return (wh_pdf * dwh) * (1.f - rprob);
}

// BSDF::sample; black when no direction is produced.
template <bool FULL>
__device__ __forceinline__ Col leaf_sample_body(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                                float& pdf) {
    if (FULL && f.type == kDiffuseTransmission) {  // Diffuse_Transmission_BSDF::sample (bsdf.cpp:114-126)
        const float max_r = max_component(f.reflectance), max_t = max_component(f.transmittance);
        const float sign = u_scatter < max_r / (max_r + max_t) ? 1.f : -1.f;
        wi = local_to_world(f, mul(sample_hemisphere_cosine(u0, u1), sign));
        pdf = leaf_pdf<FULL>(f, wo, wi);
        return leaf_evaluate<FULL>(f, wo, wi);
    }
    if (FULL && f.type == kTranslucent) {  // Pbrt3_Translucent_BSDF::sample (bsdf_pbrt.cpp:160-209)
        const float max_r = max_component(f.reflectance), max_t = max_component(f.transmittance);
        const float rp = max_r / (max_r + max_t);
        const bool reflect_side = u_scatter < rp;
        const float u = one_minus_eps_min_s(reflect_side ? u_scatter / rp : (u_scatter - rp) / (1.f - rp));
        if (u < 0.5f) {
            const V3 l = sample_hemisphere_cosine(u0, u1);
            wi = local_to_world(f, reflect_side ? l : -l);
        } else {
            const V3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, world_to_local(f, wo), f.alpha, f.alpha));
            if (reflect_side) {
                const V3 c = reflect(wo, wh);
                if (dot(c, f.n) <= 0.f) return col(0.f, 0.f, 0.f);
                wi = c;
            } else {
                if (dot(wh, wo) < 0.f) return col(0.f, 0.f, 0.f);
                V3 c;
                if (!refract(wo, wh, f.eta_o / f.eta_i, c)) return col(0.f, 0.f, 0.f);
                if (dot(c, f.n) >= 0.f) return col(0.f, 0.f, 0.f);
                wi = c;
            }
        }
        pdf = leaf_pdf<FULL>(f, wo, wi);
        if (pdf == 0.f) return col(0.f, 0.f, 0.f);
        return leaf_evaluate<FULL>(f, wo, wi);
    }
    if (FULL && (f.type == kPlastic || f.type == kPbrt3Plastic || f.type == kCoatedDiffuse || f.type == kUber)) {
        // Plastic_BRDF::sample (src/ref/bsdf.cpp:236-251), Ashikhmin_Shirley_Phong_BRDF::sample
        // (:462-478): the first 1D sample picks the diffuse or the specular lobe
        if (u_scatter < 0.5f) {
            wi = local_to_world(f, sample_hemisphere_cosine(u0, u1));
        } else {
            const V3 wo_l = world_to_local(f, wo);
            if (f.type == kCoatedDiffuse || f.type == kUber) {
                const V3 wh_l = ggx_sample_vndf(u0, u1, wo_l, f.alpha_x, f.alpha_y);
                wi = local_to_world(f, reflect(wo_l, wh_l));
            } else {
                const V3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, wo_l, f.alpha, f.alpha));
                wi = reflect(wo, wh);
            }
        }
        if (dot(f.n, wi) <= 0.f) return col(0.f, 0.f, 0.f);
        pdf = leaf_pdf<FULL>(f, wo, wi);
        return leaf_evaluate<FULL>(f, wo, wi);
    }
    if (f.type == kDiffuse || (FULL && f.type == kFourier)) {  // Pbrt3_Fourier_BSDF::sample: as diffuse
        wi = local_to_world(f, sample_hemisphere_cosine(u0, u1));
        pdf = leaf_pdf<FULL>(f, wo, wi);
        return leaf_evaluate<FULL>(f, wo, wi);
    }
    if (f.type == kMetal) {
        const V3 wo_l = world_to_local(f, wo);
        const V3 wh_l = ggx_sample_vndf(u0, u1, wo_l, f.alpha_x, f.alpha_y);
        const V3 wi_l = reflect(wo_l, wh_l);
        if (wi_l.z <= 0.f) return col(0.f, 0.f, 0.f);
        wi = local_to_world(f, wi_l);
        pdf = vndf_pdf_aniso(wo_l, wh_l, f.alpha_x, f.alpha_y) / (4 * dot(wh_l, wo_l));
        return leaf_evaluate<FULL>(f, wo, wi);
    }
    const V3 wo_l = world_to_local(f, wo);
    const V3 wh = local_to_world(f, ggx_sample_vndf(u0, u1, wo_l, f.alpha, f.alpha));
    const V3 rwi = reflect(wo, wh);
    if (dot(rwi, f.n) <= 0.f) return col(0.f, 0.f, 0.f);
    const float fresnel = dielectric_fresnel(dot(wo, wh), f.eta_i / f.eta_o);
    const float rprob = glass_reflection_probability(f, fresnel);
    if (u_scatter < rprob) {
        wi = rwi;
    } else {
        if (!refract(wo, wh, f.eta_o / f.eta_i, wi)) return col(0.f, 0.f, 0.f);
        if (dot(wi, f.n) >= 0.f) return col(0.f, 0.f, 0.f);
    }
    pdf = leaf_pdf<FULL>(f, wo, wi);
    if (pdf == 0.f) return col(0.f, 0.f, 0.f);
    return leaf_evaluate<FULL>(f, wo, wi);
}

// Mix_BSDF (src/ref/bsdf.cpp:497-567) and Scaled_BSDF (:572-592) over leaf BSDFs;
// every other BSDF forwards.  FULL = false compiles the mix out.
__device__ __forceinline__ bool possible_for(const Bsdf& f, float n_dot_wi) {
    return (n_dot_wi > 0.f && f.reflection) || (n_dot_wi < 0.f && f.transmission);
}
template <bool FULL>
__device__ __forceinline__ Col bsdf_evaluate_body(const Bsdf& f, V3 wo, V3 wi) {
    if (FULL && f.type == kScaled) {
        Bsdf a = f;
        set_material(a, *f.sub[0]);
        return mul(leaf_evaluate<true>(a, wo, wi), f.mix_p);
    }
    if (FULL && f.type == kMix) {
        Bsdf a = f, b = f;
        set_material(a, *f.sub[0]);
        set_material(b, *f.sub[1]);
        Col f1 = col(0.f, 0.f, 0.f), f2 = col(0.f, 0.f, 0.f);
        const float n_dot_wi = dot(f.n, wi);
        if (possible_for(a, n_dot_wi)) f1 = leaf_evaluate<true>(a, wo, wi);
        if (possible_for(b, n_dot_wi)) f2 = leaf_evaluate<true>(b, wo, wi);
        return (col(1.f, 1.f, 1.f) - f.mix_coeff) * f1 + f.mix_coeff * f2;
    }
    return leaf_evaluate<FULL>(f, wo, wi);
}
template <bool FULL>
__device__ __forceinline__ float bsdf_pdf_body(const Bsdf& f, V3 wo, V3 wi) {
    if (FULL && f.type == kScaled) {
        Bsdf a = f;
        set_material(a, *f.sub[0]);
        return leaf_pdf<true>(a, wo, wi);
    }
    if (FULL && f.type == kMix) {
        Bsdf a = f, b = f;
        set_material(a, *f.sub[0]);
        set_material(b, *f.sub[1]);
        float pdf1 = 0.f, pdf2 = 0.f;
        const float n_dot_wi = dot(f.n, wi);
        if (possible_for(a, n_dot_wi)) pdf1 = leaf_pdf<true>(a, wo, wi);
        if (possible_for(b, n_dot_wi)) pdf2 = leaf_pdf<true>(b, wo, wi);
        return (1.f - f.mix_p) * pdf1 + f.mix_p * pdf2;
    }
    return leaf_pdf<FULL>(f, wo, wi);
}
// wi must come in as the zero vector: the reference's default-constructed
// direction, which a leaf sample that gives up early leaves as it is.
template <bool FULL>
__device__ __forceinline__ Col bsdf_sample_body(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                                float& pdf) {
    if (FULL && f.type == kScaled) {
        Bsdf a = f;
        set_material(a, *f.sub[0]);
        return mul(leaf_sample<true>(a, u0, u1, u_scatter, wo, wi, pdf), f.mix_p);
    }
    if (FULL && f.type == kMix) {
        Bsdf a = f, b = f;
        set_material(a, *f.sub[0]);
        set_material(b, *f.sub[1]);
        Col f1 = col(0.f, 0.f, 0.f), f2 = col(0.f, 0.f, 0.f);
        float pdf1 = 0.f, pdf2 = 0.f;
        if (u_scatter < f.mix_p) {
            f2 = leaf_sample<true>(b, u0, u1, u_scatter / f.mix_p, wo, wi, pdf2);
            if (possible_for(a, dot(f.n, wi))) {
                pdf1 = leaf_pdf<true>(a, wo, wi);
                f1 = leaf_evaluate<true>(a, wo, wi);
            }
        } else {
            f1 = leaf_sample<true>(a, u0, u1, (u_scatter - f.mix_p) / (1.f - f.mix_p), wo, wi, pdf1);
            if (possible_for(b, dot(f.n, wi))) {
                pdf2 = leaf_pdf<true>(b, wo, wi);
                f2 = leaf_evaluate<true>(b, wo, wi);
            }
        }
        pdf = (1.f - f.mix_p) * pdf1 + f.mix_p * pdf2;
        return (col(1.f, 1.f, 1.f) - f.mix_coeff) * f1 + f.mix_coeff * f2;
    }
    return leaf_sample<FULL>(f, u0, u1, u_scatter, wo, wi, pdf);
}

static __device__ __noinline__ Col bsdf_evaluate_full(const Bsdf& f, V3 wo, V3 wi) { return bsdf_evaluate_body<true>(f, wo, wi); }
static __device__ __noinline__ float bsdf_pdf_full(const Bsdf& f, V3 wo, V3 wi) { return bsdf_pdf_body<true>(f, wo, wi); }
static __device__ __noinline__ Col bsdf_sample_full(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                             float& pdf) {
    return bsdf_sample_body<true>(f, u0, u1, u_scatter, wo, wi, pdf);
}
// The plain (diffuse, metal, rough glass) sampling routine is called out of
// line too: the shade kernel calls it at two places, and its stalls are mostly
// instruction fetch (ncu: 29.6 cycles of no_instruction per issue).  C3 render
// on GB300: 1.546 s against 1.598 s inlined; evaluation out of line as well
// measured 1.565 s.
static __device__ __noinline__ Col bsdf_sample_plain(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo,
                                                     V3& wi, float& pdf) {
    return bsdf_sample_body<false>(f, u0, u1, u_scatter, wo, wi, pdf);
}
template <bool FULL = true>
__device__ __forceinline__ Col bsdf_evaluate(const Bsdf& f, V3 wo, V3 wi) {
    if constexpr (FULL) return bsdf_evaluate_full(f, wo, wi);
    else return bsdf_evaluate_body<false>(f, wo, wi);
}
template <bool FULL = true>
__device__ __forceinline__ float bsdf_pdf(const Bsdf& f, V3 wo, V3 wi) {
    if constexpr (FULL) return bsdf_pdf_full(f, wo, wi);
    else return bsdf_pdf_body<false>(f, wo, wi);
}
template <bool FULL = true>
__device__ __forceinline__ Col bsdf_sample(const Bsdf& f, float u0, float u1, float u_scatter, V3 wo, V3& wi,
                                           float& pdf) {
    if constexpr (FULL) return bsdf_sample_full(f, u0, u1, u_scatter, wo, wi, pdf);
    else return bsdf_sample_plain(f, u0, u1, u_scatter, wo, wi, pdf);
}

// mis_power_heuristic (src/ref/direct_lighting.cpp:18-24)
__device__ __forceinline__ float mis_power(float p1, float p2) {
    if (p1 == __int_as_float(0x7f800000)) return 1.f;
    return p1 * p1 / (p1 * p1 + p2 * p2);
}

// ---------------------------------------------------------------- pcg32
// pcg32 (third-party/pcg/pcg_basic.c:46-75) and RNG::get_float / bounded
// draws (src/lib/random.h:17-72)
struct Pcg {
    uint64_t state, inc;
};
__device__ __forceinline__ uint32_t pcg_next(Pcg& r) {
    const uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + r.inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((-rot) & 31));
}
__device__ __forceinline__ Pcg pcg_seed(uint64_t initstate, uint64_t initseq) {
    Pcg r;
    r.state = 0u;
    r.inc = (initseq << 1u) | 1u;
    pcg_next(r);
    r.state += initstate;
    pcg_next(r);
    return r;
}
__device__ __forceinline__ float pcg_float(Pcg& r) {
    return __uint_as_float((pcg_next(r) >> 9) | 0x3f800000u) - 1.0f;
}
__device__ __forceinline__ uint32_t pcg_bounded_fast(Pcg& r, uint32_t bound) {
    return (uint32_t)(((uint64_t)pcg_next(r) * bound) >> 32);
}

} // namespace yar
