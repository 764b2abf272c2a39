// direct.cu - the reference's direct-lighting algorithm on the device
// (estimate_direct_lighting, src/ref/direct_lighting.cpp:415-520; render_scene's
// pixel loop, src/ref/reference_renderer.cpp:331-409).
//
// Per sample: the camera ray, then at its hit every point and directional
// light, every rectangular and sphere light over its k x k sample arrays, the
// environment light over its sample count, and the delta ray of a delta
// event.  The sample arrays are extra rows of the sample tables (2D array
// grids before 1D ones, as Stratified_Pixel_Sampler::next_pixel draws them).
// The draws past the tables (the scattering-type sample, the environment's
// light and BSDF samples) come from the pixel's pcg stream in sample order; a
// sample's share of them depends on what its camera ray hit, so the kernel
// runs in three passes: camera rays and their draw counts, the per-pixel
// prefix of those counts, then the shading of every sample from its own
// jump-ahead of the pixel stream.  Shadow and probe rays are traced inline.
#include "wavefront.cuh"

namespace yar {

namespace {

// A ray traced inside a kernel: the traversal reloads the world ray from a
// ray record, so every thread owns one record in `rec` (2 float4).
__device__ __forceinline__ bool trace_inline_closest(const Scene_Dev& S, float4* rec, uint32_t slot, V3 o, V3 d,
                                                     float4& h4, uint2& h2, int* err) {
    rec[2 * (size_t)slot] = make_float4(o.x, o.y, o.z, __int_as_float(0x7f800000));
    rec[2 * (size_t)slot + 1] = make_float4(d.x, d.y, d.z, 0.f);
    Traversal<false> tr;
    Local_Stack stack;
    tr.begin(S.ds, slot, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), __int_as_float(0x7f800000));
    while (tr.template step<1 << 30>(S.ds, rec, stack)) {
    }
    const int status = tr.status();
    if (status < 0) atomicOr(err, 1);
    atomicAdd(reinterpret_cast<unsigned long long*>(err + 2), 1ull);  // closest-hit rays
    h4 = make_float4(tr.hit.t, tr.hit.b0, tr.hit.b1, tr.hit.b2);
    h2 = status > 0 ? make_uint2(tr.hit.prim, tr.hit.object) : make_uint2(0xffffffffu, 0xffffffffu);
    return status > 0;
}
__device__ __forceinline__ bool trace_inline_any(const Scene_Dev& S, float4* rec, uint32_t slot, V3 o, V3 d,
                                                 float tmax, int* err) {
    rec[2 * (size_t)slot] = make_float4(o.x, o.y, o.z, tmax);
    rec[2 * (size_t)slot + 1] = make_float4(d.x, d.y, d.z, 0.f);
    Traversal<true> tr;
    Local_Stack stack;
    tr.begin(S.ds, slot, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), tmax);
    while (tr.template step<1 << 30>(S.ds, rec, stack)) {
    }
    const int status = tr.status();
    if (status < 0) atomicOr(err, 1);
    atomicAdd(reinterpret_cast<unsigned long long*>(err + 4), 1ull);  // any-hit rays
    return status > 0;
}

__device__ __forceinline__ int4 object_info(const Scene_Dev& S, uint32_t object) {
    const float4 f = __ldg(S.obj_render + 7 * (size_t)object + 6);
    return make_int4(__float_as_int(f.x), __float_as_int(f.y), __float_as_int(f.z), __float_as_int(f.w));
}

// get_emitted_radiance (direct_lighting.cpp:386-413) of a light object hit.
__device__ __forceinline__ Col emitted(const Scene_Dev& S, int4 oinfo, bool flipped) {
    if ((uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_RECTANGULAR) {
        const float4 le = __ldg(&S.lights[oinfo.w].le);
        return col(le.x, le.y, le.z);
    }
    if ((uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_SPHERE) {
        const float4 le = __ldg(&S.sphere_lights[oinfo.w].le);
        return col(le.x, le.y, le.z);
    }
    if ((uint32_t)oinfo.z == YAR_LIGHT_DIFFUSE_TRIANGLE_MESH && !flipped) {
        const float4 le = __ldg(&S.mesh_lights[oinfo.w].le);
        return col(le.x, le.y, le.z);
    }
    return col(0.f, 0.f, 0.f);
}

// direct_lighting_from_point_light / _directional_light (direct_lighting.cpp:26-107)
__device__ Col direct_point_or_directional(const Scene_Dev& S, const Shading& sc, const Bsdf& f, int i, float4* rec,
                                           uint32_t slot, int* err) {
    const Delta_Light_Dev& D = S.delta_lights[i];
    const float4 da = __ldg(&D.a), db = __ldg(&D.b), dc = __ldg(&D.c);
    const Col I = col(dc.x, dc.y, dc.z);
    if (__float_as_uint(da.w) == YAR_LIGHT_DIRECTIONAL) {
        const V3 dir = v3(db.x, db.y, db.z);
        const float n_dot_l = dot(sc.n, dir);
        if (n_dot_l <= 0.f) return col(0.f, 0.f, 0.f);
        if (trace_inline_any(S, rec, slot, origin_for_direction(sc, dir), dir, __int_as_float(0x7f800000), err))
            return col(0.f, 0.f, 0.f);
        return mul(I * bsdf_evaluate<true>(f, sc.wo, dir), n_dot_l);
    }
    const V3 lp = v3(da.x, da.y, da.z);
    const V3 position = origin_for_point(sc, lp);
    const V3 lv = lp - position;
    const float dist = len(lv);
    const V3 wi = divs(lv, dist);
    const float n_dot_l = dot(sc.n, wi);
    if (n_dot_l <= 0.f) return col(0.f, 0.f, 0.f);
    if (trace_inline_any(S, rec, slot, position, wi, dist * (1.f - 1e-5f), err)) return col(0.f, 0.f, 0.f);
    return mul(I * bsdf_evaluate<true>(f, sc.wo, wi), n_dot_l / (dist * dist));
}

// direct_lighting_from_rectangular_light (direct_lighting.cpp:109-194)
__device__ Col direct_rect(const Scene_Dev& S, const Shading& sc, const Bsdf& f, int light, float2 ul, float2 ub,
                           float u_scatter, float4* rec, uint32_t slot, int* err) {
    const Rect_Light_Dev& Ld = S.lights[light];
    const float4 lr0 = __ldg(&Ld.r0), lr1 = __ldg(&Ld.r1), lr2 = __ldg(&Ld.r2);
    const float4 lle = __ldg(&Ld.le), lsz = __ldg(&Ld.sz);
    const V3 light_n = v3(lr0.z, lr1.z, lr2.z);
    const Col Le = col(lle.x, lle.y, lle.z);
    const float size_x = lle.w, size_y = lsz.x;
    Col out = col(0.f, 0.f, 0.f);
    bool have = false;
    {
        const V3 lp = xform_point(lr0, lr1, lr2, v3(size_x * (ul.x - 0.5f), size_y * (ul.y - 0.5f), 0.0f));
        const V3 position = origin_for_point(sc, lp);
        const V3 lv = lp - position;
        const float dist = len(lv);
        const V3 wi = divs(lv, dist);
        const float lndw = dot(light_n, -wi);
        if (lndw > 1e-4f) {
            const float ndw = dot(sc.n, wi);
            if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
                const Col fv = bsdf_evaluate<true>(f, sc.wo, wi);
                if (!black(fv) && !trace_inline_any(S, rec, slot, position, wi, dist * (1.f - 1e-5f), err)) {
                    const float light_pdf = (dist * dist) / (size_x * size_y * lndw);
                    const float w = mis_power(light_pdf, bsdf_pdf<true>(f, sc.wo, wi));
                    out = col(0.f, 0.f, 0.f) + mul(Le * fv, w * fabsf(ndw) / light_pdf);
                    have = true;
                }
            }
        }
    }
    {
        V3 wi = v3(0.f, 0.f, 0.f);
        float bpdf = 0.f;
        const Col fv = bsdf_sample<true>(f, ub.x, ub.y, u_scatter, sc.wo, wi, bpdf);
        if (!black(fv)) {
            const float lndw = dot(light_n, -wi);
            if (lndw > 1e-4f) {
                const V3 position = origin_for_direction(sc, wi);
                float4 h4;
                uint2 h2;
                if (trace_inline_closest(S, rec, slot, position, wi, h4, h2, err)) {
                    const int4 oi = object_info(S, h2.y);
                    if ((uint32_t)oi.z == YAR_LIGHT_DIFFUSE_RECTANGULAR && oi.w == light) {
                        const uint32_t tri_offset = __float_as_uint(__ldg(S.ds.objects + 6 * (size_t)h2.y + 4).w);
                        const size_t g = (size_t)tri_offset + h2.x;
                        const float4 q0 = __ldg(S.ds.tris + 3 * g), q1 = __ldg(S.ds.tris + 3 * g + 1),
                                     q2 = __ldg(S.ds.tris + 3 * g + 2);
                        const V3 hp = bary(v3(q0.x, q0.y, q0.z), v3(q1.x, q1.y, q1.z), v3(q2.x, q2.y, q2.z), h4.y,
                                           h4.z, h4.w);
                        const float d = len(hp - position);
                        const float light_pdf = (d * d) / (size_x * size_y * lndw);
                        const float w = mis_power(bpdf, light_pdf);
                        const Col c = mul(Le * fv, w * fabsf(dot(sc.n, wi)) / bpdf);
                        out = have ? out + c : col(0.f, 0.f, 0.f) + c;
                    }
                }
            }
        }
    }
    return out;
}

// direct_lighting_from_sphere_light (direct_lighting.cpp:196-260)
__device__ Col direct_sphere(const Scene_Dev& S, const Shading& sc, const Bsdf& f, int light, float2 ul, float2 ub,
                             float u_scatter, float4* rec, uint32_t slot, int* err) {
    const float4 sa = __ldg(&S.sphere_lights[light].a), sle = __ldg(&S.sphere_lights[light].le);
    const Col Le = col(sle.x, sle.y, sle.z);
    Sphere_Sampler ss;
    sphere_sampler_init(ss, v3(sa.x, sa.y, sa.z), sa.w, sc.position);
    Col out = col(0.f, 0.f, 0.f);
    bool have = false;
    {
        const V3 lp = sphere_sampler_sample(ss, ul.x, ul.y);
        const V3 position = origin_for_point(sc, lp);
        const V3 lv = lp - position;
        const float dist = len(lv);
        const V3 wi = divs(lv, dist);
        const float ndw = dot(sc.n, wi);
        if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
            const Col fv = bsdf_evaluate<true>(f, sc.wo, wi);
            if (!black(fv) && !trace_inline_any(S, rec, slot, position, wi, dist * (1.f - 1e-5f), err)) {
                const float w = mis_power(ss.cone_pdf, bsdf_pdf<true>(f, sc.wo, wi));
                out = col(0.f, 0.f, 0.f) + mul(Le * fv, w * fabsf(ndw) / ss.cone_pdf);
                have = true;
            }
        }
    }
    {
        V3 wi = v3(0.f, 0.f, 0.f);
        float bpdf = 0.f;
        const Col fv = bsdf_sample<true>(f, ub.x, ub.y, u_scatter, sc.wo, wi, bpdf);
        if (!black(fv) && dot(-ss.axes[2], wi) >= ss.cos_theta_max) {
            float4 h4;
            uint2 h2;
            if (trace_inline_closest(S, rec, slot, origin_for_direction(sc, wi), wi, h4, h2, err)) {
                const int4 oi = object_info(S, h2.y);
                if ((uint32_t)oi.z == YAR_LIGHT_DIFFUSE_SPHERE && oi.w == light) {
                    const float w = mis_power(bpdf, ss.cone_pdf);
                    const Col c = mul(Le * fv, w * fabsf(dot(sc.n, wi)) / bpdf);
                    out = have ? out + c : col(0.f, 0.f, 0.f) + c;
                }
            }
        }
    }
    return out;
}

// direct_lighting_from_environment_light (direct_lighting.cpp:324-384)
__device__ Col direct_env(const Scene_Dev& S, const Shading& sc, const Bsdf& f, float2 ul, float2 ub, float u_scatter,
                          float4* rec, uint32_t slot, int* err) {
    Col out = col(0.f, 0.f, 0.f);
    bool have = false;
    {
        V3 wi;
        float light_pdf;
        const Col Le = env_light_sample(S, ul.x, ul.y, wi, light_pdf);
        const float ndw = dot(sc.n, wi);
        if ((ndw > 0.f && f.reflection) || (ndw < 0.f && f.transmission)) {
            const Col fv = bsdf_evaluate<true>(f, sc.wo, wi);
            if (!black(fv) && !trace_inline_any(S, rec, slot, origin_for_direction(sc, wi), wi,
                                                __int_as_float(0x7f800000), err)) {
                const float w = mis_power(light_pdf, bsdf_pdf<true>(f, sc.wo, wi));
                out = col(0.f, 0.f, 0.f) + mul(Le * fv, w * fabsf(ndw) / light_pdf);
                have = true;
            }
        }
    }
    {
        V3 wi = v3(0.f, 0.f, 0.f);
        float bpdf = 0.f;
        const Col fv = bsdf_sample<true>(f, ub.x, ub.y, u_scatter, sc.wo, wi, bpdf);
        if (!black(fv)) {
            const Col Le = env_radiance(S, wi, false);
            if (!black(Le) && !trace_inline_any(S, rec, slot, origin_for_direction(sc, wi), wi,
                                                __int_as_float(0x7f800000), err)) {
                const float w = mis_power(bpdf, env_light_pdf(S, wi));
                const Col c = mul(Le * fv, w * fabsf(dot(sc.n, wi)) / bpdf);
                out = have ? out + c : col(0.f, 0.f, 0.f) + c;
            }
        }
    }
    return out;
}

// Pass 1: the camera ray of every sample of the chunk, its hit, and how many
// raw pcg draws its shading takes (the scattering-type sample, then 5 per
// environment sample when the hit has a BSDF).
__global__ void __launch_bounds__(kBlock)
direct_camera_kernel(Render_Params p, Scene_Dev S, uint32_t paths, const Queues q, float4* rec, float4* hit4,
                     uint2* hit2, uint32_t* draws, int env_samples, int* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= paths) return;
    const float4 r0 = q.ext_rays[0][2 * (size_t)i], r1 = q.ext_rays[0][2 * (size_t)i + 1];
    float4 h4;
    uint2 h2;
    const bool hit = trace_inline_closest(S, rec, i, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), h4, h2, err);
    hit4[i] = h4;
    hit2[i] = h2;
    uint32_t n = 0;
    if (hit) {
        n = 1;
        const int4 oi = object_info(S, h2.y);
        if ((uint32_t)oi.z == YAR_LIGHT_NULL && (uint32_t)oi.x != YAR_MATERIAL_NULL && S.env_map &&
            S.materials[oi.y].has_bsdf)
            n += 5u * (uint32_t)env_samples;
    }
    draws[i] = n;
}

// Pass 2: a pixel's draws in sample order become each sample's offset.
__global__ void direct_prefix_kernel(uint32_t pixels, int spp, uint32_t* draws) {
    const uint32_t lp = blockIdx.x * blockDim.x + threadIdx.x;
    if (lp >= pixels) return;
    uint32_t acc = 0;
    for (int k = 0; k < spp; k++) {
        const uint32_t n = draws[(size_t)lp * spp + k];
        draws[(size_t)lp * spp + k] = acc;
        acc += n;
    }
}

// Pass 3: estimate_direct_lighting of every sample.
// TEXTURED: image textures or bump maps in the scene (a separate
// instantiation: their calls take the plain kernel from 228 registers without
// spills to 168 with 768 B of spill stores).
template <bool TEXTURED>
__global__ void __launch_bounds__(kBlock)
direct_shade_kernel(Render_Params p, Scene_Dev S, uint32_t chunk_first, uint32_t paths, const Queues q, float4* rec,
                    const float4* __restrict__ hit4, const uint2* __restrict__ hit2,
                    const uint32_t* __restrict__ draw_offset, uint32_t stream_base, const float* __restrict__ s1d,
                    const float2* __restrict__ s2d, const int* __restrict__ array_sides, int env_samples,
                    const float2* __restrict__ image_samples, float4* __restrict__ radiance, int* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= paths) return;
    const uint32_t lp = i / (uint32_t)p.spp, sample = i - lp * (uint32_t)p.spp;
    const float4 r1 = q.ext_rays[0][2 * (size_t)i + 1];
    const V3 dir = v3(r1.x, r1.y, r1.z);
    Col L = col(0.f, 0.f, 0.f);
    const uint2 h2 = hit2[i];
    if (h2.y == 0xffffffffu) {
        if (S.env_map) L = env_radiance(S, dir, true);
    } else {
        int x, y;
        Pcg rng = pixel_pcg(p, pixel_stream(p, chunk_first + lp, x, y));
        pcg_advance(rng, stream_base + draw_offset[i]);
        const float4 h4 = hit4[i];
        Shading sc;
        int4 oinfo;
        init_shading(S, dir, h2.y, h2.x, h4.y, h4.z, h4.w, sc, oinfo);
        float u_sc = pcg_float(rng);
        float bsdf_prob = 1.f;
        V3 delta_wi = v3(0.f, 0.f, 0.f);
        Col delta_atten = col(1.f, 1.f, 1.f);
        int delta = 0;
        const bool is_light = (uint32_t)oinfo.z != YAR_LIGHT_NULL;
        const Material_Dev* mat = (uint32_t)oinfo.x != YAR_MATERIAL_NULL ? &S.materials[oinfo.y] : nullptr;
        // Image textures and bump maps at the camera hit, with the camera ray's
        // differentials (the delta ray's hit adds its emission only)
        Tex_Site site;
        const bool textured = TEXTURED && mat && !is_light && (mat->texture | mat->texture2 | mat->bump) != 0u;
        if (textured) {
            Path_State ps{};
            ps.image_samples = image_samples;
            ps.chunk_first = chunk_first;
            texture_site(p, S, ps, i, 0, 0u, sc, h4, h2, site);
            if (mat->bump) apply_bump(S, *mat, site, h2.y, h2.x, h4.y, h4.z, h4.w, sc);
        }
        float delta_kind = 0.f;
        if (mat && mat->delta != kDeltaNone) {
            delta = delta_scattering(sc, *mat, S.materials, u_sc, delta_wi, delta_atten, bsdf_prob, delta_kind);
            if (textured && delta == 1 && mat->delta == kDeltaGlass && (mat->texture | mat->texture2) != 0u)
                delta_atten = textured_glass_attenuation(S, site, *mat, delta_kind, delta_atten);
        }
        if (is_light) {
            L = emitted(S, oinfo, sc.flipped);
        } else if (mat && (delta == 0 || bsdf_prob != 0.f)) {
            Bsdf f;
            make_bsdf(sc, *mat, S.materials, f);
            if (textured && (mat->texture | mat->texture2) != 0u) textured_bsdf_params(S, site, *mat, f);
            for (int l = 0; l < p.delta_lights; l++)  // point lights, then directional lights
                if (__float_as_uint(__ldg(&S.delta_lights[l].a).w) == YAR_LIGHT_POINT)
                    L = L + direct_point_or_directional(S, sc, f, l, rec, i, err);
            for (int l = 0; l < p.delta_lights; l++)
                if (__float_as_uint(__ldg(&S.delta_lights[l].a).w) == YAR_LIGHT_DIRECTIONAL)
                    L = L + direct_point_or_directional(S, sc, f, l, rec, i, err);
            // the sample arrays: per rectangular, then sphere light: light grids, BSDF grids, scattering grids
            int grid2 = 0, grid1 = 0;
            const float* s1 = s1d + (size_t)lp * p.n1d * p.spp + sample;
            const float2* s2 = s2d + (size_t)lp * p.n2d * p.spp + sample;
            for (int kind = 0; kind < 2; kind++) {
                const int n = kind == 0 ? p.rect_lights : p.sphere_lights;
                for (int l = 0; l < n; l++) {
                    const int k = array_sides[kind == 0 ? l : p.rect_lights + l];
                    const int count = k * k;
                    Col L2 = col(0.f, 0.f, 0.f);
                    const float da = 1.f / (float)k, d1 = 1.f / (float)count;
                    for (int e = 0; e < count; e++) {
                        // Stratified_Pixel_Sampler's array element e of this sample
                        // (pixel_sampling.cpp:100-141): grid e at the sample's position
                        const float2 g0 = s2[(size_t)(grid2 + e) * p.spp];
                        const float2 g1 = s2[(size_t)(grid2 + count + e) * p.spp];
                        const float g2 = s1[(size_t)(grid1 + e) * p.spp];
                        const int ex = e % k, ey = e / k;
                        const float2 ul = make_float2(one_minus_eps_min(((float)ex + g0.x) * da),
                                                      one_minus_eps_min(((float)ey + g0.y) * da));
                        const float2 ub = make_float2(one_minus_eps_min(((float)ex + g1.x) * da),
                                                      one_minus_eps_min(((float)ey + g1.y) * da));
                        const float us = one_minus_eps_min(((float)e + g2) * d1);
                        L2 = L2 + (kind == 0 ? direct_rect(S, sc, f, l, ul, ub, us, rec, i, err)
                                             : direct_sphere(S, sc, f, l, ul, ub, us, rec, i, err));
                    }
                    L = L + mul(L2, 1.f / (float)count);  // ColorRGB::operator/= multiplies by 1/v
                    grid2 += 2 * count;
                    grid1 += count;
                }
            }
            if (S.env_map) {
                Col L2 = col(0.f, 0.f, 0.f);
                for (int e = 0; e < env_samples; e++) {
                    const float ul0 = pcg_float(rng), ul1 = pcg_float(rng);
                    const float ub0 = pcg_float(rng), ub1 = pcg_float(rng);
                    const float us = pcg_float(rng);
                    L2 = L2 + direct_env(S, sc, f, make_float2(ul0, ul1), make_float2(ub0, ub1), us, rec, i, err);
                }
                L = L + mul(L2, 1.f / (float)env_samples);
            }
        }
        if (delta == 1) {
            float4 dh4;
            uint2 dh2;
            Col em = col(0.f, 0.f, 0.f);
            if (trace_inline_closest(S, rec, i, origin_for_direction(sc, delta_wi), delta_wi, dh4, dh2, err)) {
                Shading dsc;
                int4 doi;
                init_shading(S, delta_wi, dh2.y, dh2.x, dh4.y, dh4.z, dh4.w, dsc, doi);
                em = emitted(S, doi, dsc.flipped);
            } else if (S.env_map) {
                em = env_radiance(S, delta_wi, true);
            }
            L = L + delta_atten * em;
        }
    }
    radiance[(size_t)chunk_first * p.spp + i] = make_float4(L.r, L.g, L.b, 0.f);
}

} // namespace

int render_direct(yar_gpu_ctx* ctx, float* rgb_out, yar_render_stats* stats) {
    Render_Params p;
    if (int rc0 = prepare_render_params(ctx, p)) return rc0;
    cudaSetDevice(ctx->device);
    const Render_Scene& R = ctx->render;
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t pixels = (uint64_t)p.sw * p.sh;
    const uint64_t samples = pixels * p.spp;
    const uint64_t chunk_pixels = std::max<uint64_t>(1, std::min<uint64_t>(pixels, kChunkSampleBudget / p.spp));
    const uint64_t cap = chunk_pixels * p.spp;
    // k x k arrays per rectangular, then sphere light (reference_renderer.cpp:101-128)
    std::vector<int> sides;
    for (const yar_rect_light_desc& l : R.host_rect_lights) sides.push_back((int)std::ceil(std::sqrt((double)l.sample_count)));
    for (const yar_sphere_light_desc& l : R.host_sphere_lights)
        sides.push_back((int)std::ceil(std::sqrt((double)l.sample_count)));
    if (sides.empty()) sides.push_back(1);
    const int env_samples = R.has_environment ? R.environment.sample_count : 0;
    if (R.has_environment && env_samples < 1) return fail(ctx, YAR_ERR_UNSUPPORTED, "environment light without samples");
    // the pixel stream after the sample tables: image, 2D array grids, 1D array grids
    const uint64_t base = 2ull * p.spp + (uint64_t)p.n2d * (3 * p.spp - 1) + (uint64_t)p.n1d * (2 * p.spp - 1);
    if (base > 0xffffffffull) return fail(ctx, YAR_ERR_UNSUPPORTED, "too many sample arrays");

    std::vector<Device_Buffer>& B = ctx->render_scratch;
    for (Device_Buffer& b : B) device_free(b);
    B.assign(20, Device_Buffer{});
    int rc = YAR_OK;
    auto alloc = [&](int i, size_t bytes) {
        if (rc == YAR_OK) rc = device_alloc(ctx, B[i], bytes);
    };
    alloc(0, samples * sizeof(float4));                   // radiance
    alloc(1, samples * sizeof(float2));                   // image-plane samples
    alloc(2, cap * std::max(1, p.n1d) * sizeof(float));   // s1d: 1D array grids
    alloc(3, cap * std::max(1, p.n2d) * sizeof(float2));  // s2d: 2D array grids
    alloc(4, cap * sizeof(float4));                       // coeff (camera kernel)
    alloc(5, cap * sizeof(float4));                       // L (camera kernel)
    alloc(6, cap * sizeof(uint32_t));                     // info (camera kernel)
    alloc(7, cap * sizeof(uint4));                        // rng (camera kernel)
    alloc(8, cap * 2 * sizeof(float4));                   // camera rays
    alloc(9, cap * sizeof(uint32_t));                     // camera ray slots
    alloc(10, cap * 2 * sizeof(float4));                  // per-thread ray records
    alloc(11, cap * sizeof(float4));                      // hit4
    alloc(12, cap * sizeof(uint2));                       // hit2
    alloc(13, cap * sizeof(uint32_t));                    // draws / draw offsets
    alloc(14, pixels * sizeof(double));                   // pixel variance
    alloc(15, (size_t)p.tiles_x * p.tiles_y * sizeof(double));
    alloc(16, (size_t)p.rw * p.rh * 3 * sizeof(float));   // rgb
    alloc(17, 6 * sizeof(int));                           // traversal error, ray counters (2 x u64)
    alloc(18, sides.size() * sizeof(int));                // array sides
    if (rc != YAR_OK) return rc;
    Path_State ps{};
    ps.coeff = dptr<float4>(B[4]);
    ps.L = dptr<float4>(B[5]);
    ps.info = dptr<uint32_t>(B[6]);
    ps.rng = dptr<uint4>(B[7]);
    Queues q{};
    q.ext_rays[0] = dptr<float4>(B[8]);
    q.ext_slot[0] = dptr<uint32_t>(B[9]);
    Scene_Dev S = scene_dev(ctx->ds, ctx->render);
    cudaStream_t st = ctx->stream;
    int* err = dptr<int>(B[17]);
    cudaError_t e = cudaMemsetAsync(err, 0, 6 * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B[18].ptr, sides.data(), sides.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    uint32_t launches = 0;
    for (uint64_t first = 0; first < pixels && e == cudaSuccess; first += chunk_pixels) {
        const uint32_t cp = (uint32_t)std::min<uint64_t>(chunk_pixels, pixels - first);
        const uint32_t paths = cp * (uint32_t)p.spp;
        e = launch_generate(p, (uint32_t)first, cp, dptr<float>(B[2]), dptr<float>(B[3]), dptr<float2>(B[1]), ps, q,
                            st);
        if (e != cudaSuccess) break;
        direct_camera_kernel<<<(paths + kBlock - 1) / kBlock, kBlock, 0, st>>>(
            p, S, paths, q, dptr<float4>(B[10]), dptr<float4>(B[11]), dptr<uint2>(B[12]), dptr<uint32_t>(B[13]),
            env_samples, err);
        direct_prefix_kernel<<<(cp + kBlock - 1) / kBlock, kBlock, 0, st>>>(cp, p.spp, dptr<uint32_t>(B[13]));
        (p.textured ? direct_shade_kernel<true> : direct_shade_kernel<false>)<<<(paths + kBlock - 1) / kBlock,
                                                                              kBlock, 0, st>>>(
            p, S, (uint32_t)first, paths, q, dptr<float4>(B[10]), dptr<float4>(B[11]), dptr<uint2>(B[12]),
            dptr<uint32_t>(B[13]), (uint32_t)base, dptr<float>(B[2]), dptr<float2>(B[3]), dptr<int>(B[18]),
            env_samples, dptr<float2>(B[1]), dptr<float4>(B[0]), err);
        launches += 5;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        samples_kernel<<<(uint32_t)((pixels + kBlock - 1) / kBlock), kBlock, 0, st>>>(p, dptr<float4>(B[0]),
                                                                                      dptr<double>(B[14]));
        tile_variance_kernel<<<p.tiles_x * p.tiles_y, kTileVarThreads, 0, st>>>(p, dptr<double>(B[14]),
                                                                                dptr<double>(B[15]));
        film_kernel<<<(uint32_t)(((uint64_t)p.rw * p.rh + kBlock - 1) / kBlock), kBlock, 0, st>>>(
            p, dptr<float4>(B[0]), dptr<float2>(B[1]), dptr<float>(B[16]));
        launches += 3;
        e = cudaGetLastError();
    }
    std::vector<double> tile_var((size_t)p.tiles_x * p.tiles_y);
    int host_err[6] = {0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgb_out, B[16].ptr, (size_t)p.rw * p.rh * 3 * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tile_var.data(), B[15].ptr, tile_var.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_err, err, sizeof(host_err), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "direct-lighting render");
    if (host_err[0]) return fail(ctx, YAR_ERR_CAPACITY, "kd-tree traversal stack overflow");
    unsigned long long rays[2];
    memcpy(rays, host_err + 2, sizeof(rays));
    if (stats) {
        double acc = 0.0;
        int64_t count = 0;
        for (int t = 0; t < p.tiles_x * p.tiles_y; t++) {
            acc += tile_var[t];
            const int tx = t % p.tiles_x, ty = t / p.tiles_x;
            count += (int64_t)std::min(kTile, p.sw - tx * kTile) * std::min(kTile, p.sh - ty * kTile);
        }
        stats->variance = p.spp > 1 ? acc / (double)count : 0.0;
        stats->seconds = (float)std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        stats->paths = samples;
        stats->rays_closest = rays[0];
        stats->rays_any = rays[1];
        stats->kernel_launches = launches;
    }
    return YAR_OK;
}

} // namespace yar
