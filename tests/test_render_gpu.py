"""GPU parity of the render path (yar_gpu_render <- render_scene) against the
reference's own FP32 renders (golden fixtures) and the oracle.

The sampler, camera, traversal, shading, BSDF and film arithmetic follow the
reference operation by operation.  sin/cos are the one place where the
device and the host C library round differently: the device returns the
correctly rounded float, glibc's sinf/cosf differ from it by one unit in the
last place for about 1.3% of the arguments the samplers produce.  So the bar
is: at least 90% of pixels bit-identical to the reference render, a mean
relative error of the whole image below 1e-4, and the luminance variance
within 1e-5 relative.  Measured on GB300: 96.5% / 5.6e-10 on the diffuse
Cornell box, 96.0% / 1.2e-5 with the GGX metal and rough-glass boxes (a
one-ulp direction change can turn a glossy path toward or away from the
light, so a few pixels carry Monte Carlo-sized differences)."""
import numpy as np
import pytest

import oracle
from conftest import constant_bumps_with_delta_materials, golden
from yar_gb300 import scenes
from yar_gb300.scene import FlatScene

pytestmark = pytest.mark.gpu

MEAN_REL_TOL = 1e-4
BIT_EQUAL_MIN = 0.90
VARIANCE_REL_TOL = 1e-5
# Scenes with point, spot and directional lights: the few samples whose paths
# diverge from the reference's (sin/cos rounding) can pick up a point light's
# 1/d^2 peak near a wall.  The share of bit-identical pixels is unchanged
# (97-98% measured), but those samples move the mean relative error and the
# image variance by up to ~2e-4 and ~1e-4.
LIGHTS_MEAN_REL_TOL = 3e-4
LIGHTS_VARIANCE_REL_TOL = 1e-4
# Environment maps: every lookup takes an atan2 and an acos, and glibc's
# atan2f/acosf round differently from the correctly rounded value more often
# than sinf/cosf do (89.3% bit-identical pixels on cornell_envmap_64; an oracle
# run with correctly rounded trigonometry gives the same figure).
ENV_BIT_EQUAL_MIN = 0.85
# pbrt3 fourier materials evaluate up to 8 cosines and an acos per BSDF
# evaluation: 88.2% bit-identical pixels on cornell_fourier_64 (mean relative
# error 1.3e-9); an oracle run with correctly rounded trigonometry gives the
# same figure.
FOURIER_BIT_EQUAL_MIN = 0.85
# Wide pixel filters (gaussian of radius 1.5, triangle of radius 2): a sample
# whose path diverges through sin/cos rounding reaches up to 16 pixels with
# its weight, so the mean relative error of the same divergences is larger
# (1.1e-4 measured on cornell_gaussian_64 at 91.5% bit-identical pixels).
FILTER_MEAN_REL_TOL = 3e-4


def sample_region_pixels(s):
    """Pixels of the film's sample region (Film::Film, src/ref/film.cpp:53-86)."""
    import math
    r = float(s.config["pixel_filter_radius"])
    x0, y0, x1, y1 = (int(v) for v in s.config["render_region"])
    w = math.ceil(x1 - 1 + 0.5 + r) - math.floor(x0 + 0.5 - r)
    h = math.ceil(y1 - 1 + 0.5 + r) - math.floor(y0 + 0.5 - r)
    return w * h


def compare(img, ref):
    same = np.all(img.view(np.uint32) == ref.view(np.uint32), axis=2).mean()
    rel = float(np.abs(img.astype(np.float64) - ref).sum() / max(ref.astype(np.float64).sum(), 1e-30))
    return same, rel


@pytest.mark.parametrize("name", ["cornell_c1_64", "cornell_ggx_64", "cornell_delta_64", "cornell_refractor_64",
                                  "cornell_layered_64", "cornell_layered_yar_64", "cornell_lights_64",
                                  "cornell_meshlight_64", "cornell_spherelight_64", "cornell_translucent_64", "cornell_transmission_64", "cornell_uber_64", "cornell_mix_64", "cornell_envconst_64",
                  "cornell_envmap_64", "cornell_direct_64", "cornell_direct_env_64",
                                  "cornell_texture_64", "cornell_gaussian_64", "cornell_triangle_64",
                                  "cornell_alpha_64", "cornell_bump_64", "cornell_fourier_64",
                                  "cornell_spectex_64", "cornell_direct_tex_64"])
def test_render_matches_reference_golden(gpu_ctx, name):
    s = FlatScene.read(golden(name + ".yfs"))
    g = np.load(golden(name + ".npz"))
    gpu_ctx.upload_scene(s)
    w = int(s.config["render_region"][2] - s.config["render_region"][0])
    h = int(s.config["render_region"][3] - s.config["render_region"][1])
    img, stats = gpu_ctx.render(w, h)
    same, rel = compare(img, g["image"])
    lights = s.delta_lights.shape[0] > 0 or s.environment is not None
    wide = int(s.config["pixel_filter_type"]) != 0 or float(s.config["pixel_filter_radius"]) > 0.5
    trig_heavy = s.environment is not None
    bar = ENV_BIT_EQUAL_MIN if trig_heavy else FOURIER_BIT_EQUAL_MIN if s.fourier_tables.shape[0] else BIT_EQUAL_MIN
    assert same >= bar, (same, rel)
    assert rel < (LIGHTS_MEAN_REL_TOL if lights else FILTER_MEAN_REL_TOL if wide else MEAN_REL_TOL), (same, rel)
    vtol = LIGHTS_VARIANCE_REL_TOL if lights else VARIANCE_REL_TOL
    assert abs(stats.variance - float(g["variance"])) <= vtol * float(g["variance"])
    assert stats.paths == sample_region_pixels(s) * 16
    assert stats.rays_closest >= stats.paths


RENDER_GOLDENS = ["cornell_c1_64", "cornell_ggx_64", "cornell_delta_64", "cornell_refractor_64", "cornell_layered_64",
                  "cornell_layered_yar_64", "cornell_lights_64", "cornell_meshlight_64", "cornell_spherelight_64",
                  "cornell_translucent_64", "cornell_transmission_64", "cornell_uber_64", "cornell_mix_64", "cornell_envconst_64",
                  "cornell_envmap_64", "cornell_direct_64", "cornell_direct_env_64", "cornell_texture_64",
                  "cornell_gaussian_64", "cornell_triangle_64", "cornell_alpha_64", "cornell_bump_64",
                  "cornell_fourier_64", "cornell_spectex_64", "cornell_direct_tex_64"]


@pytest.mark.parametrize("name", RENDER_GOLDENS)
@pytest.mark.parametrize("seed_offset,maxb", [(1, 8), (5, 3)])
def test_render_bit_identical_to_oracle_with_correctly_rounded_trig(gpu_ctx, name, seed_offset, maxb):
    """The only arithmetic the CUDA path does not share with the reference is
    the sine and cosine of sampled angles: the device rounds them correctly,
    the reference takes the C library's sinf/cosf.  With the oracle switched to
    correctly rounded values, every pixel and the variance are bit-identical."""
    s = FlatScene.read(golden(name + ".yfs"))
    s.config["rng_seed_offset"] = seed_offset
    s.config["max_light_bounces"] = maxb
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


@pytest.mark.parametrize("seed_offset,spp_xy,maxb", [(7, (2, 3), 5), (0, (1, 1), 1), (3, (4, 4), 12)])
def test_render_matches_oracle_other_configs(gpu_ctx, seed_offset, spp_xy, maxb):
    """Seeds, non-square sample grids, a single bounce, and maxdepth 12, which
    exceeds the sampler's 10-bounce dimension budget: the draws past it come
    from the pixel's pcg stream in sample order, as in the reference.
    Bit-identical to the oracle with correctly rounded sine and cosine."""
    s = FlatScene.read(golden("cornell_ggx_64.yfs"))
    s.config["rng_seed_offset"] = seed_offset
    s.config["x_pixel_sample_count"], s.config["y_pixel_sample_count"] = spp_xy
    s.config["max_light_bounces"] = maxb
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


@pytest.mark.parametrize("name,nx,ny,size", [("cornell_ggx_64", 11, 10, 64), ("cornell_delta_64", 26, 20, 16),
                                              ("cornell_direct_64", 13, 8, 32)])
def test_many_samples_per_pixel_bit_identical_to_oracle(gpu_ctx, name, nx, ny, size):
    """Above 96 samples per pixel the sample-table kernel runs smaller blocks
    (each thread shuffles its row's spp values in shared memory), and 26 x 20
    strata are not square: images and variance bit-identical to the oracle
    with correctly rounded trigonometry, in both rendering algorithms."""
    s = FlatScene.read(golden(name + ".yfs"))
    s.config["x_pixel_sample_count"], s.config["y_pixel_sample_count"] = nx, ny
    s.config["render_region"] = (0, 0, size, size)
    s.camera["image_extent"] = (size, size)
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(size, size)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var
    assert stats.paths == size * size * nx * ny


def _past_budget_scene(name):
    s = FlatScene.read(golden(name + ".yfs"))
    return scenes.make_ceiling_refractor(s) if name == "cornell_delta_64" else s


@pytest.mark.parametrize("name,maxb,rr,seed_offset", [
    ("cornell_c1_64", 16, 3, 1), ("cornell_ggx_64", 14, 1, 4), ("cornell_delta_64", 12, 1, 2),
    ("cornell_delta_64", 9, 1, 6), ("cornell_delta_64", 16, 1, 11), ("cornell_mix_64", 12, 2, 3), ("cornell_uber_64", 12, 1, 5),
    ("cornell_envmap_64", 13, 3, 8), ("cornell_meshlight_64", 12, 2, 9), ("cornell_spectex_64", 12, 1, 3)])
def test_render_past_the_dimension_budget_bit_identical(gpu_ctx, name, maxb, rr, seed_offset):
    """Paths that run past the sampler's dimension budget (deep paths, and
    delta chains whose Russian roulette takes extra dimensions, so even
    maxdepth 9 can) draw from the pixel's stream after the sample tables,
    sample after sample.  The device defers them and finishes them in waves
    of one sample per pixel: bit-identical to the oracle with correctly
    rounded trigonometry."""
    s = _past_budget_scene(name)
    s.config["max_light_bounces"] = maxb
    s.config["russian_roulette_bounce_count_threshold"] = rr
    s.config["rng_seed_offset"] = seed_offset
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


@pytest.mark.parametrize("name,maxb,past_budget", [("cornell_c1_64", 8, False), ("cornell_bump_64", 8, False),
                                                  ("cornell_delta_64", 16, True), ("cornell_envmap_64", 13, True)])
def test_device_driven_bounces_match_host_driven(gpu_ctx, name, maxb, past_budget):
    """The first render of a scene reads each bounce's queue lengths on the host
    (and tunes the traversal kernels); later renders drive the bounces, and the
    exact tail's waves, from the device.  Both give the same image, variance and
    ray counts, bit for bit."""
    s = _past_budget_scene(name) if past_budget else FlatScene.read(golden(name + ".yfs"))
    s.config["max_light_bounces"] = maxb
    gpu_ctx.upload_scene(s)
    img1, st1 = gpu_ctx.render(64, 64)
    img2, st2 = gpu_ctx.render(64, 64)
    assert np.array_equal(img1.view(np.uint32), img2.view(np.uint32))
    assert st1.variance == st2.variance
    assert (st1.rays_closest, st1.rays_any, st1.paths) == (st2.rays_closest, st2.rays_any, st2.paths)
    assert st1.kernel_launches != st2.kernel_launches  # the second render ran the other loop


@pytest.mark.parametrize("maxb,rr,seed_offset", [(1, 3, 0), (2, 1, 5), (3, 2, 9), (8, 1, 2)])
def test_render_delta_paths_match_oracle(gpu_ctx, maxb, rr, seed_offset):
    """Mirror, smooth glass and a perfect-refractor ceiling: delta vertices at
    the last bounce, Russian roulette right after a delta bounce, light reached
    only through the refractor."""
    s = scenes.make_ceiling_refractor(FlatScene.read(golden("cornell_delta_64.yfs")))
    s.config["max_light_bounces"] = maxb
    s.config["russian_roulette_bounce_count_threshold"] = rr
    s.config["rng_seed_offset"] = seed_offset
    ref, ref_var = oracle.render(s, threads=8)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    same, rel = compare(img, ref)
    assert same >= BIT_EQUAL_MIN, (same, rel)
    assert rel < MEAN_REL_TOL, (same, rel)
    assert abs(stats.variance - ref_var) <= VARIANCE_REL_TOL * ref_var


@pytest.mark.parametrize("pbrt3,seed_offset,maxb", [(1, 4, 3), (0, 8, 5)])
def test_render_layered_materials_match_oracle(gpu_ctx, pbrt3, seed_offset, maxb):
    """Plastic (pbrt-v3's and YAR's forms) and coated diffuse at other seeds
    and depths."""
    s = FlatScene.read(golden("cornell_layered_64.yfs"))
    s.config["pbrt3_scene"] = pbrt3
    s.config["rng_seed_offset"] = seed_offset
    s.config["max_light_bounces"] = maxb
    ref, ref_var = oracle.render(s, threads=8)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    same, rel = compare(img, ref)
    assert same >= BIT_EQUAL_MIN, (same, rel)
    assert rel < MEAN_REL_TOL, (same, rel)
    assert abs(stats.variance - ref_var) <= VARIANCE_REL_TOL * ref_var


@pytest.mark.parametrize("seed_offset,maxb", [(2, 1), (9, 4)])
def test_render_point_spot_directional_lights_match_oracle(gpu_ctx, seed_offset, maxb):
    """Point, spot and directional lights beside the quad light, at other seeds
    and depths (maxdepth 1: direct light only): bit-identical to the oracle
    with correctly rounded sines and cosines, and within the lights bars of
    the oracle as the reference computes it."""
    s = FlatScene.read(golden("cornell_lights_64.yfs"))
    s.config["rng_seed_offset"] = seed_offset
    s.config["max_light_bounces"] = maxb
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    exact, exact_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    assert np.array_equal(img.view(np.uint32), exact.view(np.uint32))
    assert stats.variance == exact_var
    ref, ref_var = oracle.render(s, threads=8)
    same, rel = compare(img, ref)
    assert same >= BIT_EQUAL_MIN, (same, rel)
    assert rel < LIGHTS_MEAN_REL_TOL, (same, rel)


def test_render_rejects_delta_lights_out_of_order(gpu_ctx):
    from yar_gb300 import native
    s = FlatScene.read(golden("cornell_lights_64.yfs"))
    s.delta_lights = s.delta_lights[::-1].copy()
    gpu_ctx.upload_scene(s)
    with pytest.raises(native.YarError) as e:
        gpu_ctx.render(64, 64)
    assert e.value.code == native.YAR_ERR_INVALID


@pytest.mark.parametrize("samples", [(4, 2), (1, 9)])
def test_render_direct_lighting_sphere_lights_bit_identical(gpu_ctx, samples):
    """The direct-lighting algorithm over sphere lights' k x k sample arrays
    (and the quad light's), against the oracle with correctly rounded
    trigonometry."""
    s = FlatScene.read(golden("cornell_spherelight_64.yfs"))
    s.config["rendering_algorithm"] = 0
    sl = s.sphere_lights.copy()
    sl["sample_count"] = samples
    s.sphere_lights = sl
    rl = s.rect_lights.copy()
    rl["sample_count"] = 2
    s.rect_lights = rl
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


def test_render_unsupported_features_fail_cleanly(gpu_ctx):
    from yar_gb300 import native
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    s.config["pixel_filter_type"] = 3  # no such filter
    gpu_ctx.upload_scene(s)
    with pytest.raises(native.YarError) as e:
        gpu_ctx.render(64, 64)
    assert e.value.code == native.YAR_ERR_UNSUPPORTED
    s.config["pixel_filter_type"] = 0
    gpu_ctx.upload_scene(s)
    img, _ = gpu_ctx.render(64, 64)
    assert img.mean() > 0


def test_render_identical_for_every_traversal_kernel():
    """The traversal kernel choice (fixed, or timed per scene on the first
    secondary bounce) changes no bit of the image or the variance."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from yar_gb300 import native
    s = FlatScene.read(golden("cornell_ggx_64.yfs"))
    s.config["x_pixel_sample_count"], s.config["y_pixel_sample_count"] = 8, 8  # 262144 paths: tuning runs
    results = []
    for kernel in (native.TRAVERSAL_AUTO, native.TRAVERSAL_PERSISTENT_64, native.TRAVERSAL_PERSISTENT_128,
                   native.TRAVERSAL_PER_RAY, native.TRAVERSAL_PER_RAY_VOTE):
        ctx = native.Context(0, traversal_kernel=kernel)
        try:
            ctx.upload_scene(s)
            for _ in range(2 if kernel == native.TRAVERSAL_AUTO else 1):
                img, stats = ctx.render(64, 64)
                results.append((img, stats.variance))
        finally:
            ctx.close()
    img0, var0 = results[0]
    for img, var in results[1:]:
        assert np.array_equal(img.view(np.uint32), img0.view(np.uint32))
        assert var == var0


def test_cli_render_writes_the_reference_exr(tmp_path):
    """python -m yar_gb300 render: the EXR holds the render's pixels as the
    reference's writer would store them, with yar_render_device = gpu."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import os
    from yar_gb300 import exr, native
    from yar_gb300.__main__ import main
    out = os.path.join(tmp_path, "c.exr")
    assert main(["render", golden("cornell_c1_64.yfs"), "--out", out]) == 0
    got, attrs = exr.read_exr(out)
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    ctx = native.Context(0)
    try:
        ctx.upload_scene(s)
        img, st = ctx.render(64, 64)
    finally:
        ctx.close()
    want = exr.to_half_bits(img).view(np.float16).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert attrs["yar_render_device"][1] == b"gpu"
    assert attrs["yar_spp"][1] == (16).to_bytes(4, "little")


@pytest.mark.parametrize("seed_offset,spp_xy", [(2, (4, 4)), (6, (3, 2))])
def test_textured_render_bit_identical_to_oracle(gpu_ctx, seed_offset, spp_xy):
    """Image-textured diffuse walls (EWA over the reference's mip chain, the
    camera ray's differentials scaled to the sample footprint, bilinear mip 0
    at later vertices, uv scale 2 x 3): bit-identical to the oracle with
    correctly rounded trigonometry, log2 and filter weights."""
    s = FlatScene.read(golden("cornell_texture_64.yfs"))
    s.config["rng_seed_offset"] = seed_offset
    s.config["x_pixel_sample_count"], s.config["y_pixel_sample_count"] = spp_xy
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


@pytest.mark.parametrize("seed_offset,spp_xy", [(3, (4, 4)), (7, (2, 3))])
def test_bump_mapped_render_bit_identical_to_oracle(gpu_ctx, seed_offset, spp_xy):
    """Bump maps (image and constant heights, uv scales, splayed vertex normals
    whose uv derivatives take part) on matte, plastic, translucent and rough
    glass, with textured reflectance and transmittance on glass and diffuse
    transmission: bit-identical to the oracle with correctly rounded
    trigonometry."""
    s = FlatScene.read(golden("cornell_bump_64.yfs"))
    s.config["rng_seed_offset"] = seed_offset
    s.config["x_pixel_sample_count"], s.config["y_pixel_sample_count"] = spp_xy
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


def test_constant_bump_with_delta_materials_bit_identical_to_oracle(gpu_ctx):
    """A constant bump height reads no ray differentials, so it may sit on
    delta materials: the mirror and the smooth glass reflect and refract about
    the bumped normal, bit-identical to the oracle."""
    s = constant_bumps_with_delta_materials()
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


@pytest.mark.parametrize("scale", [1.6, 0.5])
def test_probe_culling_follows_the_light_geometry(gpu_ctx, scale):
    """MIS probes that cannot reach the sampled quad light are not traced, but
    only for lights whose own triangles lie on their rectangle.  The light's
    quad scaled about its centre: grown (the check fails, every probe is
    traced, and the geometry beyond the rectangle is hit) or shrunk (probes are
    culled against the rectangle, which still holds the triangles): both
    bit-identical to the oracle, which traces every probe."""
    from yar_gb300 import native
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    k = int(np.nonzero(s.objects["area_light_type"] == native.LIGHT_RECT)[0][0])
    mesh = s.meshes[int(s.objects["mesh_index"][k])]
    v = mesh.vertices.reshape(-1, 3)
    c = v.mean(axis=0)
    mesh.vertices = (c + (v - c) * np.float32(scale)).astype(np.float32).reshape(mesh.vertices.shape)
    s.build_kdtrees()
    s.config["rng_seed_offset"] = 7
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


def test_fourier_direct_lighting_bit_identical_to_oracle(gpu_ctx):
    """The fourier boxes under the direct-lighting algorithm: the light
    samples evaluate the series, bit-identical to the oracle."""
    s = FlatScene.read(golden("cornell_fourier_64.yfs"))
    s.config["rendering_algorithm"] = 0
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(64, 64)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert stats.variance == ref_var


def test_fourier_tables_checked_on_upload(gpu_ctx):
    """A fourier table whose series reach past its coefficients, whose last
    zenith node is below 1 (the node search could end past the table) or
    whose channel count is neither 1 nor 3 is refused on upload; eta != 1
    (refraction, which the reference does not evaluate) is refused by the
    render."""
    from yar_gb300 import native
    for change in ("series", "nodes", "channels", "eta"):
        s = FlatScene.read(golden("cornell_fourier_64.yfs"))
        t = s.fourier_tables
        if change == "series":
            s.fourier_uints[int(t["series"][0]) + 1] = 10 ** 6
        elif change == "nodes":
            s.fourier_floats[int(t["nodes"][0]) + int(t["node_count"][0]) - 1] = 0.5
        elif change == "channels":
            t["channel_count"][1] = 2
        else:
            t["eta"][0] = 1.5
        with pytest.raises(native.YarError):
            gpu_ctx.upload_scene(s)
            gpu_ctx.render(64, 64)


def test_bump_maps_and_textures_refused_where_the_material_does_not_read_them(gpu_ctx):
    """A mix's sub-material may not have a bump map; a texture in a slot the
    material does not read is refused."""
    from yar_gb300 import native
    t = FlatScene.read(golden("cornell_texture_64.yfs"))
    k = int(np.nonzero(t.materials["reflectance_texture"])[0][0])
    t.materials["transmittance_texture"][k] = t.materials["reflectance_texture"][k]  # diffuse has no such slot
    gpu_ctx.upload_scene(t)
    with pytest.raises(native.YarError):
        gpu_ctx.render(64, 64)
    x = FlatScene.read(golden("cornell_mix_64.yfs"))
    mix = int(np.nonzero(x.materials["type"] == native.MATERIAL_MIX)[0][0])
    x.materials["bump"][int(x.materials["mix_materials"][mix][0])] = 1
    gpu_ctx.upload_scene(x)
    with pytest.raises(native.YarError):
        gpu_ctx.render(64, 64)


def test_direct_lighting_with_constant_bumps_on_delta_materials(gpu_ctx):
    """The direct-lighting algorithm with constant bump heights on a mirror,
    smooth glass and a floor with splayed normals: bit for bit the oracle's
    image with correctly rounded trigonometry."""
    s = constant_bumps_with_delta_materials()
    s.config["rendering_algorithm"] = 0
    gpu_ctx.upload_scene(s)
    img, st = gpu_ctx.render(64, 64)
    ref, ref_var = oracle.render(s, threads=8, correctly_rounded_trig=True)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert st.variance == ref_var


def test_specular_differentials_reach_textures_behind_delta_bounces(gpu_ctx):
    """Textures seen through the glass panel and in the mirror wall are looked
    up with the differential rays the delta bounces carry (up to the
    reference's 4 specular bounces): bit for bit the oracle's image, with the
    chains of delta bounces cut at several depths."""
    s = FlatScene.read(golden("cornell_spectex_64.yfs"))
    for maxb in (2, 5, 9):
        s.config["max_light_bounces"] = maxb
        gpu_ctx.upload_scene(s)
        img, _ = gpu_ctx.render(64, 64)
        ref, _ = oracle.render(s, threads=8, correctly_rounded_trig=True)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), maxb


def test_direct_lighting_scene_refused_by_path_tracer_only_entry_points(gpu_ctx, tmp_path):
    """The batched, guided and checkpointed renders run the path tracer only:
    a direct-lighting scene (rendering_algorithm 0) is refused by each instead
    of coming back path traced."""
    from yar_gb300 import native
    s = FlatScene.read(golden("cornell_direct_64.yfs"))
    assert int(s.config["rendering_algorithm"]) == 0
    with pytest.raises(native.YarError) as e:
        gpu_ctx.render_batch([s])
    assert e.value.code == native.YAR_ERR_UNSUPPORTED
    gpu_ctx.upload_scene(s)
    with pytest.raises(native.YarError) as e:
        gpu_ctx.guided_render(64, 64, passes=1)
    assert e.value.code == native.YAR_ERR_UNSUPPORTED
    with pytest.raises(native.YarError) as e:
        gpu_ctx.render_checkpoint(64, 64, tmp_path, "scene.pbrt")
    assert e.value.code == native.YAR_ERR_UNSUPPORTED


def test_render_c1_configuration_matches_the_reference(gpu_ctx):
    """The C1 configuration itself (256 x 256, 16 spp, maxdepth 8, seed offset
    1) against the reference's own render of it, under the render bars."""
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    s.config["render_region"] = (0, 0, 256, 256)
    s.camera["image_extent"] = (256, 256)
    g = np.load(golden("cornell_c1_256.npz"))
    gpu_ctx.upload_scene(s)
    img, stats = gpu_ctx.render(256, 256)
    same, rel = compare(img, g["image"])
    assert same >= BIT_EQUAL_MIN and rel < MEAN_REL_TOL, (same, rel)
    assert abs(stats.variance - float(g["variance"])) <= VARIANCE_REL_TOL * float(g["variance"])
    assert stats.paths == 256 * 256 * 16
