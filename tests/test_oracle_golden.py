"""The oracle (C restatement) against the reference's own outputs: the
golden fixtures are the reference renderer's results on the same inputs, and
the live reference (oracle/_ref) when it is built here."""
import numpy as np
import pytest

import oracle
from conftest import constant_bumps_with_delta_materials, golden
from yar_gb300 import scenes
from yar_gb300.scene import FlatScene, Mesh, make_object


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", ["raycast_small", "transform_small"])
def test_oracle_closest_matches_reference(name):
    s = FlatScene.read(golden(name + ".yfs"))
    g = np.load(golden(name + ".npz"))
    t, prim, obj, bary = oracle.cast_closest(s, g["rays"])
    assert np.array_equal(prim, g["prim"])
    assert np.array_equal(obj, g["obj"])
    assert np.array_equal(bits(t), bits(g["t"]))
    assert np.array_equal(bits(bary), bits(g["bary"]))
    assert (prim != 0xFFFFFFFF).mean() > 0.1


@pytest.mark.parametrize("name", ["raycast_small", "transform_small"])
def test_oracle_any_matches_reference(name):
    s = FlatScene.read(golden(name + ".yfs"))
    g = np.load(golden(name + ".npz"))
    occ = oracle.cast_any(s, g["shadow_rays"])
    assert np.array_equal(occ, g["occluded"])
    assert 0.05 < occ.mean() < 0.95


def regression_scene(g, k):
    s = FlatScene()
    s.meshes = [Mesh(g["mesh%d_vertices" % k], g["mesh%d_indices" % k], bounds=g["mesh%d_bounds" % k],
                     nodes=g["mesh%d_nodes" % k])]
    s.objects = np.array([make_object(0)])
    s.build_scene_kdtree()
    rays = np.zeros((g["mesh%d_rays" % k].shape[0], 8), np.float32)
    rays[:, 0:3] = g["mesh%d_rays" % k][:, 0:3]
    rays[:, 4:7] = g["mesh%d_rays" % k][:, 3:6]
    rays[:, 3] = np.inf
    return s, rays


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_kdtree_regression_meshes(k):
    """src/ref/test_kdtree.cpp: kd-tree t equals the brute-force t on the
    reference's FP-regression meshes and ray stream."""
    g = np.load(golden("kdtree_regression.npz"))
    s, rays = regression_scene(g, k)
    t, prim, obj, bary = oracle.cast_closest(s, rays)
    assert np.array_equal(bits(t), bits(g["mesh%d_t" % k]))
    assert np.array_equal(prim, g["mesh%d_prim" % k])


def test_watertight_known_answers():
    """The watertight intersector on the known-answer layout of the reference's
    SIMD test (src/ref/test_triangle_intersection.cpp:132-283): a ray from
    (0,0,5) along -z hits a triangle in the z=0 plane at t=5, misses one offset
    beyond its edge, and reports barycentrics that sum to 1."""
    import ctypes
    L = oracle.lib()
    o = (ctypes.c_float * 3)(0, 0, 5)
    d = (ctypes.c_float * 3)(0, 0, -1)
    b = (ctypes.c_float * 3)()
    hit = [(ctypes.c_float * 3)(*p) for p in ([-1, -1, 0], [1, -1, 0], [0, 1, 0])]
    t = L.oracle_intersect_triangle_watertight(o, d, hit[0], hit[1], hit[2], b)
    assert t == 5.0 and abs(sum(b) - 1) < 1e-6
    for dz in (1.0, 2.0, 3.0):
        shifted = [(ctypes.c_float * 3)(p[0], p[1], p[2] + dz) for p in hit]
        assert L.oracle_intersect_triangle_watertight(o, d, *shifted, b) == 5.0 - dz
    miss = [(ctypes.c_float * 3)(p[0] + 3, p[1], p[2]) for p in hit]
    assert L.oracle_intersect_triangle_watertight(o, d, *miss, b) == float("inf")
    # a shared edge is hit by exactly one of two triangles or both (never neither)
    e = [(ctypes.c_float * 3)(*p) for p in ([0, -1, 0], [0, 1, 0], [-1, 0, 0], [1, 0, 0])]
    t1 = L.oracle_intersect_triangle_watertight(o, d, e[0], e[1], e[2], b)
    t2 = L.oracle_intersect_triangle_watertight(o, d, e[1], e[0], e[3], b)
    assert min(t1, t2) == 5.0


def test_pcg32_matches_reference_stream():
    """pcg32_srandom_r(0, stream) then get_uint / get_float (src/lib/random.h)."""
    import ctypes
    L = oracle.lib()
    rng = (ctypes.c_uint64 * 2)()
    L.oracle_pcg32_seed(rng, 42, 54)
    # the pcg-basic demo stream for initstate 42, initseq 54
    expected = [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]
    assert [L.oracle_pcg32_next(rng) for _ in range(6)] == expected
    L.oracle_pcg32_seed(rng, 0, 7)
    f = [L.oracle_pcg32_float(rng) for _ in range(1000)]
    assert min(f) >= 0.0 and max(f) < 1.0


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
def test_oracle_against_live_reference_larger_batch():
    s = scenes.raycast_scene(seed=9, grid=96, spheres=12, level=3, build=True, threads=4)
    lo, hi = scenes.scene_box(s)
    rays = scenes.random_rays(lo, hi, 50000, 3)
    (rt, rp, ro, rb), _ = oracle.ref_cast(s, rays)
    t, prim, obj, bary = oracle.cast_closest(s, rays)
    assert np.array_equal(prim, rp) and np.array_equal(obj, ro) and np.array_equal(bits(t), bits(rt))
    sr = scenes.random_shadow_rays(lo, hi, 50000, 4)
    ra, _ = oracle.ref_cast(s, sr, any_hit=True)
    assert np.array_equal(oracle.cast_any(s, sr), ra)


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
def test_builder_against_live_reference_large_mesh():
    from yar_gb300 import native
    s = scenes.raycast_scene(seed=2, grid=160, spheres=2, level=3, build=False)
    ref, _ = oracle.ref_build(s)
    for m, r in zip(s.meshes, ref.meshes):
        b, nodes = native.build_mesh_kdtree(m.vertices, m.indices, 8)
        assert np.array_equal(nodes, r.nodes)


@pytest.mark.parametrize("name", ["cornell_c1_64", "cornell_ggx_64", "cornell_delta_64", "cornell_refractor_64",
                                  "cornell_layered_64", "cornell_layered_yar_64", "cornell_lights_64",
                                  "cornell_meshlight_64", "cornell_spherelight_64", "cornell_translucent_64", "cornell_transmission_64", "cornell_uber_64",
                                  "cornell_mix_64", "cornell_envconst_64", "cornell_envmap_64", "cornell_direct_64", "cornell_direct_env_64",
                                  "cornell_texture_64", "cornell_gaussian_64", "cornell_triangle_64",
                                  "cornell_alpha_64", "cornell_bump_64", "cornell_fourier_64",
                                  "cornell_spectex_64", "cornell_direct_tex_64"])
def test_oracle_render_matches_reference_golden(name):
    """The oracle's path loop, sampler, shading, BSDFs (diffuse, GGX metal, rough
    glass, plastic in both of the reference's forms, coated diffuse), delta
    scattering (mirror, smooth glass, perfect refractor), MIS and film
    reproduce the reference's FP32 render and variance bit for bit."""
    s = FlatScene.read(golden(name + ".yfs"))
    g = np.load(golden(name + ".npz"))
    img, var = oracle.render(s, threads=4)
    assert np.array_equal(bits(img), bits(g["image"]))
    assert var == float(g["variance"])


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
def test_oracle_render_against_live_reference_past_the_sampler_budget(tmp_path):
    """maxdepth 12 exceeds the sampler's 10-bounce dimension budget, so later
    draws come from the pixel's raw pcg stream in path order; the oracle keeps
    that order exactly (src/ref/pixel_sampling.cpp:159-173)."""
    p = tmp_path / "c.pbrt"
    p.write_text(scenes.cornell_pbrt(seed=4, width=32, height=32, spp=4, maxdepth=12, box_materials=scenes.GGX_BOXES))
    y = tmp_path / "c.yfs"
    oracle.ref_flatten(str(p), str(y), seed_offset=3)
    ref_img, info = oracle.ref_render(str(p), seed_offset=3, threads=4)
    img, var = oracle.render(FlatScene.read(str(y)), threads=4)
    assert np.array_equal(bits(img), bits(ref_img))
    assert var == info["variance"]


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
@pytest.mark.parametrize("maxb,rr", [(1, 3), (2, 1), (12, 1)])
def test_oracle_delta_paths_against_live_reference(maxb, rr):
    """Delta vertices at the last bounce (the delta ray still adds the light it
    reaches), Russian roulette right after a delta bounce, and paths past the
    sampler's dimension budget, on the perfect-refractor scene."""
    s = scenes.make_ceiling_refractor(FlatScene.read(golden("cornell_delta_64.yfs")))
    s.config["x_pixel_sample_count"] = s.config["y_pixel_sample_count"] = 2
    s.config["max_light_bounces"] = maxb
    s.config["russian_roulette_bounce_count_threshold"] = rr
    ref_img, info = oracle.ref_render_flat(s, threads=8)
    img, var = oracle.render(s, threads=8)
    assert np.array_equal(bits(img), bits(ref_img))
    assert var == info["variance"]


def test_oracle_correctly_rounded_trig_changes_only_the_trig():
    """The oracle's correctly-rounded-trig switch (the CUDA path's sines and
    cosines) moves only a few percent of the pixels, and switching back
    restores the reference's image bit for bit."""
    s = FlatScene.read(golden("cornell_ggx_64.yfs"))
    g = np.load(golden("cornell_ggx_64.npz"))
    img_cr, _ = oracle.render(s, threads=4, correctly_rounded_trig=True)
    same = np.all(bits(img_cr) == bits(g["image"]), axis=2).mean()
    assert 0.9 <= same < 1.0
    img, var = oracle.render(s, threads=4)
    assert np.array_equal(bits(img), bits(g["image"]))
    assert var == float(g["variance"])


def test_texture_scene_file_round_trip(tmp_path):
    """The TEXS chunk (texture records, mip records, texels) and the material
    records' texture fields survive a write and a read."""
    s = FlatScene.read(golden("cornell_texture_64.yfs"))
    assert s.textures.shape[0] == 1 and s.texture_mips.shape[0] == 7
    assert int(s.texture_mips["width"][0]) == 64 and int(s.texture_mips["texel_offset"][-1]) == 5460
    p = tmp_path / "t.yfs"
    s.write(str(p))
    t = FlatScene.read(str(p))
    assert np.array_equal(t.textures, s.textures) and np.array_equal(t.texture_mips, s.texture_mips)
    assert np.array_equal(t.texels, s.texels) and np.array_equal(t.materials, s.materials)
    assert sorted(int(x) for x in s.materials["reflectance_texture"]) == [0, 0, 0, 0, 1, 1]


def test_alpha_texture_file_round_trip(tmp_path):
    """A mesh's alpha texture (MESH chunk flag 4) survives a write and a read,
    in the Python and the C++ readers (the reference harness reads the file
    to render it)."""
    s = FlatScene.read(golden("cornell_alpha_64.yfs"))
    assert [m.alpha_texture for m in s.meshes].count(1) == 1
    p = tmp_path / "a.yfs"
    s.write(str(p))
    t = FlatScene.read(str(p))
    assert [m.alpha_texture for m in t.meshes] == [m.alpha_texture for m in s.meshes]
    assert np.array_equal(t.materials, s.materials) and np.array_equal(t.texels, s.texels)
    q = tmp_path / "b.yfs"
    t.write(str(q))
    assert open(str(p), "rb").read() == open(str(q), "rb").read()


def test_textured_scenes_outside_the_restated_part_are_refused():
    """Image textures are restated for the reflectance and transmittance slots
    and bump maps, with camera-ray and specular differentials; on other
    parameters, in a slot the material does not read, or as the bump map of a
    mix's sub-material the oracle refuses the scene."""
    for change in ("other", "slot", "mix_bump"):
        s = FlatScene.read(golden("cornell_texture_64.yfs"))
        if change == "other":
            s.materials["other_textured_parameters"][-1] = 1
        elif change == "slot":
            k = int(np.nonzero(s.materials["reflectance_texture"])[0][0])
            s.materials["transmittance_texture"][k] = s.materials["reflectance_texture"][k]  # diffuse: no such slot
        else:
            s = FlatScene.read(golden("cornell_mix_64.yfs"))
            mix = int(np.nonzero(s.materials["type"] == 8)[0][0])
            s.materials["bump"][int(s.materials["mix_materials"][mix][0])] = 1
        with pytest.raises(Exception):
            oracle.render(s, threads=2)


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
def test_oracle_constant_bump_on_delta_materials_against_live_reference():
    """A constant bump height on a mirror and on smooth glass (the bump comes
    before the delta check, src/ref/delta_scattering.cpp:252-257) and on a floor
    with splayed vertex normals: the oracle against the reference's render of
    the same flat scene, bit for bit."""
    s = constant_bumps_with_delta_materials()
    s.config["max_light_bounces"] = 5
    ref, info = oracle.ref_render_flat(s, threads=8)
    img, var = oracle.render(s, threads=8)
    assert np.array_equal(bits(img), bits(ref))
    assert var == info["variance"]


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not built here")
def test_oracle_specular_differentials_against_live_reference(tmp_path):
    """Textures behind chains of delta bounces, past the reference's 4
    specular bounces with differential rays and past the sampler's dimension
    budget (maxdepth 12, another seed): the oracle against the reference's
    render of the same flat scene, bit for bit."""
    from yar_gb300 import exr
    exr.write_exr(str(tmp_path / "checks.exr"), scenes.texture_image(), False, {})
    pbrt = tmp_path / "spectex.pbrt"
    pbrt.write_text(scenes.specular_texture_pbrt("checks.exr", seed=29, width=32, height=32, spp=4, maxdepth=12))
    yfs = tmp_path / "spectex.yfs"
    oracle.ref_flatten(str(pbrt), str(yfs), seed_offset=3)
    s = scenes.texture_glass_panel(FlatScene.read(str(yfs)))
    ref, info = oracle.ref_render_flat(s, threads=8, textures_from=str(pbrt))
    img, var = oracle.render(s, threads=8)
    assert np.array_equal(bits(img), bits(ref))
    assert var == info["variance"]


def test_oracle_c1_configuration_matches_reference_golden():
    """The C1 configuration (256 x 256 from the flattened Cornell box) against
    the reference's render of its pbrt scene, bit for bit."""
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    s.config["render_region"] = (0, 0, 256, 256)
    s.camera["image_extent"] = (256, 256)
    g = np.load(golden("cornell_c1_256.npz"))
    img, var = oracle.render(s, threads=8)
    assert np.array_equal(bits(img), bits(g["image"]))
    assert var == float(g["variance"])
