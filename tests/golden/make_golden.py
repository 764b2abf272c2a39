"""Generates the golden fixtures in tests/golden/ by running the reference
renderer itself (oracle/_ref/yar_ref, built from the reference sources by
oracle/build_ref.sh).  Run from the repository root:

    python tests/golden/make_golden.py

Fixtures
  raycast_small.yfs / .npz   small terrain + icosphere scene, kd-trees built by
                             the reference builder; 4096 closest-hit rays with
                             the reference's (t, prim, object, bary) and 4096
                             shadow rays with its occlusion bits.
  transform_small.yfs / .npz objects under rotation + non-uniform scale +
                             translation (two-level transform path), same rays.
  kdtree_regression.npz      the two hand-built meshes of the reference's
                             kd-tree FP-regression test (src/ref/test_kdtree.cpp
                             :196-246, parsed from that file), their reference
                             kd-trees, and 4096 rays of the test's own ray
                             stream (:20-83) with the reference's t and triangle.
  cornell_c1_64.yfs / .npz   the Cornell box flattened by the reference loader
                             and builder at 64x64, 16 spp, maxdepth 8, seed 1,
                             and the reference's FP32 render of it.
  cornell_ggx_64.yfs / .npz  the same with a GGX metal box and a rough-glass box.
  cornell_delta_64.yfs / .npz the same with a mirror box and a smooth-glass box
                             (delta scattering) and a second light above the
                             ceiling, seed 5.
  cornell_refractor_64.yfs / .npz  cornell_delta_64 with the ceiling turned
                             into a perfect refractor (IOR 1/1.5 on its
                             upward-facing normal: no total internal
                             reflection from the room) that lets the upper
                             light in, rendered by the reference from the flat
                             scene (pbrt has no perfect refractor).
  cornell_layered_64.yfs / .npz  the same with a pbrt "plastic" box
                             (Pbrt3_Plastic_BRDF) and a pbrt "substrate" box
                             (Ashikhmin-Shirley coated diffuse), seed 6.
  cornell_layered_yar_64.yfs / .npz  cornell_layered_64 as a non-pbrt scene
                             (YAR's Plastic_BRDF, alpha = roughness^2),
                             rendered by the reference from the flat scene.
  cornell_lights_64.yfs / .npz  the GGX Cornell box lit also by a point, a
                             spot (with penumbra) and a distant light, seed 7.
  cornell_meshlight_64.yfs / .npz  the GGX Cornell box with two hexagonal
                             emitting meshes (triangle-mesh lights: one with
                             geometric normals on the ceiling, one with vertex
                             normals on the left wall) besides the quad light,
                             seed 8.
  cornell_spherelight_64.yfs / .npz  cornell_ggx_64 with two emitting spheres
                             (sphere lights shown by level-2 icospheres, added
                             on the flat scene), rendered by the reference from
                             the flat scene.
  cornell_translucent_64.yfs / .npz  a pbrt "translucent" tall box, seed 9.
  cornell_transmission_64.yfs / .npz  cornell_translucent_64 with the short box
                             turned into YAR's diffuse-transmission material,
                             rendered by the reference from the flat scene.
  cornell_uber_64.yfs / .npz  pbrt "uber" boxes: one with a delta-reflection
                             layer, one with opacity (passthrough), seed 10.
  cornell_mix_64.yfs / .npz  pbrt "mix" boxes: matte with metal (Mix_BSDF) and
                             mirror with plastic (a delta layer and a scaled
                             BSDF), seed 11.
  cornell_envconst_64.yfs / .npz  the GGX Cornell box lit also by a constant
                             pbrt "infinite" light through its open side, seed 12.
  cornell_envmap_64.yfs / .npz  the delta-box Cornell box with an "infinite"
                             light of a 64 x 32 sky map with a sun (written by
                             yar_gb300.exr), seed 13.
  cornell_texture_64.yfs / .npz  GGX boxes, the back wall, the left wall and
                             the floor lit with pbrt "imagemap" textures of a
                             48 x 40 checker image (uv scale 1 and 2 x 3;
                             EWA filtering with camera-ray differentials), seed 17.
  cornell_bump_64.yfs / .npz  bump maps and textures on every texture slot:
                             the back wall matte (checker Kd, image bump map),
                             the left wall plastic (checker Kd 2 x 3, bump
                             map 2 x 2), the floor matte with splayed vertex
                             normals and a constant bump height, the right
                             wall translucent (image bump map), a rough glass
                             panel with splayed normals (bump map 2 x 2;
                             checker Kr and Kt set on the flattened scene),
                             the ceiling made diffuse transmission with
                             checker reflectance and transmittance, GGX boxes;
                             rendered by the reference from the edited flat
                             scene, seed 21.
  cornell_spectex_64.yfs / .npz  textures seen through delta bounces: the
                             floor, back and left walls checker-textured, the
                             right wall a mirror with uvs and splayed vertex
                             normals, a smooth glass panel with uvs and
                             splayed normals in front of the room (checker Kr
                             2 x 3 and Kt set on the flattened scene), a
                             mirror box and a glass box without uvs; the
                             texture lookups behind the panel and in the
                             mirror use the specular differential rays;
                             rendered by the reference from the edited flat
                             scene, seed 23.
  cornell_direct_tex_64.yfs / .npz  the cornell_spectex_64 scene with an image
                             bump map on the back wall, rendered by the
                             direct-lighting algorithm (2 quad-light samples;
                             textures and the bump read the camera-ray
                             differentials), seed 31.
  cornell_fourier_64.yfs / .npz  pbrt "fourier" boxes: a one-channel and a
                             three-channel layerlab table written by
                             write_fourier_bsdf (15 zenith nodes, glossy lobes
                             of up to 8 azimuthal terms, series lengths that
                             vary per node pair), seed 23.
  cornell_direct_64.yfs / .npz  the reference's direct-lighting algorithm
                             (pbrt "directlighting"): GGX boxes, the quad light
                             with 4 samples (2 x 2 arrays), point, spot and
                             distant lights, seed 15.
  cornell_direct_env_64.yfs / .npz  direct lighting with delta boxes, the quad
                             light with 3 samples and a sky map with 2 samples,
                             seed 16.
  checkpoint_c1/             the reference's checkpoint directory (metadata and
                             four tile files) of a 72 x 72, 4 spp Cornell box
                             render (seed 14) with input file name
                             "cornell_checkpoint.pbrt"; checkpoint_c1.yfs / .npz
                             are that scene and the reference's image.
"""
import os
import re
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from yar_gb300 import scenes  # noqa: E402
from yar_gb300.scene import FlatScene, Mesh, make_object  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
from yar_gb300.build import reference_root  # noqa: E402

REFERENCE = reference_root()  # $YAR_REFERENCE_ROOT, else a `reference` folder beside the repository


def rays_and_results(flat, seed, n=4096):
    lo, hi = scenes.scene_box(flat)
    pad = 0.25 * (hi - lo)
    rays = scenes.random_rays(lo - pad, hi + pad, n, seed)
    # a slice of axis-aligned directions and rays starting on split planes
    rays[: n // 16, 4:7] = 0.0
    rays[: n // 16, 4 + (np.arange(n // 16) % 3)] = np.where(np.arange(n // 16) % 2 == 0, 1.0, -1.0)
    shadow = scenes.random_shadow_rays(lo, hi, n, seed + 1)
    (t, prim, obj, bary), _ = oracle.ref_cast(flat, rays)
    occ, _ = oracle.ref_cast(flat, shadow, any_hit=True)
    return dict(rays=rays, t=t, prim=prim, obj=obj, bary=bary, shadow_rays=shadow, occluded=occ)


def raycast_small():
    flat = scenes.raycast_scene(seed=3, grid=24, spheres=6, level=2, build=False)
    flat, _ = oracle.ref_build(flat)
    flat.write(os.path.join(HERE, "raycast_small.yfs"))
    np.savez_compressed(os.path.join(HERE, "raycast_small.npz"), **rays_and_results(flat, 11))


def transform_small():
    rng = np.random.default_rng(5)
    flat = FlatScene()
    sv, si = scenes.icosphere(1.0, 2)
    bv = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
                  np.float32)
    bi = np.array([[0, 1, 2], [2, 3, 0], [0, 1, 5], [5, 4, 0], [1, 2, 6], [6, 5, 1], [2, 3, 7], [7, 6, 2],
                   [3, 0, 4], [4, 7, 3], [4, 5, 6], [6, 7, 4]], np.int32)
    flat.meshes = [Mesh(sv, si), Mesh(bv, bi)]
    objects = []
    for k in range(12):
        a, b = rng.uniform(0, 2 * np.pi, 2)
        ca, sa, cb, sb = np.cos(a), np.sin(a), np.cos(b), np.sin(b)
        rot = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]]) @ np.array([[1, 0, 0], [0, cb, -sb], [0, sb, cb]])
        m = np.zeros((3, 4))
        m[:, :3] = rot @ np.diag(rng.uniform(0.2, 0.7, 3))
        m[:, 3] = rng.uniform(-2, 2, 3)
        objects.append(make_object(k % 2, m.astype(np.float32).reshape(12)))
    flat.objects = np.array(objects)
    flat, _ = oracle.ref_build(flat)
    flat.write(os.path.join(HERE, "transform_small.yfs"))
    np.savez_compressed(os.path.join(HERE, "transform_small.npz"), **rays_and_results(flat, 21))


def parse_regression_meshes():
    text = open(os.path.join(REFERENCE, "src/ref/test_kdtree.cpp"), encoding="latin-1").read()
    body = text[text.index("create_custom_meshes()"):]
    meshes = []
    for block in re.findall(r"mesh\.vertices = \{(.*?)\};\s*mesh\.indices = \{(.*?)\};", body, re.S)[:2]:
        nums = [float(x.rstrip("f")) for x in re.findall(r"-?\d+\.\d+f?", block[0])]
        idx = [int(x) for x in re.findall(r"\d+", block[1])]
        meshes.append((np.array(nums, np.float32).reshape(-1, 3), np.array(idx, np.int32).reshape(-1, 3)))
    return meshes


def kdtree_regression(n=4096):
    out = {}
    for k, (v, i) in enumerate(parse_regression_meshes()):
        flat = FlatScene()
        flat.meshes = [Mesh(v, i)]
        flat.objects = np.array([make_object(0)])
        flat, _ = oracle.ref_build(flat)
        with tempfile.TemporaryDirectory() as d:
            s, o = os.path.join(d, "m.yfs"), os.path.join(d, "o.bin")
            flat.write(s)
            info = oracle._ref("regress", s, o, n)
            raw = np.fromfile(o, np.uint8).reshape(n, 32)
        assert info["kdtree_vs_brute_force_mismatches"] == 0, info
        out["mesh%d_vertices" % k] = v
        out["mesh%d_indices" % k] = i
        out["mesh%d_bounds" % k] = flat.meshes[0].bounds
        out["mesh%d_nodes" % k] = flat.meshes[0].nodes
        out["mesh%d_rays" % k] = raw[:, :24].copy().view(np.float32)
        out["mesh%d_t" % k] = raw[:, 24:28].copy().view(np.float32).reshape(n)
        out["mesh%d_prim" % k] = raw[:, 28:32].copy().view(np.uint32).reshape(n)
    np.savez_compressed(os.path.join(HERE, "kdtree_regression.npz"), **out)


def cornell_c1_64():
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=1, width=64, height=64, spp=16, maxdepth=8))
        yfs = os.path.join(HERE, "cornell_c1_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_c1_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_ggx_64():
    """The Cornell box with a GGX metal box and a rough-glass box."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell_ggx.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=2, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES))
        yfs = os.path.join(HERE, "cornell_ggx_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_ggx_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_delta_64():
    """The Cornell box with a mirror box, a smooth-glass box and a light above
    the ceiling."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell_delta.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=5, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.DELTA_BOXES,
                                                  upper_light=scenes.UPPER_LIGHT))
        yfs = os.path.join(HERE, "cornell_delta_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_delta_64.npz"), image=img, variance=np.float64(info["variance"]))


def _filter_golden(name, pixel_filter, seed):
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, name + ".pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=seed, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, pixel_filter=pixel_filter))
        yfs = os.path.join(HERE, name + ".yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), image=img, variance=np.float64(info["variance"]))


def cornell_gaussian_64():
    """The GGX Cornell box through a Gaussian pixel filter of radius 1.5, alpha 2."""
    _filter_golden("cornell_gaussian_64", '"gaussian" "float xwidth" [1.5] "float ywidth" [1.5] "float alpha" [2]', 6)


def cornell_triangle_64():
    """The GGX Cornell box through a triangle pixel filter of radius 2."""
    _filter_golden("cornell_triangle_64", '"triangle" "float xwidth" [2] "float ywidth" [2]', 7)


def cornell_c1_256():
    """The C1 configuration itself: the Cornell box at 256 x 256, 16 spp,
    maxdepth 8, seed offset 1 (the image and variance only; the scene is
    cornell_c1_64.yfs at 256 x 256)."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=1, width=256, height=256, spp=16, maxdepth=8))
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_c1_256.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_refractor_64():
    """cornell_delta_64 with a perfect-refractor ceiling (object 1)."""
    s = FlatScene.read(os.path.join(HERE, "cornell_delta_64.yfs"))
    scenes.make_ceiling_refractor(s)
    s.write(os.path.join(HERE, "cornell_refractor_64.yfs"))
    img, info = oracle.ref_render_flat(s, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_refractor_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_layered_64():
    """The Cornell box with a plastic box and a coated-diffuse (substrate) box."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell_layered.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=6, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.LAYERED_BOXES))
        yfs = os.path.join(HERE, "cornell_layered_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_layered_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_layered_yar_64():
    """cornell_layered_64 rendered as a non-pbrt scene."""
    s = FlatScene.read(os.path.join(HERE, "cornell_layered_64.yfs"))
    s.config["pbrt3_scene"] = 0
    s.write(os.path.join(HERE, "cornell_layered_yar_64.yfs"))
    img, info = oracle.ref_render_flat(s, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_layered_yar_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_lights_64():
    """The GGX Cornell box with point, spot and distant lights besides the quad light."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell_lights.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=7, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, light_sources=scenes.DELTA_LIGHTS))
        yfs = os.path.join(HERE, "cornell_lights_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_lights_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_meshlight_64():
    """The GGX Cornell box with two triangle-mesh lights besides the quad light."""
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, "cornell_meshlight.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=8, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, mesh_lights=scenes.MESH_LIGHTS))
        yfs = os.path.join(HERE, "cornell_meshlight_64.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_meshlight_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_spherelight_64():
    """cornell_ggx_64 with two sphere lights."""
    s = FlatScene.read(os.path.join(HERE, "cornell_ggx_64.yfs"))
    scenes.add_sphere_lights(s)
    s.write(os.path.join(HERE, "cornell_spherelight_64.yfs"))
    img, info = oracle.ref_render_flat(s, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_spherelight_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def _pbrt_golden(name, seed, **kw):
    with tempfile.TemporaryDirectory() as d:
        pbrt = os.path.join(d, name + ".pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=seed, width=64, height=64, spp=16, maxdepth=8, **kw))
        oracle.ref_flatten(pbrt, os.path.join(HERE, name + ".yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), image=img, variance=np.float64(info["variance"]))


def cornell_translucent_64():
    _pbrt_golden("cornell_translucent_64", 9, box_materials=scenes.TRANSLUCENT_BOXES)


def cornell_transmission_64():
    s = scenes.make_diffuse_transmission(FlatScene.read(os.path.join(HERE, "cornell_translucent_64.yfs")))
    s.write(os.path.join(HERE, "cornell_transmission_64.yfs"))
    img, info = oracle.ref_render_flat(s, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_transmission_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def cornell_uber_64():
    _pbrt_golden("cornell_uber_64", 10, box_materials=scenes.UBER_BOXES)


def cornell_mix_64():
    _pbrt_golden("cornell_mix_64", 11, box_materials=scenes.MIX_BOXES, named_materials=scenes.MIX_NAMED)


def cornell_envconst_64():
    _pbrt_golden("cornell_envconst_64", 12, box_materials=scenes.GGX_BOXES,
                 light_sources=scenes.ENVIRONMENT_CONSTANT)


def cornell_envmap_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "sky.exr"), scenes.environment_map(), False, {})
        pbrt = os.path.join(d, "cornell_envmap.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=13, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.DELTA_BOXES,
                                                  light_sources=scenes.environment_statements("sky.exr")))
        oracle.ref_flatten(pbrt, os.path.join(HERE, "cornell_envmap_64.yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_envmap_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_texture_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "checks.exr"), scenes.texture_image(), False, {})
        pbrt = os.path.join(d, "cornell_texture.pbrt")
        texs = scenes.texture_statements("checks.exr") + scenes.texture_statements("checks.exr", "fine", 2.0, 3.0)
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=17, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, textures=texs,
                                                  wall_textures={2: "checks", 3: "fine", 0: "fine"}))
        oracle.ref_flatten(pbrt, os.path.join(HERE, "cornell_texture_64.yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_texture_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_alpha_64():
    """The GGX Cornell box with an alpha-textured fence across the room: the
    alpha test cuts the fence's camera, bounce, probe and shadow hits."""
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "cutout.exr"), scenes.cutout_image(), False, {})
        pbrt = os.path.join(d, "cornell_alpha.pbrt")
        tex = ('Texture "cutout" "float" "imagemap" "string filename" "cutout.exr"',)
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=19, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, textures=tex,
                                                  extra_shapes=scenes.cutout_fence()))
        oracle.ref_flatten(pbrt, os.path.join(HERE, "cornell_alpha_64.yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_alpha_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_bump_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "checks.exr"), scenes.texture_image(), False, {})
        exr.write_exr(os.path.join(d, "bumps.exr"), scenes.bump_image(), False, {})
        pbrt = os.path.join(d, "cornell_bump.pbrt")
        texs = (scenes.texture_statements("checks.exr") + scenes.texture_statements("checks.exr", "fine", 2.0, 3.0) +
                ('Texture "bumps" "float" "imagemap" "string filename" "bumps.exr"',
                 'Texture "bumps2" "float" "imagemap" "string filename" "bumps.exr" "float uscale" [2] '
                 '"float vscale" [2]',
                 'Texture "lift" "float" "constant" "float value" [0.02]'))
        floor_normals = ' "normal N" [-0.1 1 -0.1 0.1 1 -0.1 0.1 1 0.1 -0.1 1 0.1]'
        walls = {
            0: ('Material "matte" "rgb Kd" [0.6 0.55 0.5] "texture bumpmap" "lift"', floor_normals),
            1: ('Material "matte" "rgb Kd" [0.7 0.7 0.7]', ""),
            2: ('Material "matte" "texture Kd" "checks" "texture bumpmap" "bumps"', ""),
            3: ('Material "plastic" "texture Kd" "fine" "rgb Ks" [0.3 0.3 0.3] "float roughness" [0.1] '
                '"texture bumpmap" "bumps2"', ""),
            4: ('Material "translucent" "rgb Kd" [0.5 0.4 0.3] "rgb Ks" [0.2 0.2 0.2] "rgb reflect" [0.6 0.6 0.6] '
                '"rgb transmit" [0.3 0.3 0.3] "float roughness" [0.2] "texture bumpmap" "bumps"', ""),
        }
        panel = scenes.bump_panel('Material "glass" "float uroughness" [0.25] "float vroughness" [0.25] '
                                  '"float index" [1.5] "rgb Kr" [1 1 1] "rgb Kt" [1 1 1] "texture bumpmap" "bumps2"')
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=21, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.GGX_BOXES, textures=texs,
                                                  wall_materials=walls, extra_shapes=panel))
        yfs = os.path.join(d, "cornell_bump.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        s = FlatScene.read(yfs)
        mats = s.materials
        checks = int(mats["reflectance_texture"][s.objects["material_index"][2]])
        assert checks > 0 and int(mats["bump_texture"][s.objects["material_index"][2]]) > 0
        # the panel: textured Kr (2 x 3) and Kt
        g = int(s.objects["material_index"][-1])
        assert int(mats["type"][g]) == 7 and int(mats["bump"][g]) == 2  # glass
        mats["reflectance_texture"][g] = checks
        mats["reflectance_uv_scale"][g] = (2.0, 3.0)
        mats["transmittance_texture"][g] = checks
        mats["transmittance_uv_scale"][g] = (1.0, 1.0)
        # the ceiling: diffuse transmission with textured reflectance and transmittance
        c = int(s.objects["material_index"][1])
        mats["type"][c] = 3  # diffuse transmission
        s.objects["material_type"][s.objects["material_index"] == c] = 3
        mats["reflectance"][c] = (0.5, 0.5, 0.5)
        mats["reflectance_texture"][c] = checks
        mats["reflectance_uv_scale"][c] = (1.0, 1.0)
        mats["transmittance"][c] = (0.4, 0.4, 0.4)
        mats["transmittance_texture"][c] = checks
        mats["transmittance_uv_scale"][c] = (3.0, 2.0)
        mats["diffuse"][c] = (0.9, 0.8, 0.7)
        s.write(os.path.join(HERE, "cornell_bump_64.yfs"))
        img, info = oracle.ref_render_flat(s, threads=8, textures_from=pbrt)
    np.savez_compressed(os.path.join(HERE, "cornell_bump_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_spectex_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "checks.exr"), scenes.texture_image(), False, {})
        pbrt = os.path.join(d, "cornell_spectex.pbrt")
        open(pbrt, "w").write(scenes.specular_texture_pbrt("checks.exr"))
        yfs = os.path.join(d, "cornell_spectex.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        s = scenes.texture_glass_panel(FlatScene.read(yfs))
        s.write(os.path.join(HERE, "cornell_spectex_64.yfs"))
        img, info = oracle.ref_render_flat(s, threads=8, textures_from=pbrt)
    np.savez_compressed(os.path.join(HERE, "cornell_spectex_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_direct_tex_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "checks.exr"), scenes.texture_image(), False, {})
        exr.write_exr(os.path.join(d, "bumps.exr"), scenes.bump_image(), False, {})
        pbrt = os.path.join(d, "cornell_direct_tex.pbrt")
        open(pbrt, "w").write(scenes.specular_texture_pbrt("checks.exr", seed=31, bump_file="bumps.exr",
                                                           integrator="directlighting", light_samples=2))
        yfs = os.path.join(d, "cornell_direct_tex.yfs")
        oracle.ref_flatten(pbrt, yfs, seed_offset=1)
        s = scenes.texture_glass_panel(FlatScene.read(yfs))
        assert int(s.config["rendering_algorithm"]) == 0
        s.write(os.path.join(HERE, "cornell_direct_tex_64.yfs"))
        img, info = oracle.ref_render_flat(s, threads=8, textures_from=pbrt)
    np.savez_compressed(os.path.join(HERE, "cornell_direct_tex_64.npz"), image=img, variance=np.float64(info["variance"]))


def write_fourier_bsdf(path, channels, nodes=15, order=8, gloss=6.0, albedo=(0.7, 0.5, 0.3)):
    """A layerlab "SCATFUN" v1 file (the subset Pbrt3_Fourier_Material::load_bsdf_file
    reads, src/lib/material_pbrt.cpp:24-102): increasing zenith cosines from -1
    to 1, an unused CDF table, (offset, length) per node pair (outgoing-major)
    and the coefficients.  The tabulated function |mu_i| f(mu_o, mu_i, phi) is
    a diffuse term plus a lobe around phi = pi, reflection pairs only (mu_o > 0,
    mu_i < 0); each pair keeps the terms above a threshold, so series lengths
    differ.  Three channels store Y, R and B."""
    import struct
    mu = np.linspace(-1.0, 1.0, nodes).astype(np.float32)
    phi = (np.arange(256) + 0.5) * (np.pi / 256)
    lum = np.array([0.2126729, 0.7151522, 0.0721750])
    offsets, counts, coeffs = [], [], []
    for o in range(nodes):
        for i in range(nodes):
            if not (mu[o] > 0 and mu[i] < 0):
                offsets.append(len(coeffs))
                counts.append(0)
                continue
            spread = gloss * (0.5 + 0.5 * float(mu[o]))
            f = abs(float(mu[i])) * (0.15 + np.exp(spread * (np.cos(phi - np.pi) - 1.0)) * (0.3 + 0.4 * float(mu[o])))
            a = np.array([np.mean(f * np.cos(k * phi)) * (1.0 if k == 0 else 2.0) for k in range(order)])
            keep = int(np.max(np.nonzero(np.abs(a) > 1e-3)[0])) + 1
            offsets.append(len(coeffs))
            counts.append(keep)
            if channels == 1:
                coeffs.extend(a[:keep])
            else:
                rgb = [a[:keep] * c for c in albedo]
                y = lum[0] * rgb[0] + lum[1] * rgb[1] + lum[2] * rgb[2]
                coeffs.extend(y)
                coeffs.extend(rgb[0])
                coeffs.extend(rgb[2])
    header = b"SCATFUN" + bytes([1]) + struct.pack("<9I", 1, nodes, len(coeffs), order, channels, 1, 0, 0, 0) + \
        struct.pack("<5f", 1.0, 0.1, 0.1, 0.0, 0.0)
    assert len(header) == 64
    table = np.stack([np.array(offsets, np.uint32), np.array(counts, np.uint32)], axis=1).reshape(-1)
    with open(path, "wb") as f:
        f.write(header)
        f.write(mu.tobytes())
        f.write(np.zeros(nodes * nodes, np.float32).tobytes())
        f.write(table.astype(np.uint32).tobytes())
        f.write(np.array(coeffs, np.float32).tobytes())


FOURIER_BOXES = ('Material "fourier" "string bsdffile" "mono.bsdf"', 'Material "fourier" "string bsdffile" "rgb.bsdf"')


def cornell_fourier_64():
    with tempfile.TemporaryDirectory() as d:
        write_fourier_bsdf(os.path.join(d, "mono.bsdf"), 1)
        write_fourier_bsdf(os.path.join(d, "rgb.bsdf"), 3, gloss=12.0)
        pbrt = os.path.join(d, "cornell_fourier.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=23, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=FOURIER_BOXES))
        oracle.ref_flatten(pbrt, os.path.join(HERE, "cornell_fourier_64.yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_fourier_64.npz"), image=img, variance=np.float64(info["variance"]))


def cornell_direct_64():
    _pbrt_golden("cornell_direct_64", 15, box_materials=scenes.GGX_BOXES, light_sources=scenes.DELTA_LIGHTS,
                 light_samples=4, integrator="directlighting")


def cornell_direct_env_64():
    from yar_gb300 import exr
    with tempfile.TemporaryDirectory() as d:
        exr.write_exr(os.path.join(d, "sky.exr"), scenes.environment_map(), False, {})
        pbrt = os.path.join(d, "cornell_direct_env.pbrt")
        open(pbrt, "w").write(scenes.cornell_pbrt(seed=16, width=64, height=64, spp=16, maxdepth=8,
                                                  box_materials=scenes.DELTA_BOXES, light_samples=3,
                                                  light_sources=scenes.environment_statements("sky.exr", samples=2),
                                                  integrator="directlighting"))
        oracle.ref_flatten(pbrt, os.path.join(HERE, "cornell_direct_env_64.yfs"), seed_offset=1)
        img, info = oracle.ref_render(pbrt, seed_offset=1, threads=8)
    np.savez_compressed(os.path.join(HERE, "cornell_direct_env_64.npz"), image=img,
                        variance=np.float64(info["variance"]))


def checkpoint_c1():
    """The reference's own checkpoint files: render_scene with a checkpoint directory."""
    import shutil
    import subprocess
    out_dir = os.path.join(HERE, "checkpoint_c1")
    shutil.rmtree(out_dir, ignore_errors=True)
    with tempfile.TemporaryDirectory() as d:
        name = "cornell_checkpoint.pbrt"
        open(os.path.join(d, name), "w").write(scenes.cornell_pbrt(seed=14, width=72, height=72, spp=4, maxdepth=6))
        oracle.ref_flatten(os.path.join(d, name), os.path.join(HERE, "checkpoint_c1.yfs"), seed_offset=1)
        raw = os.path.join(d, "img.bin")
        subprocess.run([oracle.REF_BIN, "render", name, raw, "--threads=4", "--seedoffset=1", "--checkpoint-dir=ckpt"],
                       cwd=d, check=True, stdout=subprocess.DEVNULL)
        shutil.copytree(os.path.join(d, "ckpt"), out_dir)
        data = open(raw, "rb").read()
    w, h = np.frombuffer(data[:8], np.uint32)
    variance = float(np.frombuffer(data[8:16], np.float64)[0])
    img = np.frombuffer(data[20:], np.float32).reshape(int(h), int(w), 3).copy()
    np.savez_compressed(os.path.join(HERE, "checkpoint_c1.npz"), image=img, variance=np.float64(variance))


def kdtree_cache_files():
    """The reference's kd-tree cache files (KdTree::save) of the raycast_small
    scene's first two meshes and of its scene tree."""
    flat = FlatScene.read(os.path.join(HERE, "raycast_small.yfs"))
    out_dir = os.path.join(HERE, "kdtree_cache")
    os.makedirs(out_dir, exist_ok=True)
    with tempfile.TemporaryDirectory() as d:
        a, b = os.path.join(d, "in.yfs"), os.path.join(d, "out.yfs")
        flat.write(a)
        oracle._ref("build", a, b, "--threads=2", "--cache-dir=" + d)
        for name in ("mesh_0.kdtree", "mesh_1.kdtree", "scene.kdtree"):
            with open(os.path.join(d, name), "rb") as src, open(os.path.join(out_dir, name), "wb") as dst:
                dst.write(src.read())


def exr_files():
    """The reference's EXR writer (write_openexr_image) on the C1 golden image
    (uncompressed and ZIP) and on an image of special values (exact half
    rounding ties, subnormals, overflow, signs)."""
    img = np.load(os.path.join(HERE, "cornell_c1_64.npz"))["image"].astype(np.float32)
    rng = np.random.default_rng(5)
    n = 48 * 32 * 3
    v = (rng.standard_normal(n) * 10 ** rng.uniform(-9, 5, n)).astype(np.float32)
    base = rng.integers(0x0001, 0x7BFF, 400).astype(np.uint16).view(np.float16).astype(np.float32)
    v[:400] = (base.view(np.uint32) + 0x1000).view(np.float32)     # exact ties between two halves
    v[400:410] = [0.0, -0.0, 6.0e-8, 2.98e-8, 1e-30, 65504.0, 65519.99, 65520.0, 1e9, -1e9]
    special = v.reshape(32, 48, 3)
    np.save(os.path.join(HERE, "exr_special_input.npy"), special)
    with tempfile.TemporaryDirectory() as d:
        for name, im, extra in (("exr_cornell_none", img, []), ("exr_cornell_zip", img, ["--compress"]),
                                ("exr_special_none", special, [])):
            raw = os.path.join(d, "im.f32")
            im.astype(np.float32).tofile(raw)
            out = os.path.join(HERE, name + ".exr")
            attrs = ["--spp=16", "--variance=0.25", "--input=cornell.pbrt"] if "cornell" in name else []
            oracle._ref("exr", raw, im.shape[1], im.shape[0], out, *attrs, *extra)


if __name__ == "__main__":
    if not oracle.have_reference():
        sys.exit("oracle/_ref/yar_ref is not built (oracle/build_ref.sh)")
    which = sys.argv[1:] or ["raycast_small", "transform_small", "kdtree_regression", "cornell_c1_64",
                             "cornell_ggx_64", "cornell_delta_64", "cornell_refractor_64", "cornell_layered_64",
                             "cornell_layered_yar_64", "cornell_lights_64", "cornell_meshlight_64",
                             "cornell_spherelight_64", "cornell_translucent_64", "cornell_transmission_64",
                             "cornell_uber_64", "cornell_mix_64", "cornell_envconst_64", "cornell_envmap_64",
                             "cornell_direct_64", "cornell_direct_env_64", "cornell_texture_64", "checkpoint_c1",
                             "cornell_gaussian_64", "cornell_triangle_64", "cornell_c1_256", "cornell_alpha_64",
                             "cornell_bump_64", "cornell_fourier_64", "cornell_spectex_64", "cornell_direct_tex_64",
                             "exr_files",
                             "kdtree_cache_files"]
    for name in which:
        globals()[name]()
        print("wrote", name)
