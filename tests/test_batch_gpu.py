"""GPU tests of the batched render (yar_gpu_render_batch): one graph launch
renders every scene exactly as yar_gpu_render renders it alone (the same
kernels and per-path arithmetic, device-driven bounces), so images and
variances are bit-identical; the autotuner's choices are reported."""
import numpy as np
import pytest

from conftest import constant_bumps_with_delta_materials, golden
from yar_gb300 import native, scenes
from yar_gb300.scene import FlatScene

pytestmark = pytest.mark.gpu


def test_batch_matches_single_renders(gpu_ctx):
    a = FlatScene.read(golden("cornell_c1_64.yfs"))
    b = FlatScene.read(golden("cornell_ggx_64.yfs"))
    c = scenes.large_scene(seed=9, width=96, height=80, spp=4, maxdepth=6, meshes=6, level=3, lights=4)
    d = FlatScene.read(golden("cornell_c1_64.yfs"))
    d.config["x_pixel_sample_count"], d.config["y_pixel_sample_count"] = 3, 2
    d.config["rng_seed_offset"] = 5
    flats = [a, b, c, d]
    imgs, sst, st = gpu_ctx.render_batch(flats)
    assert st.paths == sum(int((f.config["render_region"][2] - f.config["render_region"][0]) *
                               (f.config["render_region"][3] - f.config["render_region"][1]) *
                               f.config["x_pixel_sample_count"] * f.config["y_pixel_sample_count"]) for f in flats)
    assert st.branches in (2, 4, 8) and st.chunk_paths > 0 and st.gpu_seconds > 0
    assert st.rays_closest >= st.paths
    for f, img, s in zip(flats, imgs, sst):
        gpu_ctx.upload_scene(f)
        r = f.config["render_region"]
        want, ws = gpu_ctx.render(int(r[2] - r[0]), int(r[3] - r[1]))
        assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
        assert s.variance == ws.variance
        assert 0 < s.completion_seconds <= st.gpu_seconds * 1.0001
        assert 1 <= s.traversal_kernel[0] <= 3 and 1 <= s.traversal_kernel[1] <= 3


def test_batch_renders_textures_bumps_alpha_and_fourier_as_single_renders(gpu_ctx):
    """Image textures (camera-ray differentials per chunk, specular
    differential rays behind delta bounces), bump maps, the alpha test and
    fourier tables render in a batch bit for bit as alone, next to a plain
    scene; constant bumps on delta materials too."""
    flats = [FlatScene.read(golden(n + ".yfs")) for n in
             ("cornell_texture_64", "cornell_bump_64", "cornell_alpha_64", "cornell_fourier_64", "cornell_c1_64",
              "cornell_spectex_64")]
    flats.append(constant_bumps_with_delta_materials())
    big = FlatScene.read(golden("cornell_texture_64.yfs"))
    big.config["render_region"] = (0, 0, 96, 96)
    big.camera["image_extent"] = (96, 96)
    big.config["x_pixel_sample_count"], big.config["y_pixel_sample_count"] = 3, 2
    flats.append(big)
    imgs, sst, st = gpu_ctx.render_batch(flats)
    for f, img, s in zip(flats, imgs, sst):
        gpu_ctx.upload_scene(f)
        r = f.config["render_region"]
        want, ws = gpu_ctx.render(int(r[2] - r[0]), int(r[3] - r[1]))
        assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
        assert s.variance == ws.variance


def test_batch_rejects_bad_input(gpu_ctx):
    with pytest.raises(native.YarError):
        gpu_ctx.render_batch([])
