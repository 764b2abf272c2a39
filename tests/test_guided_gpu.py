"""GPU tests of the guided render (yar_gpu_guided_render): its plain mode is
the reference's path tracer in independent one-sample passes, and drawing
continuations from the learned proposal changes the noise, not the
expectation (one-sample MIS with the BSDF).

Image means are compared, at sample counts where their Monte Carlo error is
well under the stated bound: 3% between two estimators of the same image."""
import numpy as np
import pytest

from conftest import golden
from yar_gb300 import native, scenes
from yar_gb300.scene import FlatScene

pytestmark = pytest.mark.gpu

MEAN_REL_TOL = 0.03


@pytest.fixture(scope="module")
def small_room():
    s = scenes.hard_lighting_room(width=64, height=64, cells=100)
    return s


def test_plain_passes_match_the_reference_render(gpu_ctx):
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    g = np.load(golden("cornell_c1_64.npz"))
    gpu_ctx.upload_scene(s)
    img, sums, st = gpu_ctx.guided_render(64, 64, passes=64)
    assert st.passes == 64 and st.train_samples == 0
    assert np.allclose(sums / 64.0, img, rtol=1e-6, atol=1e-7)
    ref = g["image"].astype(np.float64)
    assert abs(img.mean() - ref.mean()) < MEAN_REL_TOL * ref.mean(), (img.mean(), ref.mean())
    # independent pass streams: two offsets give different images with the same mean
    img2, _, _ = gpu_ctx.guided_render(64, 64, passes=64, stream_offset=1)
    assert not np.array_equal(img, img2)
    assert abs(img2.mean() - img.mean()) < MEAN_REL_TOL * img.mean()


def test_guided_is_unbiased_and_trains(gpu_ctx, small_room):
    gpu_ctx.upload_scene(small_room)
    plain, _, st_p = gpu_ctx.guided_render(64, 64, passes=512)
    guided, _, st_g = gpu_ctx.guided_render(64, 64, passes=512, guide_fraction=0.5, train_passes=32,
                                            stream_offset=2)
    assert st_g.train_samples > 0 and np.isfinite(st_g.loss)
    assert plain.mean() > 0
    assert abs(guided.mean() - plain.mean()) < MEAN_REL_TOL * plain.mean(), (guided.mean(), plain.mean())
    # the halves of the image agree too (the opening's light pool vs the rest)
    for sl in (np.s_[:32], np.s_[32:]):
        assert abs(guided[sl].mean() - plain[sl].mean()) < 2 * MEAN_REL_TOL * plain[sl].mean()


@pytest.mark.parametrize("name", ["cornell_texture_64", "cornell_spectex_64", "cornell_bump_64"])
def test_guided_renders_of_textured_scenes_are_unbiased(gpu_ctx, name):
    """Image textures, bump maps and textures behind delta bounces in the
    guided render: the stratified form and the one-sample passes, guided,
    have the plain render's image mean."""
    s = FlatScene.read(golden(name + ".yfs"))
    s.config["x_pixel_sample_count"] = s.config["y_pixel_sample_count"] = 16
    gpu_ctx.upload_scene(s)
    plain, _ = gpu_ctx.render(64, 64)
    strat, _, st = gpu_ctx.guided_render(64, 64, samples_per_pixel=256, guide_fraction=0.5, train_passes=8,
                                         train_steps=16, learning_rate=5e-3, stream_offset=6)
    assert st.train_samples > 0
    passes, _, _ = gpu_ctx.guided_render(64, 64, passes=256, guide_fraction=0.5, train_passes=8, train_steps=16,
                                         learning_rate=5e-3, stream_offset=7)
    for img in (strat, passes):
        assert np.isfinite(img).all()
        assert abs(img.mean() - plain.mean()) < MEAN_REL_TOL * plain.mean(), (name, img.mean(), plain.mean())


def test_time_budget_stops_early(gpu_ctx, small_room):
    gpu_ctx.upload_scene(small_room)
    _, _, st = gpu_ctx.guided_render(64, 64, passes=100000, time_budget=0.5)
    assert 1 <= st.passes < 100000
    assert st.seconds >= 0.5


def test_invalid_guided_params(gpu_ctx, small_room):
    gpu_ctx.upload_scene(small_room)
    for kw in ({"passes": 0}, {"passes": 4, "guide_fraction": 1.0}, {"passes": 4, "guide_fraction": -0.1}):
        with pytest.raises(native.YarError) as e:
            gpu_ctx.guided_render(64, 64, **kw)
        assert e.value.code == native.YAR_ERR_INVALID


def test_stratified_guided_is_unbiased(gpu_ctx, small_room):
    """The stratified form: the training passes, then the pixel sampler with
    continuations from the trained proposal.  Its image mean matches the plain
    render's (yar_gpu_render at the same sample count), and with guide
    fraction 0 it is the plain render on other pixel streams (checked on the
    Cornell box, whose light is not behind an opening: its image mean is
    steady at this sample count)."""
    s = small_room
    s.config["x_pixel_sample_count"] = 16
    s.config["y_pixel_sample_count"] = 16
    gpu_ctx.upload_scene(s)
    plain, _ = gpu_ctx.render(64, 64)
    guided, sums, st = gpu_ctx.guided_render(64, 64, samples_per_pixel=256, guide_fraction=0.5, train_passes=32,
                                             stream_offset=3)
    assert st.passes == 32 and st.train_samples > 0
    assert np.allclose(sums / 256.0, guided, rtol=1e-6, atol=1e-7)
    assert abs(guided.mean() - plain.mean()) < MEAN_REL_TOL * plain.mean(), (guided.mean(), plain.mean())
    for sl in (np.s_[:32], np.s_[32:]):
        assert abs(guided[sl].mean() - plain[sl].mean()) < 2 * MEAN_REL_TOL * plain[sl].mean()
    c = FlatScene.read(golden("cornell_c1_64.yfs"))
    c.config["x_pixel_sample_count"] = c.config["y_pixel_sample_count"] = 15
    gpu_ctx.upload_scene(c)
    plain, _ = gpu_ctx.render(64, 64)
    unguided, sums0, st0 = gpu_ctx.guided_render(64, 64, samples_per_pixel=200, stream_offset=4)  # 15 x 14 strata
    assert st0.passes == 0
    assert np.array_equal(sums0, unguided.astype(np.float64).reshape(sums0.shape) * 210.0)
    assert not np.array_equal(unguided, plain)
    assert abs(unguided.mean() - plain.mean()) < 0.01 * plain.mean(), (unguided.mean(), plain.mean())


def test_stratified_form_takes_the_strata_columns(gpu_ctx):
    """strata_x sets the columns of the pixel sampler's grid (rows ceil(n /
    nx)): 16 x 12 strata hold 192 samples per pixel; grids beyond 4:1 are
    refused."""
    from yar_gb300 import native
    c = FlatScene.read(golden("cornell_c1_64.yfs"))
    c.config["x_pixel_sample_count"] = c.config["y_pixel_sample_count"] = 14
    gpu_ctx.upload_scene(c)
    img, sums, st = gpu_ctx.guided_render(64, 64, samples_per_pixel=190, strata_x=16, stream_offset=5)
    assert np.array_equal(sums, img.astype(np.float64).reshape(sums.shape) * 192.0)
    plain, _ = gpu_ctx.render(64, 64)
    assert abs(img.mean() - plain.mean()) < 0.01 * plain.mean(), (img.mean(), plain.mean())
    with pytest.raises(native.YarError):
        gpu_ctx.guided_render(64, 64, samples_per_pixel=200, strata_x=100, stream_offset=5)
