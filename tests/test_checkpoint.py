"""Checkpoint files (render_scene with a checkpoint directory,
src/ref/reference_renderer.cpp:180-324, :446-584): the reference's own files in
tests/golden/checkpoint_c1, read and merged here as the reference merges them,
and yar_gpu_render_checkpoint resuming from them, from part of them, and from
its own files."""
import os
import shutil

import numpy as np
import pytest

from conftest import golden

INPUT_NAME = "cornell_checkpoint.pbrt"


def read_tile(path):
    raw = open(path, "rb").read()
    time = np.frombuffer(raw[:4], np.float32)[0]
    variance = np.frombuffer(raw[4:12], np.float64)[0]
    bounds = np.frombuffer(raw[12:28], np.int32)
    w, h = bounds[2] - bounds[0], bounds[3] - bounds[1]
    pixels = np.frombuffer(raw[28:], np.float32).reshape(h, w, 4)
    return time, variance, bounds, pixels


def merge(tiles, width, height):
    """Film::merge_tile in tile order, then Film::get_image (box filter)."""
    film = np.zeros((height, width, 4), np.float32)
    for _, _, b, px in tiles:
        film[b[1]:b[3], b[0]:b[2]] += px
    img = np.zeros((height, width, 3), np.float32)
    w = film[..., 3]
    nz = w != 0
    inv = np.zeros_like(w)
    inv[nz] = np.float32(1) / w[nz]
    img = film[..., :3] * inv[..., None]
    return np.maximum(img, np.float32(0))


def test_reference_checkpoint_files_merge_to_the_reference_image():
    d = golden("checkpoint_c1")
    meta = open(os.path.join(d, "checkpoint")).read().split()
    assert meta == ["input_filename", INPUT_NAME, "total_tile_count", "4", "samples_per_pixer", "4"]
    tiles = [read_tile(os.path.join(d, "tile_%04d" % t)) for t in range(4)]
    g = np.load(golden("checkpoint_c1.npz"))
    img = merge(tiles, 72, 72)
    assert np.array_equal(img.view(np.uint32), g["image"].view(np.uint32))
    acc, count = 0.0, 0
    for t, (_, var, _, _) in enumerate(tiles):
        acc += var
        count += min(64, 72 - (t % 2) * 64) * min(64, 72 - (t // 2) * 64)
    assert acc / count == float(g["variance"])


def _ctx_with_scene():
    from yar_gb300 import native
    from yar_gb300.scene import FlatScene
    ctx = native.Context(0)
    ctx.upload_scene(FlatScene.read(golden("checkpoint_c1.yfs")))
    return ctx


@pytest.mark.gpu
def test_gpu_resumes_a_finished_reference_checkpoint(tmp_path):
    d = tmp_path / "ckpt"
    shutil.copytree(golden("checkpoint_c1"), d)
    ctx = _ctx_with_scene()
    img, st = ctx.render_checkpoint(72, 72, d, INPUT_NAME)
    g = np.load(golden("checkpoint_c1.npz"))
    assert np.array_equal(img.view(np.uint32), g["image"].view(np.uint32))
    assert st.variance == float(g["variance"])
    assert st.paths == 0  # nothing left to render
    assert sorted(os.listdir(d)) == ["checkpoint", "tile_0000", "tile_0001", "tile_0002", "tile_0003"]
    ctx.close()


@pytest.mark.gpu
def test_gpu_finishes_a_partial_reference_checkpoint_and_resumes_its_own(tmp_path):
    from test_render_gpu import compare, MEAN_REL_TOL, BIT_EQUAL_MIN
    d = tmp_path / "ckpt"
    shutil.copytree(golden("checkpoint_c1"), d)
    os.remove(d / "tile_0001")
    os.remove(d / "tile_0003")
    ctx = _ctx_with_scene()
    img, st = ctx.render_checkpoint(72, 72, d, INPUT_NAME)
    assert st.paths > 0
    g = np.load(golden("checkpoint_c1.npz"))
    same, rel = compare(img, g["image"])
    assert same >= BIT_EQUAL_MIN and rel < MEAN_REL_TOL, (same, rel)
    assert abs(st.variance - float(g["variance"])) <= 1e-5 * float(g["variance"])
    for t in (1, 3):  # the written tiles have the reference's bounds and size
        ref_tile = read_tile(golden(os.path.join("checkpoint_c1", "tile_%04d" % t)))
        new_tile = read_tile(d / ("tile_%04d" % t))
        assert np.array_equal(ref_tile[2], new_tile[2])
        assert new_tile[3].shape == ref_tile[3].shape
        assert new_tile[0] > 0.0
    # the tiles merged as the reference merges them give the same image
    tiles = [read_tile(d / ("tile_%04d" % t)) for t in range(4)]
    assert np.array_equal(merge(tiles, 72, 72).view(np.uint32), img.view(np.uint32))
    # resuming the now complete checkpoint renders nothing and gives the same image
    img2, st2 = ctx.render_checkpoint(72, 72, d, INPUT_NAME)
    assert st2.paths == 0
    assert np.array_equal(img2.view(np.uint32), img.view(np.uint32))
    assert st2.variance == st.variance
    ctx.close()


@pytest.mark.gpu
def test_gpu_checkpoint_from_scratch_equals_the_plain_render(tmp_path):
    ctx = _ctx_with_scene()
    plain, pst = ctx.render(72, 72)
    img, st = ctx.render_checkpoint(72, 72, tmp_path / "new", "some_scene.pbrt")
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    assert st.variance == pst.variance
    meta = open(tmp_path / "new" / "checkpoint").read().split()
    assert meta == ["input_filename", "some_scene.pbrt", "total_tile_count", "4", "samples_per_pixer", "4"]
    ctx.close()


@pytest.mark.gpu
def test_gpu_checkpoint_of_a_textured_scene_equals_the_plain_render(tmp_path, gpu_ctx):
    """Tiles rendered row by row as their own sample regions keep the camera
    differentials and the specular differential rays of textured scenes: the
    merged image is the plain render's, bit for bit."""
    from yar_gb300.scene import FlatScene
    s = FlatScene.read(golden("cornell_spectex_64.yfs"))
    s.config["render_region"] = (0, 0, 130, 72)
    s.camera["image_extent"] = (130, 72)
    gpu_ctx.upload_scene(s)
    plain, pst = gpu_ctx.render(130, 72)
    img, st = gpu_ctx.render_checkpoint(130, 72, tmp_path / "tex", "spectex.pbrt")
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    assert st.variance == pst.variance


@pytest.mark.gpu
def test_gpu_checkpoint_refuses_another_project(tmp_path):
    from yar_gb300 import native
    d = tmp_path / "ckpt"
    shutil.copytree(golden("checkpoint_c1"), d)
    ctx = _ctx_with_scene()
    with pytest.raises(native.YarError) as e:
        ctx.render_checkpoint(72, 72, d, "other.pbrt")
    assert e.value.code == native.YAR_ERR_IO
    ctx.close()


def test_gpu_written_checkpoint_merges_to_the_gpu_image():
    """checkpoint_gpu: tiles 1 and 3 written by yar_gpu_render_checkpoint
    (tests/golden/make_gpu_checkpoint.py), merged as the reference merges them."""
    d = golden("checkpoint_gpu")
    tiles = [read_tile(os.path.join(d, "tile_%04d" % t)) for t in range(4)]
    g = np.load(golden("checkpoint_gpu.npz"))
    assert np.array_equal(merge(tiles, 72, 72).view(np.uint32), g["image"].view(np.uint32))


def test_reference_resumes_a_gpu_written_checkpoint(tmp_path):
    """The reference's render_scene finds every tile in the GPU-finished
    directory, renders nothing, and returns the GPU's image and variance."""
    import subprocess
    import oracle
    from yar_gb300 import scenes
    if not oracle.have_reference():
        pytest.skip("reference not built here")
    d = tmp_path / "run"
    shutil.copytree(golden("checkpoint_gpu"), d / "ckpt")
    (d / INPUT_NAME).write_text(scenes.cornell_pbrt(seed=14, width=72, height=72, spp=4, maxdepth=6))
    raw = d / "img.bin"
    subprocess.run([oracle.REF_BIN, "render", INPUT_NAME, str(raw), "--threads=2", "--seedoffset=1",
                    "--checkpoint-dir=ckpt"], cwd=d, check=True, stdout=subprocess.DEVNULL)
    data = raw.read_bytes()
    img = np.frombuffer(data[20:], np.float32).reshape(72, 72, 3)
    variance = float(np.frombuffer(data[8:16], np.float64)[0])
    g = np.load(golden("checkpoint_gpu.npz"))
    assert np.array_equal(img.view(np.uint32), g["image"].view(np.uint32))
    assert variance == float(g["variance"])
    assert sorted(os.listdir(d / "ckpt")) == ["checkpoint", "tile_0000", "tile_0001", "tile_0002", "tile_0003"]
