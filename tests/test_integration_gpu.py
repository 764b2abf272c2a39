"""The reference-side drop-in (oracle/render_scene_gpu.cpp, built into
oracle/_ref/yar_ref_gpu): YAR's own pbrt-v3 loader and kd-tree builder feed
render_scene_gpu, which flattens the Scene_Context and renders it through
the C ABI.  Its image is the reference's render_scene image within the
render bars, and bit-identical to the oracle with correctly rounded
trigonometry on the flat scene the reference harness writes."""
import os

import numpy as np
import pytest

import oracle
from conftest import golden
from yar_gb300 import scenes
from yar_gb300.scene import FlatScene

pytestmark = pytest.mark.gpu

needs_adapter = pytest.mark.skipif(not os.path.exists(oracle.REF_GPU_BIN),
                                   reason="the drop-in adapter is built with the reference sources")


@needs_adapter
def test_render_scene_gpu_drop_in_matches_render_scene(tmp_path):
    p = tmp_path / "cornell.pbrt"
    p.write_text(scenes.cornell_pbrt(seed=1, width=64, height=64, spp=16, maxdepth=8))
    img, var = oracle.ref_render_gpu(str(p), seed_offset=1)
    g = np.load(golden("cornell_c1_64.npz"))
    same = np.all(img.view(np.uint32) == g["image"].view(np.uint32), axis=2).mean()
    rel = float(np.abs(img.astype(np.float64) - g["image"]).sum() / g["image"].astype(np.float64).sum())
    assert same >= 0.90 and rel < 1e-4, (same, rel)
    assert abs(var - float(g["variance"])) <= 1e-5 * float(g["variance"])
    want, want_var = oracle.render(FlatScene.read(golden("cornell_c1_64.yfs")), correctly_rounded_trig=True)
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    assert var == want_var
