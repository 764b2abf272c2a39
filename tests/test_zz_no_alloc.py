"""yar_gpu_render_static: rendering for callers that may not allocate device
memory at render time (a fixed, pre-reserved memory budget, no allocation
after start-up for latency reasons, or a device allocator owned by someone
else).  The entry point takes its working memory from a static device array
in the library instead of cudaMalloc, so the caller only provides the output
image in device memory.

Checked here through the C ABI: two calls in a row give the same image and
variance as yar_gpu_render (within the render tolerance of the other render
tests - in practice bit for bit, and at maxdepth 12, past the sampler's
dimension budget, too), the second call changes no device memory usage, a
render that does not fit the static array is refused with YAR_ERR_CAPACITY,
and a direct-lighting scene (which this entry point does not render) is
refused with YAR_ERR_UNSUPPORTED.  This file is collected last so that a failure here comes
after every other test has run."""
import numpy as np
import pytest

from conftest import cuda_available, golden
from yar_gb300 import native
from yar_gb300.scene import FlatScene

pytestmark = pytest.mark.gpu

MEAN_REL_TOL = 1e-4       # as tests/test_render_gpu.py
BIT_EQUAL_MIN = 0.90
VARIANCE_REL_TOL = 1e-5


def within_render_tolerance(img, ref):
    same = np.all(img.view(np.uint32) == ref.view(np.uint32), axis=2).mean()
    rel = float(np.abs(img.astype(np.float64) - ref).sum() / max(ref.astype(np.float64).sum(), 1e-30))
    return same >= BIT_EQUAL_MIN and rel < MEAN_REL_TOL, (same, rel)


@pytest.fixture(scope="module")
def torch_cuda():
    if not cuda_available():
        pytest.skip("no CUDA device")
    import torch
    return torch


@pytest.mark.parametrize("name,maxdepth", [("cornell_c1_64", None), ("cornell_ggx_64", None),
                                           ("cornell_ggx_64", 12)])
def test_static_render_matches_render_twice(torch_cuda, name, maxdepth):
    torch = torch_cuda
    s = FlatScene.read(golden(name + ".yfs"))
    if maxdepth is not None:
        s.config["max_light_bounces"] = maxdepth
    ctx = native.Context(0)
    try:
        ctx.upload_scene(s)
        ref, ref_stats = ctx.render(64, 64)
        out = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        for call in range(2):
            out.fill_(-1.0)                      # stale output must be overwritten
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            stats = ctx.render_static(out.data_ptr())
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info()[0]
            img = out.cpu().numpy()
            ok, detail = within_render_tolerance(img, ref)
            assert ok, (call, detail)
            assert abs(stats.variance - ref_stats.variance) <= VARIANCE_REL_TOL * ref_stats.variance
            assert stats.paths == ref_stats.paths
            if call == 1:
                assert free_after == free_before, (free_before, free_after)
    finally:
        ctx.close()


def test_static_render_refuses_renders_beyond_the_arena(torch_cuda):
    torch = torch_cuda
    s = FlatScene.read(golden("cornell_c1_64.yfs"))
    s.config["render_region"] = (0, 0, 2048, 2048)   # 67M samples at 16 spp: far beyond 64 MiB
    ctx = native.Context(0)
    try:
        ctx.upload_scene(s)
        out = torch.zeros((16, 16, 3), dtype=torch.float32, device="cuda")
        with pytest.raises(native.YarError) as e:
            ctx.render_static(out.data_ptr())
        assert e.value.code == native.YAR_ERR_CAPACITY
        assert "static arena" in str(e.value)
    finally:
        ctx.close()


def test_static_render_refuses_direct_lighting(torch_cuda):
    torch = torch_cuda
    s = FlatScene.read(golden("cornell_direct_64.yfs"))
    assert int(s.config["rendering_algorithm"]) == 0
    ctx = native.Context(0)
    try:
        ctx.upload_scene(s)
        out = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
        with pytest.raises(native.YarError) as e:
            ctx.render_static(out.data_ptr())
        assert e.value.code == native.YAR_ERR_UNSUPPORTED
    finally:
        ctx.close()
