import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    # The native product library and the oracle are built in-tree on first
    # use (both builds are incremental and take seconds).
    from yar_gb300 import build
    build.build_product()
    build.build_oracle()


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    if not cuda_available():
        pytest.skip("no CUDA device")
    from yar_gb300 import native
    ctx = native.Context(0)
    yield ctx
    ctx.close()


def golden(name):
    return os.path.join(GOLDEN, name)


def constant_bumps_with_delta_materials():
    """cornell_bump_64 without image textures (the flat scene keeps none), its
    boxes a mirror and smooth glass with a constant bump height: delta events
    about the bumped normal."""
    import numpy as np
    from yar_gb300 import native
    from yar_gb300.scene import FlatScene
    s = FlatScene.read(golden("cornell_bump_64.yfs"))
    m = s.materials
    m["reflectance_texture"][:] = 0
    m["transmittance_texture"][:] = 0
    m["bump"][m["bump"] == 2] = 0
    for obj, kind in ((5, native.MATERIAL_PERFECT_REFLECTOR), (6, native.MATERIAL_GLASS)):
        k = int(s.objects["material_index"][obj])
        m["type"][k] = kind
        m["reflectance"][k] = (0.9, 0.85, 0.8)
        m["transmittance"][k] = (0.95, 0.95, 0.9)
        m["index_of_refraction"][k] = 1.5
        m["u_roughness"][k] = m["v_roughness"][k] = 0.0
        m["bump"][k] = 1
        m["bump_height"][k] = 0.03
        s.objects["material_type"][s.objects["material_index"] == k] = kind
    s.textures = s.textures[:0]
    s.texture_mips = s.texture_mips[:0]
    s.texels = s.texels[:0]
    return s
