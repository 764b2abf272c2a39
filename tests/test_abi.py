"""The C-ABI library loads and exports every symbol include/yar_gpu.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "yar_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|void\*)\s+\**(yar_\w+)\s*\(", text, re.M)))


def test_header_declares_the_reference_seams():
    names = declared_functions()
    for required in ["yar_gpu_create", "yar_gpu_destroy", "yar_gpu_last_error", "yar_gpu_upload_scene",
                     "yar_gpu_cast_closest", "yar_gpu_cast_any", "yar_gpu_render", "yar_build_mesh_kdtree",
                     "yar_build_scene_kdtree"]:
        assert required in names


def test_library_exports_every_declared_symbol():
    from yar_gb300 import native
    lib = ctypes.CDLL(native.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding table covers all of them
    assert set(declared_functions()) <= set(native.EXPORTS)


def test_context_creation_fails_cleanly_without_a_device():
    import pytest
    from conftest import cuda_available
    from yar_gb300 import native
    if cuda_available():
        pytest.skip("a device is present")
    with pytest.raises(native.YarError):
        native.Context(0)


def test_struct_sizes_match_the_header():
    from yar_gb300 import native
    assert ctypes.sizeof(native.KdNode) == 8
    assert ctypes.sizeof(native.ObjectDesc) == 164
    assert ctypes.sizeof(native.MaterialDesc) == 216
    assert ctypes.sizeof(native.RectLightDesc) == 72


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler gives
    the header's structs."""
    import shutil
    import subprocess
    from yar_gb300 import native
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    mirrors = {"yar_material_desc": native.MaterialDesc, "yar_object_desc": native.ObjectDesc,
               "yar_rect_light_desc": native.RectLightDesc, "yar_delta_light_desc": native.DeltaLightDesc,
               "yar_mesh_light_desc": native.MeshLightDesc, "yar_sphere_light_desc": native.SphereLightDesc,
               "yar_camera_desc": native.CameraDesc, "yar_render_config": native.RenderConfig,
               "yar_flat_scene": native.FlatSceneDesc, "yar_texture_desc": native.TextureDesc,
               "yar_texture_mip_desc": native.TextureMipDesc, "yar_gpu_options": native.GpuOptions,
               "yar_hit_soa": native.HitSoa, "yar_fourier_desc": native.FourierDesc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "yar_gpu.h"', "int main(void) {"]
    for name, cls in mirrors.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for field, _ in cls._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, field, name, field))
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.split("\n") if l)
    for name, cls in mirrors.items():
        assert int(out[name]) == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert int(out[name + "." + field]) == getattr(cls, field).offset, (name, field)
