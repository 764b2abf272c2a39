"""yar_gb300 - GB300-native (sm_103a) path-tracing hot path of kennyalive/YAR.

native  - ctypes bindings of the C ABI (include/yar_gpu.h)
scene   - flat scenes (meshes, kd-trees, objects, materials, lights, camera)
scenes  - seeded synthetic workloads
"""
from . import native, scene, scenes  # noqa: F401

__all__ = ["native", "scene", "scenes"]
