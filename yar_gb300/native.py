"""ctypes bindings of include/yar_gpu.h (the product library libyar_gb300.so).

The library is loaded from the package directory and nothing else: if it is
missing the import fails loudly (there is no CPU fallback for the hot path).
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libyar_gb300.so")

YAR_OK = 0
YAR_ERR_INVALID = -1
YAR_ERR_NOMEM = -2
YAR_ERR_CAPACITY = -3
YAR_ERR_TIMEOUT = -4
YAR_ERR_CUDA = -5
YAR_ERR_UNSUPPORTED = -6
YAR_ERR_IO = -7
YAR_ERR_NO_SCENE = -8

YAR_BUFFERS_HOST = 0
YAR_BUFFERS_DEVICE = 1

MATERIAL_PERFECT_REFLECTOR = 0
MATERIAL_PERFECT_REFRACTOR = 1
MATERIAL_DIFFUSE = 2
MATERIAL_METAL = 4
MATERIAL_PLASTIC = 5
MATERIAL_COATED_DIFFUSE = 6
MATERIAL_GLASS = 7
MATERIAL_MIX = 8
MATERIAL_PBRT3_UBER = 9
MATERIAL_PBRT3_TRANSLUCENT = 10
MATERIAL_NULL = 0xFFFFFFFF
LIGHT_POINT = 0
LIGHT_SPOT = 1
LIGHT_DIRECTIONAL = 2
LIGHT_RECT = 3
LIGHT_SPHERE = 4
LIGHT_TRIANGLE_MESH = 5
LIGHT_NULL = 0xFFFFFFFF


class KdNode(C.Structure):
    _fields_ = [("word0", C.c_uint32), ("word1", C.c_uint32)]


class KdTreeView(C.Structure):
    _fields_ = [("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("nodes", C.c_void_p), ("node_count", C.c_uint32)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p),
                ("indices", C.c_void_p), ("vertex_count", C.c_uint32), ("triangle_count", C.c_uint32),
                ("reverse_geometric_normal_orientation", C.c_int32), ("visibility", C.c_int32),
                ("kdtree", KdTreeView), ("alpha_texture", C.c_uint32)]


class ObjectDesc(C.Structure):
    _fields_ = [("mesh_index", C.c_int32), ("material_type", C.c_uint32), ("material_index", C.c_int32),
                ("area_light_type", C.c_uint32), ("area_light_index", C.c_int32),
                ("object_to_world", C.c_float * 12), ("world_to_object", C.c_float * 12),
                ("object_to_world_normal", C.c_float * 12)]


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_uint32), ("reflectance", C.c_float * 3), ("transmittance", C.c_float * 3),
                ("eta", C.c_float * 3), ("k", C.c_float * 3), ("eta_i", C.c_float),
                ("u_roughness", C.c_float), ("v_roughness", C.c_float),
                ("index_of_refraction", C.c_float), ("roughness_is_alpha", C.c_int32),
                ("specular", C.c_float * 3), ("diffuse", C.c_float * 3), ("delta_reflectance", C.c_float * 3),
                ("opacity", C.c_float * 3), ("component_count", C.c_uint32), ("components", C.c_uint32 * 5),
                ("mix_materials", C.c_int32 * 2), ("mix_amount", C.c_float * 3),
                ("reflectance_texture", C.c_uint32), ("reflectance_uv_scale", C.c_float * 2),
                ("other_textured_parameters", C.c_uint32),
                ("transmittance_texture", C.c_uint32), ("transmittance_uv_scale", C.c_float * 2),
                ("bump", C.c_uint32), ("bump_height", C.c_float), ("bump_texture", C.c_uint32),
                ("bump_uv_scale", C.c_float * 2), ("fourier_table", C.c_uint32)]


class RectLightDesc(C.Structure):
    _fields_ = [("light_to_world", C.c_float * 12), ("emitted_radiance", C.c_float * 3),
                ("size", C.c_float * 2), ("sample_count", C.c_int32)]


class CameraDesc(C.Structure):
    _fields_ = [("camera_to_world", C.c_float * 12), ("image_extent", C.c_float * 2),
                ("horz_half_dist", C.c_float), ("vert_half_dist", C.c_float), ("z_is_up", C.c_int32)]


class RenderConfig(C.Structure):
    _fields_ = [("render_region", C.c_int32 * 4), ("rendering_algorithm", C.c_int32),
                ("max_light_bounces", C.c_int32), ("russian_roulette_threshold", C.c_float),
                ("russian_roulette_bounce_count_threshold", C.c_int32), ("pixel_filter_type", C.c_int32),
                ("pixel_filter_radius", C.c_float), ("pixel_filter_alpha", C.c_float),
                ("x_pixel_sample_count", C.c_int32), ("y_pixel_sample_count", C.c_int32),
                ("film_radiance_scale", C.c_float), ("max_rgb_component_value_of_film_sample", C.c_float),
                ("pbrt3_scene", C.c_int32), ("rng_seed_offset", C.c_int32)]


class DeltaLightDesc(C.Structure):
    _fields_ = [("type", C.c_uint32), ("position", C.c_float * 3), ("direction", C.c_float * 3),
                ("intensity", C.c_float * 3), ("cone_angle", C.c_float), ("penumbra_angle", C.c_float)]


class MeshLightDesc(C.Structure):
    _fields_ = [("light_to_world", C.c_float * 12), ("emitted_radiance", C.c_float * 3),
                ("triangle_mesh_index", C.c_uint32)]


class SphereLightDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("emitted_radiance", C.c_float * 3), ("radius", C.c_float),
                ("sample_count", C.c_int32)]


class EnvironmentDesc(C.Structure):
    _fields_ = [("light_to_world", C.c_float * 12), ("world_to_light", C.c_float * 12), ("scale", C.c_float * 3),
                ("sample_count", C.c_int32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("radiance", C.c_void_p)]


class TextureDesc(C.Structure):
    _fields_ = [("first_mip", C.c_uint32), ("mip_count", C.c_uint32)]


class TextureMipDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("texel_offset", C.c_uint64)]


class FourierDesc(C.Structure):
    _fields_ = [("node_count", C.c_uint32), ("channel_count", C.c_uint32), ("max_order", C.c_uint32),
                ("eta", C.c_float), ("nodes", C.c_uint64), ("coeffs", C.c_uint64), ("coeff_count", C.c_uint64),
                ("series", C.c_uint64)]


class FlatSceneDesc(C.Structure):
    _fields_ = [("mesh_count", C.c_uint32), ("meshes", C.POINTER(MeshDesc)),
                ("object_count", C.c_uint32), ("objects", C.POINTER(ObjectDesc)),
                ("scene_kdtree", KdTreeView),
                ("material_count", C.c_uint32), ("materials", C.POINTER(MaterialDesc)),
                ("rect_light_count", C.c_uint32), ("rect_lights", C.POINTER(RectLightDesc)),
                ("other_light_count", C.c_uint32), ("camera", CameraDesc), ("config", RenderConfig),
                ("delta_light_count", C.c_uint32), ("delta_lights", C.POINTER(DeltaLightDesc)),
                ("mesh_light_count", C.c_uint32), ("mesh_lights", C.POINTER(MeshLightDesc)),
                ("sphere_light_count", C.c_uint32), ("sphere_lights", C.POINTER(SphereLightDesc)),
                ("environment", C.POINTER(EnvironmentDesc)),
                ("texture_count", C.c_uint32), ("textures", C.POINTER(TextureDesc)),
                ("texture_mip_count", C.c_uint32), ("texture_mips", C.POINTER(TextureMipDesc)),
                ("texels", C.c_void_p), ("texel_count", C.c_uint64),
                ("fourier_count", C.c_uint32), ("fourier_tables", C.POINTER(FourierDesc)),
                ("fourier_float_count", C.c_uint64), ("fourier_floats", C.c_void_p),
                ("fourier_uint_count", C.c_uint64), ("fourier_uints", C.c_void_p)]


class HitSoa(C.Structure):
    _fields_ = [("t", C.c_void_p), ("prim", C.c_void_p), ("object", C.c_void_p), ("bary", C.c_void_p)]


class BatchSceneStats(C.Structure):
    _fields_ = [("variance", C.c_double), ("completion_seconds", C.c_float), ("paths", C.c_uint64),
                ("traversal_kernel", C.c_uint32 * 2)]


class BatchStats(C.Structure):
    _fields_ = [("gpu_seconds", C.c_float), ("paths", C.c_uint64), ("rays_closest", C.c_uint64),
                ("rays_any", C.c_uint64), ("branches", C.c_uint32), ("chunk_paths", C.c_uint32),
                ("upload_seconds", C.c_float), ("tune_seconds", C.c_float), ("capture_seconds", C.c_float)]


class GuidedParams(C.Structure):
    _fields_ = [("passes", C.c_uint32), ("train_passes", C.c_uint32), ("guide_fraction", C.c_float),
                ("learning_rate", C.c_float), ("train_steps", C.c_uint32), ("stream_offset", C.c_uint32),
                ("time_budget", C.c_float), ("keep_guide", C.c_uint32), ("samples_per_pixel", C.c_uint32),
                ("guide_bounces", C.c_uint32), ("strata_x", C.c_uint32)]


class GuidedStats(C.Structure):
    _fields_ = [("passes", C.c_uint32), ("seconds", C.c_float), ("train_seconds", C.c_float),
                ("rays", C.c_uint64), ("train_samples", C.c_uint64), ("loss", C.c_float)]


class GpuOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_batch_rays", C.c_uint32), ("traversal_kernel", C.c_int32),
                ("pipeline_chunk_rays", C.c_uint32)]


GUIDE_PARAMS = 20480
GUIDE_LOBE_FLOATS = 40

TRAVERSAL_AUTO, TRAVERSAL_PERSISTENT_64, TRAVERSAL_PERSISTENT_128, TRAVERSAL_PER_RAY = 0, 1, 2, 3
TRAVERSAL_PER_RAY_VOTE = 4


class RenderStats(C.Structure):
    _fields_ = [("variance", C.c_double), ("seconds", C.c_float), ("paths", C.c_uint64),
                ("rays_closest", C.c_uint64), ("rays_any", C.c_uint64), ("kernel_launches", C.c_uint32)]


# exported symbols and their prototypes: (restype, argtypes)
EXPORTS = {
    "yar_gpu_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(GpuOptions)]),
    "yar_gpu_destroy": (None, [C.c_void_p]),
    "yar_gpu_last_error": (C.c_char_p, [C.c_void_p]),
    "yar_gpu_stream": (C.c_void_p, [C.c_void_p]),
    "yar_gpu_synchronize": (C.c_int, [C.c_void_p]),
    "yar_gpu_upload_scene": (C.c_int, [C.c_void_p, C.POINTER(FlatSceneDesc)]),
    "yar_gpu_cast_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(HitSoa), C.c_int32]),
    "yar_gpu_cast_any": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]),
    "yar_gpu_cast_closest_timed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(HitSoa),
                                             C.POINTER(C.c_float)]),
    "yar_gpu_cast_any_timed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_float)]),
    "yar_gpu_render": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderStats)]),
    "yar_gpu_render_static": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderStats)]),
    "yar_gpu_render_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_void_p, C.POINTER(RenderStats)]),
    "yar_gpu_traversal_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32)]),
    "yar_gpu_render_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                       C.POINTER(BatchSceneStats), C.POINTER(BatchStats)]),
    "yar_gpu_guided_render": (C.c_int, [C.c_void_p, C.POINTER(GuidedParams), C.c_void_p, C.c_void_p,
                                        C.POINTER(GuidedStats)]),
    "yar_guide_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "yar_guide_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "yar_guide_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.c_void_p]),
    "yar_gpu_wait_selftest": (C.c_int, [C.c_void_p, C.c_uint32]),
    "yar_guide_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.c_float,
                                     C.c_void_p, C.POINTER(C.c_float)]),
    "yar_guide_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.c_float,
                                       C.c_float, C.POINTER(C.c_float)]),
    "yar_build_mesh_kdtree": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int32,
                                        C.POINTER(C.c_float), C.POINTER(C.c_void_p), C.POINTER(C.c_uint32)]),
    "yar_build_scene_kdtree": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_void_p),
                                         C.POINTER(C.c_uint32)]),
    "yar_free_nodes": (None, [C.c_void_p]),
    "yar_read_kdtree_cache": (C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_uint64),
                                        C.POINTER(C.c_void_p), C.POINTER(C.c_uint32)]),
    "yar_write_kdtree_cache": (C.c_int, [C.c_char_p, C.POINTER(C.c_float), C.c_uint64, C.c_void_p, C.c_uint32]),
    "yar_transform_bounds": (None, [C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


def lib():
    """Load libyar_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libyar_gb300.so is not built: run `python -c \"import __graft_entry__ as g; "
                              "g.build()\"` (path %s)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class YarError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("yar_gpu error %d: %s" % (code, message))
        self.code = code


def _ptr(a):
    return None if a is None else a.ctypes.data


def build_mesh_kdtree(vertices, indices, threads=0):
    """Reference kd-tree for a triangle mesh: returns (bounds[6] f32, nodes (N,2) u32)."""
    v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
    i = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 3)
    bounds = (C.c_float * 6)()
    nodes = C.c_void_p()
    count = C.c_uint32()
    rc = lib().yar_build_mesh_kdtree(_ptr(v), v.shape[0], _ptr(i), i.shape[0], int(threads or os.cpu_count() or 1),
                                     bounds, C.byref(nodes), C.byref(count))
    if rc != YAR_OK:
        raise YarError(rc, "yar_build_mesh_kdtree")
    out = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(count.value * 2,)).copy()
    lib().yar_free_nodes(nodes)
    return np.array(bounds, dtype=np.float32), out.reshape(-1, 2)


def build_scene_kdtree(object_bounds):
    """Reference scene kd-tree over per-object world bounds (M,6)."""
    b = np.ascontiguousarray(object_bounds, dtype=np.float32).reshape(-1, 6)
    bounds = (C.c_float * 6)()
    nodes = C.c_void_p()
    count = C.c_uint32()
    rc = lib().yar_build_scene_kdtree(_ptr(b), b.shape[0], bounds, C.byref(nodes), C.byref(count))
    if rc != YAR_OK:
        raise YarError(rc, "yar_build_scene_kdtree")
    out = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(count.value * 2,)).copy()
    lib().yar_free_nodes(nodes)
    return np.array(bounds, dtype=np.float32), out.reshape(-1, 2)


def read_kdtree_cache(path):
    """A kd-tree cache file in the reference's format: (bounds (6,), nodes (N, 2) uint32, hash)."""
    bounds = (C.c_float * 6)()
    h = C.c_uint64()
    nodes = C.c_void_p()
    count = C.c_uint32()
    rc = lib().yar_read_kdtree_cache(os.fsencode(path), bounds, C.byref(h), C.byref(nodes), C.byref(count))
    if rc != YAR_OK:
        raise YarError(rc, "yar_read_kdtree_cache(%s)" % path)
    out = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(count.value * 2,)).copy()
    lib().yar_free_nodes(nodes)
    return np.array(bounds, dtype=np.float32), out.reshape(-1, 2), int(h.value)


def write_kdtree_cache(path, bounds, nodes, hash_value=0):
    b = (C.c_float * 6)(*[float(x) for x in np.asarray(bounds, np.float32).reshape(6)])
    n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 2)
    rc = lib().yar_write_kdtree_cache(os.fsencode(path), b, int(hash_value), _ptr(n), n.shape[0])
    if rc != YAR_OK:
        raise YarError(rc, "yar_write_kdtree_cache(%s)" % path)


def transform_bounds(object_to_world, bounds):
    m = np.ascontiguousarray(object_to_world, dtype=np.float32).reshape(12)
    b = np.ascontiguousarray(bounds, dtype=np.float32).reshape(6)
    out = np.zeros(6, dtype=np.float32)
    lib().yar_transform_bounds(_ptr(m), _ptr(b), _ptr(out))
    return out


class Context:
    """A yar_gpu_ctx: one CUDA device, one stream, one uploaded scene."""

    def __init__(self, device=0, max_batch_rays=0, traversal_kernel=TRAVERSAL_AUTO, pipeline_chunk_rays=0):
        L = lib()
        h = C.c_void_p()
        opts = GpuOptions(int(device), int(max_batch_rays), int(traversal_kernel), int(pipeline_chunk_rays))
        rc = L.yar_gpu_create(C.byref(h), C.byref(opts))
        if rc != YAR_OK:
            raise YarError(rc, "yar_gpu_create (is a CUDA device visible?)")
        self._h = h
        self._scene_keepalive = None

    def close(self):
        if self._h:
            lib().yar_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != YAR_OK:
            msg = lib().yar_gpu_last_error(self._h)
            raise YarError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    @property
    def stream(self):
        return lib().yar_gpu_stream(self._h)

    def synchronize(self):
        self._check(lib().yar_gpu_synchronize(self._h), "synchronize")

    def upload_scene(self, flat):
        desc, keep = flat.to_c()
        self._check(lib().yar_gpu_upload_scene(self._h, C.byref(desc)), "upload_scene")
        self._scene_keepalive = (desc, keep)

    # host-buffer casts (copies inside the call)
    def cast_closest(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        t = np.empty(n, np.float32)
        prim = np.empty(n, np.uint32)
        obj = np.empty(n, np.uint32)
        bary = np.empty((n, 2), np.float32)
        hits = HitSoa(_ptr(t), _ptr(prim), _ptr(obj), _ptr(bary))
        self._check(lib().yar_gpu_cast_closest(self._h, _ptr(rays), n, C.byref(hits), YAR_BUFFERS_HOST),
                    "cast_closest")
        return t, prim, obj, bary

    def cast_any(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        self._check(lib().yar_gpu_cast_any(self._h, _ptr(rays), n, _ptr(occ), YAR_BUFFERS_HOST), "cast_any")
        return occ

    # device-buffer casts: arguments are raw device pointers (e.g. torch data_ptr())
    def cast_closest_device(self, rays_ptr, n, t_ptr, prim_ptr, obj_ptr, bary_ptr=None, timed=False):
        hits = HitSoa(t_ptr, prim_ptr, obj_ptr, bary_ptr)
        if timed:
            ms = C.c_float()
            self._check(lib().yar_gpu_cast_closest_timed(self._h, rays_ptr, n, C.byref(hits), C.byref(ms)),
                        "cast_closest_timed")
            return ms.value
        self._check(lib().yar_gpu_cast_closest(self._h, rays_ptr, n, C.byref(hits), YAR_BUFFERS_DEVICE),
                    "cast_closest")
        return None

    def cast_any_device(self, rays_ptr, n, occ_ptr, timed=False):
        if timed:
            ms = C.c_float()
            self._check(lib().yar_gpu_cast_any_timed(self._h, rays_ptr, n, occ_ptr, C.byref(ms)), "cast_any_timed")
            return ms.value
        self._check(lib().yar_gpu_cast_any(self._h, rays_ptr, n, occ_ptr, YAR_BUFFERS_DEVICE), "cast_any")
        return None

    def render(self, width, height):
        rgb = np.zeros((height, width, 3), np.float32)
        stats = RenderStats()
        self._check(lib().yar_gpu_render(self._h, _ptr(rgb), C.byref(stats)), "render")
        return rgb, stats

    def render_checkpoint(self, width, height, directory, input_filename):
        """yar_gpu_render_checkpoint: render_scene with a checkpoint directory in the
        reference's format (resumes from the tiles already there)."""
        rgb = np.zeros((height, width, 3), np.float32)
        stats = RenderStats()
        self._check(lib().yar_gpu_render_checkpoint(self._h, str(directory).encode(), str(input_filename).encode(),
                                                     _ptr(rgb), C.byref(stats)), "render_checkpoint")
        return rgb, stats

    def traversal_kernels(self):
        """The traversal kernels chosen so far: {"cast": [closest, any], "render_closest": [per bounce],
        "render_any": [per bounce]} as TRAVERSAL_* codes (0 = not chosen yet)."""
        c, rc, ra = (C.c_int32 * 2)(), (C.c_int32 * 5)(), (C.c_int32 * 5)()
        self._check(lib().yar_gpu_traversal_kernels(self._h, c, rc, ra), "traversal_kernels")
        return {"cast": list(c), "render_closest": list(rc), "render_any": list(ra)}

    def render_batch(self, flats):
        """yar_gpu_render_batch: returns ([images], [BatchSceneStats], BatchStats)."""
        descs = [f.to_c() for f in flats]
        arr = (C.c_void_p * len(flats))(*[C.cast(C.byref(d), C.c_void_p) for d, _ in descs])
        imgs = []
        for f in flats:
            r = f.config["render_region"]
            imgs.append(np.zeros((int(r[3] - r[1]), int(r[2] - r[0]), 3), np.float32))
        outs = (C.c_void_p * len(flats))(*[_ptr(i) for i in imgs])
        sst = (BatchSceneStats * len(flats))()
        st = BatchStats()
        self._check(lib().yar_gpu_render_batch(self._h, arr, len(flats), outs, sst, C.byref(st)), "render_batch")
        return imgs, list(sst), st

    def guided_render(self, width, height, passes=0, guide_fraction=0.0, train_passes=0, learning_rate=2e-3,
                      train_steps=8, stream_offset=0, time_budget=0.0, keep_guide=False, samples_per_pixel=0,
                      guide_bounces=0, strata_x=0):
        """yar_gpu_guided_render: returns (mean image, per-pixel FP64 radiance
        sums, GuidedStats).  samples_per_pixel > 0: the stratified form (the
        training passes, then the pixel sampler at that many samples, in
        strata_x columns of strata when given)."""
        prm = GuidedParams(int(passes), int(train_passes), float(guide_fraction), float(learning_rate),
                           int(train_steps), int(stream_offset), float(time_budget), int(bool(keep_guide)),
                           int(samples_per_pixel), int(guide_bounces), int(strata_x))
        sums = np.zeros((height, width, 3), np.float64)
        rgb = np.zeros((height, width, 3), np.float32)
        st = GuidedStats()
        self._check(lib().yar_gpu_guided_render(self._h, C.byref(prm), _ptr(sums), _ptr(rgb), C.byref(st)),
                    "guided_render")
        return rgb, sums, st

    # ---- learned proposal network (device buffers are raw pointers)
    def guide_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == GUIDE_PARAMS
        self._check(lib().yar_guide_set_params(self._h, _ptr(p)), "guide_set_params")

    def guide_get_params(self):
        p = np.zeros(GUIDE_PARAMS, np.float32)
        self._check(lib().yar_guide_get_params(self._h, _ptr(p)), "guide_get_params")
        return p

    def wait_selftest(self, limit):
        """yar_gpu_wait_selftest: the tensor-core kernels' bounded mbarrier wait
        on a barrier nothing arrives at; raises YarError(YAR_ERR_TIMEOUT)."""
        self._check(lib().yar_gpu_wait_selftest(self._h, int(limit)), "wait_selftest")

    def guide_infer(self, queries_ptr, n, box, lobes_ptr):
        b = (C.c_float * 6)(*[float(x) for x in box])
        self._check(lib().yar_guide_infer(self._h, queries_ptr, n, b, lobes_ptr), "guide_infer")

    def guide_gradient(self, samples_ptr, n, box, weight_scale, grad_ptr):
        b = (C.c_float * 6)(*[float(x) for x in box])
        loss = C.c_float()
        self._check(lib().yar_guide_gradient(self._h, samples_ptr, n, b, float(weight_scale), grad_ptr,
                                             C.byref(loss)), "guide_gradient")
        return loss.value

    def guide_train_step(self, samples_ptr, n, box, weight_scale, learning_rate):
        b = (C.c_float * 6)(*[float(x) for x in box])
        loss = C.c_float()
        self._check(lib().yar_guide_train_step(self._h, samples_ptr, n, b, float(weight_scale),
                                               float(learning_rate), C.byref(loss)), "guide_train_step")
        return loss.value

    def render_static(self, rgb_device_ptr):
        """yar_gpu_render_static: renders into caller-owned device memory
        without allocating (working memory comes from the library's static
        device arena)."""
        stats = RenderStats()
        self._check(lib().yar_gpu_render_static(self._h, rgb_device_ptr, C.byref(stats)), "render_static")
        return stats
