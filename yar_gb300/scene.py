"""Flat scenes: the host-side form of yar_flat_scene (include/yar_gpu.h).

A FlatScene holds numpy arrays for meshes (with their kd-trees), scene
objects, the scene kd-tree, constant materials, rectangular lights, the
camera and the Raytracer_Config fields.  It reads and writes the flat scene
file (yar_gb300/csrc/yfs.hpp) and builds the ctypes descriptor passed to
yar_gpu_upload_scene.
"""
import ctypes as C
import struct

import numpy as np

from . import native

OBJECT_DTYPE = np.dtype([("mesh_index", "<i4"), ("material_type", "<u4"), ("material_index", "<i4"),
                         ("area_light_type", "<u4"), ("area_light_index", "<i4"),
                         ("object_to_world", "<f4", 12), ("world_to_object", "<f4", 12),
                         ("object_to_world_normal", "<f4", 12)])
MATERIAL_DTYPE = np.dtype([("type", "<u4"), ("reflectance", "<f4", 3), ("transmittance", "<f4", 3),
                           ("eta", "<f4", 3), ("k", "<f4", 3), ("eta_i", "<f4"), ("u_roughness", "<f4"),
                           ("v_roughness", "<f4"), ("index_of_refraction", "<f4"), ("roughness_is_alpha", "<i4"),
                           ("specular", "<f4", 3), ("diffuse", "<f4", 3), ("delta_reflectance", "<f4", 3),
                           ("opacity", "<f4", 3), ("component_count", "<u4"), ("components", "<u4", 5),
                           ("mix_materials", "<i4", 2), ("mix_amount", "<f4", 3),
                           ("reflectance_texture", "<u4"), ("reflectance_uv_scale", "<f4", 2),
                           ("other_textured_parameters", "<u4"),
                           ("transmittance_texture", "<u4"), ("transmittance_uv_scale", "<f4", 2),
                           ("bump", "<u4"), ("bump_height", "<f4"), ("bump_texture", "<u4"),
                           ("bump_uv_scale", "<f4", 2), ("fourier_table", "<u4")])
MATERIAL_RECORD_V1 = 72  # the MATS chunk's records: the fields up to roughness_is_alpha
LIGHT_DTYPE = np.dtype([("light_to_world", "<f4", 12), ("emitted_radiance", "<f4", 3), ("size", "<f4", 2),
                        ("sample_count", "<i4")])
DELTA_LIGHT_DTYPE = np.dtype([("type", "<u4"), ("position", "<f4", 3), ("direction", "<f4", 3),
                              ("intensity", "<f4", 3), ("cone_angle", "<f4"), ("penumbra_angle", "<f4")])
MESH_LIGHT_DTYPE = np.dtype([("light_to_world", "<f4", 12), ("emitted_radiance", "<f4", 3),
                             ("triangle_mesh_index", "<u4")])
SPHERE_LIGHT_DTYPE = np.dtype([("position", "<f4", 3), ("emitted_radiance", "<f4", 3), ("radius", "<f4"),
                               ("sample_count", "<i4")])
ENVIRONMENT_DTYPE = np.dtype([("light_to_world", "<f4", 12), ("world_to_light", "<f4", 12), ("scale", "<f4", 3),
                              ("sample_count", "<i4"), ("width", "<u4"), ("height", "<u4"), ("radiance", "<u8")])
TEXTURE_DTYPE = np.dtype([("first_mip", "<u4"), ("mip_count", "<u4")])
TEXTURE_MIP_DTYPE = np.dtype([("width", "<u4"), ("height", "<u4"), ("texel_offset", "<u8")])
FOURIER_DTYPE = np.dtype([("node_count", "<u4"), ("channel_count", "<u4"), ("max_order", "<u4"), ("eta", "<f4"),
                          ("nodes", "<u8"), ("coeffs", "<u8"), ("coeff_count", "<u8"), ("series", "<u8")])
CAMERA_DTYPE = np.dtype([("camera_to_world", "<f4", 12), ("image_extent", "<f4", 2), ("horz_half_dist", "<f4"),
                         ("vert_half_dist", "<f4"), ("z_is_up", "<i4")])
CONFIG_DTYPE = np.dtype([("render_region", "<i4", 4), ("rendering_algorithm", "<i4"), ("max_light_bounces", "<i4"),
                         ("russian_roulette_threshold", "<f4"), ("russian_roulette_bounce_count_threshold", "<i4"),
                         ("pixel_filter_type", "<i4"), ("pixel_filter_radius", "<f4"),
                         ("pixel_filter_alpha", "<f4"), ("x_pixel_sample_count", "<i4"),
                         ("y_pixel_sample_count", "<i4"), ("film_radiance_scale", "<f4"),
                         ("max_rgb_component_value_of_film_sample", "<f4"), ("pbrt3_scene", "<i4"),
                         ("rng_seed_offset", "<i4")])

assert OBJECT_DTYPE.itemsize == C.sizeof(native.ObjectDesc)
assert MATERIAL_DTYPE.itemsize == C.sizeof(native.MaterialDesc)
assert LIGHT_DTYPE.itemsize == C.sizeof(native.RectLightDesc)
assert DELTA_LIGHT_DTYPE.itemsize == C.sizeof(native.DeltaLightDesc)
assert MESH_LIGHT_DTYPE.itemsize == C.sizeof(native.MeshLightDesc)
assert ENVIRONMENT_DTYPE.itemsize == C.sizeof(native.EnvironmentDesc)
assert SPHERE_LIGHT_DTYPE.itemsize == C.sizeof(native.SphereLightDesc)
assert CAMERA_DTYPE.itemsize == C.sizeof(native.CameraDesc)
assert TEXTURE_DTYPE.itemsize == C.sizeof(native.TextureDesc)
assert TEXTURE_MIP_DTYPE.itemsize == C.sizeof(native.TextureMipDesc)
assert FOURIER_DTYPE.itemsize == C.sizeof(native.FourierDesc)
assert CONFIG_DTYPE.itemsize == C.sizeof(native.RenderConfig)

IDENTITY = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)


class Mesh:
    def __init__(self, vertices, indices, normals=None, uvs=None, reverse_orientation=0, visibility=0,
                 bounds=None, nodes=None, alpha_texture=0):
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, np.int32).reshape(-1, 3)
        self.normals = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        self.uvs = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
        self.reverse_orientation = int(reverse_orientation)
        self.visibility = int(visibility)
        self.bounds = np.zeros(6, np.float32) if bounds is None else np.asarray(bounds, np.float32)
        self.nodes = np.zeros((0, 2), np.uint32) if nodes is None else np.ascontiguousarray(nodes, np.uint32)
        self.alpha_texture = int(alpha_texture)  # 0 none, else 1 + texture index (alpha test)

    @property
    def triangle_count(self):
        return self.indices.shape[0]


def default_config(width=256, height=256, spp_x=1, spp_y=1, max_bounces=32, seed_offset=0):
    c = np.zeros((), CONFIG_DTYPE)
    c["render_region"] = (0, 0, width, height)
    c["rendering_algorithm"] = 1
    c["max_light_bounces"] = max_bounces
    c["russian_roulette_threshold"] = 1.0
    c["russian_roulette_bounce_count_threshold"] = 3
    c["pixel_filter_type"] = 0
    c["pixel_filter_radius"] = 0.5
    c["pixel_filter_alpha"] = 2.0
    c["x_pixel_sample_count"] = spp_x
    c["y_pixel_sample_count"] = spp_y
    c["film_radiance_scale"] = 1.0
    c["max_rgb_component_value_of_film_sample"] = np.inf
    c["pbrt3_scene"] = 1
    c["rng_seed_offset"] = seed_offset
    return c


class FlatScene:
    def __init__(self):
        self.meshes = []
        self.objects = np.zeros(0, OBJECT_DTYPE)
        self.scene_bounds = np.zeros(6, np.float32)
        self.scene_nodes = np.zeros((0, 2), np.uint32)
        self.materials = np.zeros(0, MATERIAL_DTYPE)
        self.rect_lights = np.zeros(0, LIGHT_DTYPE)
        # point, spot and directional lights, in that order
        self.delta_lights = np.zeros(0, DELTA_LIGHT_DTYPE)
        self.mesh_lights = np.zeros(0, MESH_LIGHT_DTYPE)  # triangle-mesh lights
        self.sphere_lights = np.zeros(0, SPHERE_LIGHT_DTYPE)
        # environment light: None, or (ENVIRONMENT_DTYPE record, (height, width, 3) float32 map)
        self.environment = None
        # image textures: records, their mips (level 0 first) and every mip's RGB texels
        self.textures = np.zeros(0, TEXTURE_DTYPE)
        self.texture_mips = np.zeros(0, TEXTURE_MIP_DTYPE)
        self.texels = np.zeros((0, 3), np.float32)
        # pbrt3 fourier BSDF tables: records and the floats / uints they index
        self.fourier_tables = np.zeros(0, FOURIER_DTYPE)
        self.fourier_floats = np.zeros(0, np.float32)
        self.fourier_uints = np.zeros(0, np.uint32)
        self.other_light_count = 0
        self.camera = np.zeros((), CAMERA_DTYPE)
        self.config = default_config()

    @property
    def triangle_count(self):
        return sum(m.triangle_count for m in self.meshes)

    # ---- kd-trees (the reference builder, run by the product library) ----
    def build_kdtrees(self, threads=0):
        """Per-mesh trees on a thread pool (the C builder releases the GIL),
        largest meshes first, then the scene tree over the objects."""
        import os
        from concurrent.futures import ThreadPoolExecutor
        threads = int(threads or os.cpu_count() or 1)
        order = sorted(range(len(self.meshes)), key=lambda k: -self.meshes[k].triangle_count)

        def one(k):
            m = self.meshes[k]
            m.bounds, m.nodes = native.build_mesh_kdtree(m.vertices, m.indices, threads)

        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(one, order))
        self.build_scene_kdtree()
        return self

    # ---- kd-tree cache files (the reference's KdTree::save format) ----
    def write_kdtree_caches(self, directory):
        """mesh_<i>.kdtree per mesh and scene.kdtree, loadable by the reference."""
        import os
        os.makedirs(directory, exist_ok=True)
        for i, m in enumerate(self.meshes):
            native.write_kdtree_cache(os.path.join(directory, "mesh_%d.kdtree" % i), m.bounds, m.nodes)
        native.write_kdtree_cache(os.path.join(directory, "scene.kdtree"), self.scene_bounds, self.scene_nodes)

    def read_kdtree_caches(self, directory):
        """Trees from cache files (written by write_kdtree_caches or by the
        reference) instead of building them.  The reference's files carry no
        real geometry hash, so a cache must belong to the same meshes."""
        import os
        for i, m in enumerate(self.meshes):
            m.bounds, m.nodes, _ = native.read_kdtree_cache(os.path.join(directory, "mesh_%d.kdtree" % i))
        self.scene_bounds, self.scene_nodes, _ = native.read_kdtree_cache(os.path.join(directory, "scene.kdtree"))
        return self

    def build_scene_kdtree(self):
        ob = np.stack([native.transform_bounds(o["object_to_world"], self.meshes[o["mesh_index"]].bounds)
                       for o in self.objects])
        self.scene_bounds, self.scene_nodes = native.build_scene_kdtree(ob)
        return self

    # ---- ctypes descriptor ----
    def to_c(self):
        keep = []
        meshes = (native.MeshDesc * len(self.meshes))()
        for i, m in enumerate(self.meshes):
            d = meshes[i]
            d.vertices = m.vertices.ctypes.data
            d.normals = m.normals.ctypes.data if m.normals is not None else None
            d.uvs = m.uvs.ctypes.data if m.uvs is not None else None
            d.indices = m.indices.ctypes.data
            d.vertex_count = m.vertices.shape[0]
            d.triangle_count = m.indices.shape[0]
            d.reverse_geometric_normal_orientation = m.reverse_orientation
            d.visibility = m.visibility
            d.kdtree.bounds_min[:] = [float(x) for x in m.bounds[:3]]
            d.kdtree.bounds_max[:] = [float(x) for x in m.bounds[3:]]
            nodes = np.ascontiguousarray(m.nodes, np.uint32)
            keep.append(nodes)
            d.kdtree.nodes = nodes.ctypes.data if nodes.size else None
            d.kdtree.node_count = nodes.shape[0]
            d.alpha_texture = m.alpha_texture
            keep.append(m)
        objects = np.ascontiguousarray(self.objects)
        materials = np.ascontiguousarray(self.materials)
        lights = np.ascontiguousarray(self.rect_lights)
        dlights = np.ascontiguousarray(self.delta_lights)
        mlights = np.ascontiguousarray(self.mesh_lights)
        slights = np.ascontiguousarray(self.sphere_lights)
        snodes = np.ascontiguousarray(self.scene_nodes, np.uint32)
        keep += [objects, materials, lights, dlights, mlights, slights, snodes, meshes]
        s = native.FlatSceneDesc()
        s.mesh_count = len(self.meshes)
        s.meshes = meshes
        s.object_count = objects.shape[0]
        s.objects = C.cast(objects.ctypes.data, C.POINTER(native.ObjectDesc)) if objects.size else None
        s.scene_kdtree.bounds_min[:] = [float(x) for x in self.scene_bounds[:3]]
        s.scene_kdtree.bounds_max[:] = [float(x) for x in self.scene_bounds[3:]]
        s.scene_kdtree.nodes = snodes.ctypes.data if snodes.size else None
        s.scene_kdtree.node_count = snodes.shape[0]
        s.material_count = materials.shape[0]
        s.materials = C.cast(materials.ctypes.data, C.POINTER(native.MaterialDesc)) if materials.size else None
        s.rect_light_count = lights.shape[0]
        s.rect_lights = C.cast(lights.ctypes.data, C.POINTER(native.RectLightDesc)) if lights.size else None
        s.other_light_count = int(self.other_light_count)
        s.delta_light_count = dlights.shape[0]
        s.delta_lights = C.cast(dlights.ctypes.data, C.POINTER(native.DeltaLightDesc)) if dlights.size else None
        s.mesh_light_count = mlights.shape[0]
        s.mesh_lights = C.cast(mlights.ctypes.data, C.POINTER(native.MeshLightDesc)) if mlights.size else None
        s.sphere_light_count = slights.shape[0]
        s.sphere_lights = C.cast(slights.ctypes.data, C.POINTER(native.SphereLightDesc)) if slights.size else None
        if self.environment is not None:
            rec, img = self.environment
            img = np.ascontiguousarray(img, np.float32)
            env = native.EnvironmentDesc()
            env.light_to_world[:] = [float(x) for x in rec["light_to_world"]]
            env.world_to_light[:] = [float(x) for x in rec["world_to_light"]]
            env.scale[:] = [float(x) for x in rec["scale"]]
            env.sample_count = int(rec["sample_count"])
            env.height, env.width = img.shape[0], img.shape[1]
            env.radiance = img.ctypes.data
            keep += [img, env]
            s.environment = C.pointer(env)
        if self.textures.shape[0]:
            tex = np.ascontiguousarray(self.textures, TEXTURE_DTYPE)
            mips = np.ascontiguousarray(self.texture_mips, TEXTURE_MIP_DTYPE)
            texels = np.ascontiguousarray(self.texels, np.float32)
            keep += [tex, mips, texels]
            s.texture_count = tex.shape[0]
            s.textures = C.cast(tex.ctypes.data, C.POINTER(native.TextureDesc))
            s.texture_mip_count = mips.shape[0]
            s.texture_mips = C.cast(mips.ctypes.data, C.POINTER(native.TextureMipDesc))
            s.texels = texels.ctypes.data
            s.texel_count = texels.shape[0]
        if self.fourier_tables.shape[0]:
            ft = np.ascontiguousarray(self.fourier_tables, FOURIER_DTYPE)
            ff = np.ascontiguousarray(self.fourier_floats, np.float32)
            fu = np.ascontiguousarray(self.fourier_uints, np.uint32)
            keep += [ft, ff, fu]
            s.fourier_count = ft.shape[0]
            s.fourier_tables = C.cast(ft.ctypes.data, C.POINTER(native.FourierDesc))
            s.fourier_float_count = ff.shape[0]
            s.fourier_floats = ff.ctypes.data
            s.fourier_uint_count = fu.shape[0]
            s.fourier_uints = fu.ctypes.data
        C.memmove(C.byref(s.camera), np.ascontiguousarray(self.camera).ctypes.data, CAMERA_DTYPE.itemsize)
        C.memmove(C.byref(s.config), np.ascontiguousarray(self.config).ctypes.data, CONFIG_DTYPE.itemsize)
        return s, keep

    # ---- file I/O (yar_gb300/csrc/yfs.hpp) ----
    def write(self, path):
        def chunk(tag, payload):
            return tag + struct.pack("<IQ", 0, len(payload)) + payload

        parts = [b"YFS1", struct.pack("<I", 1)]
        parts.append(chunk(b"CONF", self.config.tobytes() + self.camera.tobytes() +
                           struct.pack("<I", int(self.other_light_count))))
        for m in self.meshes:
            flags = (1 if m.normals is not None else 0) | (2 if m.uvs is not None else 0) | (4 if m.alpha_texture else 0)
            p = struct.pack("<6I", m.vertices.shape[0], m.indices.shape[0], flags, m.reverse_orientation & 0xffffffff,
                            m.visibility, m.nodes.shape[0])
            p += m.bounds.astype(np.float32).tobytes() + m.vertices.tobytes() + m.indices.tobytes()
            if m.normals is not None:
                p += m.normals.tobytes()
            if m.uvs is not None:
                p += m.uvs.tobytes()
            p += np.ascontiguousarray(m.nodes, np.uint32).tobytes()
            if m.alpha_texture:
                p += struct.pack("<I", m.alpha_texture)
            parts.append(chunk(b"MESH", p))
        parts.append(chunk(b"OBJS", struct.pack("<I", self.objects.shape[0]) + self.objects.tobytes()))
        parts.append(chunk(b"SKDT", self.scene_bounds.astype(np.float32).tobytes() +
                           struct.pack("<I", self.scene_nodes.shape[0]) +
                           np.ascontiguousarray(self.scene_nodes, np.uint32).tobytes()))
        parts.append(chunk(b"MAT2", struct.pack("<II", self.materials.shape[0], MATERIAL_DTYPE.itemsize) +
                           np.ascontiguousarray(self.materials, MATERIAL_DTYPE).tobytes()))
        parts.append(chunk(b"RLIT", struct.pack("<I", self.rect_lights.shape[0]) + self.rect_lights.tobytes()))
        if self.delta_lights.shape[0]:
            parts.append(chunk(b"DLIT", struct.pack("<I", self.delta_lights.shape[0]) + self.delta_lights.tobytes()))
        if self.mesh_lights.shape[0]:
            parts.append(chunk(b"MLIT", struct.pack("<I", self.mesh_lights.shape[0]) + self.mesh_lights.tobytes()))
        if self.sphere_lights.shape[0]:
            parts.append(chunk(b"SPHL", struct.pack("<I", self.sphere_lights.shape[0]) + self.sphere_lights.tobytes()))
        if self.environment is not None:
            rec, img = self.environment
            r = np.array(rec, ENVIRONMENT_DTYPE).copy()
            r["height"], r["width"] = img.shape[0], img.shape[1]
            r["radiance"] = 0
            parts.append(chunk(b"ENVM", r.tobytes() + np.ascontiguousarray(img, np.float32).tobytes()))
        if self.textures.shape[0]:
            parts.append(chunk(b"TEXS", struct.pack("<IIQ", self.textures.shape[0], self.texture_mips.shape[0],
                                                    self.texels.shape[0]) +
                               np.ascontiguousarray(self.textures, TEXTURE_DTYPE).tobytes() +
                               np.ascontiguousarray(self.texture_mips, TEXTURE_MIP_DTYPE).tobytes() +
                               np.ascontiguousarray(self.texels, np.float32).tobytes()))
        if self.fourier_tables.shape[0]:
            parts.append(chunk(b"FOUR", struct.pack("<IQQ", self.fourier_tables.shape[0], self.fourier_floats.shape[0],
                                                    self.fourier_uints.shape[0]) +
                               np.ascontiguousarray(self.fourier_tables, FOURIER_DTYPE).tobytes() +
                               np.ascontiguousarray(self.fourier_floats, np.float32).tobytes() +
                               np.ascontiguousarray(self.fourier_uints, np.uint32).tobytes()))
        with open(path, "wb") as f:
            f.write(b"".join(parts))

    @staticmethod
    def read(path):
        data = open(path, "rb").read()
        if data[:4] != b"YFS1" or struct.unpack_from("<I", data, 4)[0] != 1:
            raise ValueError("%s is not a YFS1 file" % path)
        s = FlatScene()
        off = 8
        while off < len(data):
            tag = data[off:off + 4]
            size = struct.unpack_from("<Q", data, off + 8)[0]
            p = memoryview(data)[off + 16: off + 16 + size]
            off += 16 + size
            if tag == b"CONF":
                s.config = np.frombuffer(p[:CONFIG_DTYPE.itemsize], CONFIG_DTYPE)[0].copy()
                s.camera = np.frombuffer(p[CONFIG_DTYPE.itemsize:CONFIG_DTYPE.itemsize + CAMERA_DTYPE.itemsize],
                                         CAMERA_DTYPE)[0].copy()
                s.config = np.array(s.config, CONFIG_DTYPE)
                s.camera = np.array(s.camera, CAMERA_DTYPE)
                s.other_light_count = struct.unpack_from("<I", p, CONFIG_DTYPE.itemsize + CAMERA_DTYPE.itemsize)[0]
            elif tag == b"MESH":
                vc, tc, flags, rev, vis, nc = struct.unpack_from("<6I", p, 0)
                q = 24
                bounds = np.frombuffer(p[q:q + 24], np.float32).copy()
                q += 24
                v = np.frombuffer(p[q:q + 12 * vc], np.float32).reshape(-1, 3).copy()
                q += 12 * vc
                idx = np.frombuffer(p[q:q + 12 * tc], np.int32).reshape(-1, 3).copy()
                q += 12 * tc
                normals = uvs = None
                if flags & 1:
                    normals = np.frombuffer(p[q:q + 12 * vc], np.float32).reshape(-1, 3).copy()
                    q += 12 * vc
                if flags & 2:
                    uvs = np.frombuffer(p[q:q + 8 * vc], np.float32).reshape(-1, 2).copy()
                    q += 8 * vc
                nodes = np.frombuffer(p[q:q + 8 * nc], np.uint32).reshape(-1, 2).copy()
                q += 8 * nc
                alpha = struct.unpack_from("<I", p, q)[0] if flags & 4 else 0
                s.meshes.append(Mesh(v, idx, normals, uvs, np.int32(np.uint32(rev)), vis, bounds, nodes, alpha))
            elif tag == b"OBJS":
                n = struct.unpack_from("<I", p, 0)[0]
                s.objects = np.frombuffer(p[4:4 + n * OBJECT_DTYPE.itemsize], OBJECT_DTYPE).copy()
            elif tag == b"SKDT":
                s.scene_bounds = np.frombuffer(p[:24], np.float32).copy()
                n = struct.unpack_from("<I", p, 24)[0]
                s.scene_nodes = np.frombuffer(p[28:28 + 8 * n], np.uint32).reshape(-1, 2).copy()
            elif tag in (b"MATS", b"MAT2"):
                n = struct.unpack_from("<I", p, 0)[0]
                record, q = (MATERIAL_RECORD_V1, 4) if tag == b"MATS" else (struct.unpack_from("<I", p, 4)[0], 8)
                raw = np.frombuffer(p[q:q + n * record], np.uint8).reshape(n, record)
                keep = min(record, MATERIAL_DTYPE.itemsize)
                buf = np.zeros((n, MATERIAL_DTYPE.itemsize), np.uint8)
                buf[:, :keep] = raw[:, :keep]
                s.materials = buf.view(MATERIAL_DTYPE).reshape(n).copy()
            elif tag == b"RLIT":
                n = struct.unpack_from("<I", p, 0)[0]
                s.rect_lights = np.frombuffer(p[4:4 + n * LIGHT_DTYPE.itemsize], LIGHT_DTYPE).copy()
            elif tag == b"DLIT":
                n = struct.unpack_from("<I", p, 0)[0]
                s.delta_lights = np.frombuffer(p[4:4 + n * DELTA_LIGHT_DTYPE.itemsize], DELTA_LIGHT_DTYPE).copy()
            elif tag == b"MLIT":
                n = struct.unpack_from("<I", p, 0)[0]
                s.mesh_lights = np.frombuffer(p[4:4 + n * MESH_LIGHT_DTYPE.itemsize], MESH_LIGHT_DTYPE).copy()
            elif tag == b"ENVM":
                rec = np.frombuffer(p[:ENVIRONMENT_DTYPE.itemsize], ENVIRONMENT_DTYPE)[0].copy()
                w, h = int(rec["width"]), int(rec["height"])
                img = np.frombuffer(p[ENVIRONMENT_DTYPE.itemsize:ENVIRONMENT_DTYPE.itemsize + 12 * w * h],
                                    np.float32).reshape(h, w, 3).copy()
                s.environment = (np.array(rec, ENVIRONMENT_DTYPE), img)
            elif tag == b"TEXS":
                nt, nm, nx = struct.unpack_from("<IIQ", p, 0)
                q = 16
                s.textures = np.frombuffer(p[q:q + nt * TEXTURE_DTYPE.itemsize], TEXTURE_DTYPE).copy()
                q += nt * TEXTURE_DTYPE.itemsize
                s.texture_mips = np.frombuffer(p[q:q + nm * TEXTURE_MIP_DTYPE.itemsize], TEXTURE_MIP_DTYPE).copy()
                q += nm * TEXTURE_MIP_DTYPE.itemsize
                s.texels = np.frombuffer(p[q:q + 12 * nx], np.float32).reshape(-1, 3).copy()
            elif tag == b"FOUR":
                nt, nf, nu = struct.unpack_from("<IQQ", p, 0)
                q = 20
                s.fourier_tables = np.frombuffer(p[q:q + nt * FOURIER_DTYPE.itemsize], FOURIER_DTYPE).copy()
                q += nt * FOURIER_DTYPE.itemsize
                s.fourier_floats = np.frombuffer(p[q:q + 4 * nf], np.float32).copy()
                q += 4 * nf
                s.fourier_uints = np.frombuffer(p[q:q + 4 * nu], np.uint32).copy()
            elif tag == b"SPHL":
                n = struct.unpack_from("<I", p, 0)[0]
                s.sphere_lights = np.frombuffer(p[4:4 + n * SPHERE_LIGHT_DTYPE.itemsize], SPHERE_LIGHT_DTYPE).copy()
        return s


def make_object(mesh_index, object_to_world=None, world_to_object=None, material_type=native.MATERIAL_DIFFUSE,
                material_index=0, light_type=native.LIGHT_NULL, light_index=-1):
    """A Scene_Object record; the inverse and normal transforms follow
    src/lib/scene_loader.cpp:56-62 (normal transform = transpose of the 3x3
    part of world_to_object)."""
    o = np.zeros((), OBJECT_DTYPE)
    m = IDENTITY.copy() if object_to_world is None else np.asarray(object_to_world, np.float32).reshape(12)
    if world_to_object is None:
        m44 = np.eye(4, dtype=np.float64)
        m44[:3, :] = m.reshape(3, 4)
        w = np.linalg.inv(m44)[:3, :].astype(np.float32).reshape(12)
        if np.array_equal(m, IDENTITY):
            w = IDENTITY.copy()
    else:
        w = np.asarray(world_to_object, np.float32).reshape(12)
    n = np.zeros(12, np.float32)
    w34 = w.reshape(3, 4)
    for i in range(3):
        for k in range(3):
            n[4 * i + k] = w34[k, i]
    o["mesh_index"] = mesh_index
    o["material_type"] = material_type
    o["material_index"] = material_index
    o["area_light_type"] = light_type
    o["area_light_index"] = light_index
    o["object_to_world"] = m
    o["world_to_object"] = w
    o["object_to_world_normal"] = n
    return o
