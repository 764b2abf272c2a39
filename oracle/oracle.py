"""TEST INFRASTRUCTURE ONLY: Python access to the oracle (oracle/liboracle.so,
the C restatement of the reference path) and to the reference harness
(oracle/_ref/yar_ref, the reference renderer built from its own sources).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only as the checker of the CUDA path.
"""
import ctypes as C
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "yar_ref")
REF_GPU_BIN = os.path.join(HERE, "_ref", "yar_ref_gpu")


class RayStats(C.Structure):
    _fields_ = [("nodes", C.c_uint64), ("leaf_words", C.c_uint64), ("triangle_tests", C.c_uint64),
                ("object_visits", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise ImportError("oracle/liboracle.so is not built (run the build step)")
        L = C.CDLL(ORACLE_LIB)
        L.oracle_cast_closest.restype = C.c_int
        L.oracle_cast_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]
        L.oracle_cast_any.restype = C.c_int
        L.oracle_cast_any.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.oracle_intersect_triangle_watertight.restype = C.c_float
        L.oracle_intersect_triangle_watertight.argtypes = [C.c_void_p] * 6
        L.oracle_pcg32_seed.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
        L.oracle_pcg32_next.restype = C.c_uint32
        L.oracle_pcg32_next.argtypes = [C.c_void_p]
        L.oracle_pcg32_float.restype = C.c_float
        L.oracle_pcg32_float.argtypes = [C.c_void_p]
        L.oracle_pixel_samples.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
        L.oracle_render_trig.restype = C.c_int
        L.oracle_render_trig.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32]
        _lib = L
    return _lib


def cast_closest(flat, rays, with_stats=False):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = rays.shape[0]
    desc, keep = flat.to_c()
    t = np.empty(n, np.float32)
    prim = np.empty(n, np.uint32)
    obj = np.empty(n, np.uint32)
    bary = np.empty((n, 2), np.float32)
    stats = (RayStats * n)() if with_stats else None
    rc = lib().oracle_cast_closest(C.addressof(desc), rays.ctypes.data, n, t.ctypes.data, prim.ctypes.data,
                                   obj.ctypes.data, bary.ctypes.data, C.addressof(stats) if stats else None)
    if rc != 0:
        raise RuntimeError("oracle_cast_closest failed: %d" % rc)
    out = (t, prim, obj, bary)
    if with_stats:
        return out + (np.ctypeslib.as_array(stats).view(np.uint64).reshape(n, 4),)
    return out


def cast_any(flat, rays, with_stats=False):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = rays.shape[0]
    desc, keep = flat.to_c()
    occ = np.empty(n, np.uint8)
    stats = (RayStats * n)() if with_stats else None
    rc = lib().oracle_cast_any(C.addressof(desc), rays.ctypes.data, n, occ.ctypes.data,
                               C.addressof(stats) if stats else None)
    if rc != 0:
        raise RuntimeError("oracle_cast_any failed: %d" % rc)
    if with_stats:
        return occ, np.ctypeslib.as_array(stats).view(np.uint64).reshape(n, 4)
    return occ


def render(flat, threads=0, rows=None, correctly_rounded_trig=False):
    """The reference's render.  correctly_rounded_trig: sines and cosines of
    sampled angles correctly rounded (as the CUDA path computes them) instead
    of the C library's sinf/cosf (as the reference computes them)."""
    w = int(flat.config["render_region"][2] - flat.config["render_region"][0])
    h = int(flat.config["render_region"][3] - flat.config["render_region"][1])
    rgb = np.zeros((h, w, 3), np.float32)
    var = C.c_double(0.0)
    desc, keep = flat.to_c()
    r0, r1 = (0, h) if rows is None else rows
    rc = lib().oracle_render_trig(C.addressof(desc), rgb.ctypes.data, C.addressof(var), r0, r1,
                                  int(threads or os.cpu_count() or 1), int(bool(correctly_rounded_trig)))
    if rc != 0:
        raise RuntimeError("oracle_render failed: %d" % rc)
    return rgb, var.value


# ---------------------------------------------------------------- reference harness
def have_reference():
    if not os.path.exists(REF_BIN):
        return False
    try:
        subprocess.run([REF_BIN], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=30)
        return True
    except OSError:
        return False


def _ref(*args, timeout=3600):
    r = subprocess.run([REF_BIN] + [str(a) for a in args], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("yar_ref %s failed (%d): %s %s" % (args[0], r.returncode, r.stdout[-2000:],
                                                            r.stderr[-2000:]))
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return json.loads(lines[-1]) if lines else {}


def ref_flatten(pbrt_path, yfs_path, spp=0, seed_offset=0):
    args = ["flatten", pbrt_path, yfs_path]
    if spp:
        args.append("--spp=%d" % spp)
    if seed_offset:
        args.append("--seedoffset=%d" % seed_offset)
    return _ref(*args)


def ref_render(pbrt_path, spp=0, seed_offset=0, threads=0, checkpoint_dir=None):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "img.bin")
        args = ["render", pbrt_path, out, "--threads=%d" % (threads or os.cpu_count() or 1)]
        if spp:
            args.append("--spp=%d" % spp)
        if seed_offset:
            args.append("--seedoffset=%d" % seed_offset)
        if checkpoint_dir:
            args.append("--checkpoint-dir=%s" % checkpoint_dir)
        info = _ref(*args)
        raw = open(out, "rb").read()
    w, h = np.frombuffer(raw[:8], np.uint32)
    variance = float(np.frombuffer(raw[8:16], np.float64)[0])
    seconds = float(np.frombuffer(raw[16:20], np.float32)[0])
    img = np.frombuffer(raw[20:], np.float32).reshape(int(h), int(w), 3).copy()
    info.update(variance=variance, seconds=seconds)
    return img, info


def ref_render_gpu(pbrt_path, spp=0, seed_offset=0):
    """The drop-in render_scene_gpu (oracle/render_scene_gpu.cpp): the
    reference's pbrt loader and kd-tree builder, rendered through the C ABI."""
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "img.bin")
        args = [pbrt_path, out]
        if spp:
            args.append("--spp=%d" % spp)
        if seed_offset:
            args.append("--seedoffset=%d" % seed_offset)
        r = subprocess.run([REF_GPU_BIN] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError("yar_ref_gpu failed (%d): %s %s" % (r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
        raw = open(out, "rb").read()
    w, h = np.frombuffer(raw[:8], np.uint32)
    variance = float(np.frombuffer(raw[8:16], np.float64)[0])
    img = np.frombuffer(raw[20:], np.float32).reshape(int(h), int(w), 3).copy()
    return img, variance


def ref_build(flat, threads=0):
    from yar_gb300.scene import FlatScene
    with tempfile.TemporaryDirectory() as d:
        a, b = os.path.join(d, "in.yfs"), os.path.join(d, "out.yfs")
        flat.write(a)
        info = _ref("build", a, b, "--threads=%d" % (threads or os.cpu_count() or 1))
        return FlatScene.read(b), info


def ref_cast(flat, rays, any_hit=False, threads=0, repeat=1):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = rays.shape[0]
    with tempfile.TemporaryDirectory() as d:
        s, r, o = os.path.join(d, "s.yfs"), os.path.join(d, "r.bin"), os.path.join(d, "o.bin")
        flat.write(s)
        rays.tofile(r)
        args = ["cast", s, r, o, "--threads=%d" % (threads or os.cpu_count() or 1), "--repeat=%d" % repeat]
        if any_hit:
            args.append("--any")
        info = _ref(*args)
        raw = np.fromfile(o, np.uint8)
    if any_hit:
        return raw, info
    t = raw[:4 * n].view(np.float32)
    prim = raw[4 * n:8 * n].view(np.uint32)
    obj = raw[8 * n:12 * n].view(np.uint32)
    bary = raw[12 * n:20 * n].view(np.float32).reshape(n, 2)
    return (t, prim, obj, bary), info


def ref_bench_cast(flat, rays, shadow, warmup=0, steps=1, threads=0, build=False):
    """The ray-cast benchmark through the reference (harness bench-cast): W
    untimed and K timed steps of one KdTree::intersect batch over `rays` and one
    KdTree::intersect_any batch over `shadow` on all host threads.  build: the
    kd-trees come from the reference builder instead of the flat scene."""
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    shadow = np.ascontiguousarray(shadow, np.float32).reshape(-1, 8)
    with tempfile.TemporaryDirectory() as d:
        s, r, a = os.path.join(d, "s.yfs"), os.path.join(d, "r.bin"), os.path.join(d, "a.bin")
        flat.write(s)
        rays.tofile(r)
        shadow.tofile(a)
        args = ["bench-cast", s, r, a, "--threads=%d" % (threads or os.cpu_count() or 1), "--warmup=%d" % warmup,
                "--steps=%d" % steps]
        if build:
            args.append("--build")
        return _ref(*args)


def ref_render_flat(flat, spp=0, threads=0, textures_from=None):
    """The reference renderer on a flat scene (harness render-yfs).  A textured
    flat scene names the pbrt scene it was flattened from (`textures_from`),
    whose texture files the reference loads."""
    with tempfile.TemporaryDirectory() as d:
        s, out = os.path.join(d, "s.yfs"), os.path.join(d, "img.bin")
        flat.write(s)
        args = ["render-yfs", s, out, "--threads=%d" % (threads or os.cpu_count() or 1)]
        if spp:
            args.append("--spp=%d" % spp)
        if textures_from:
            args.append("--textures-from=%s" % textures_from)
        info = _ref(*args)
        raw = open(out, "rb").read()
    w, h = np.frombuffer(raw[:8], np.uint32)
    variance = float(np.frombuffer(raw[8:16], np.float64)[0])
    img = np.frombuffer(raw[20:], np.float32).reshape(int(h), int(w), 3).copy()
    info.update(variance=variance)
    return img, info
