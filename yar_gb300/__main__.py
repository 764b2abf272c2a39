"""Command line: render a flat scene on the GPU and write the reference's EXR.

    python -m yar_gb300 render SCENE --out image.exr [--spp N] [--seedoffset K] [--compress] [--resolution WxH]
    python -m yar_gb300 guided SCENE --out image.exr --passes N [--guide-fraction A] [--train-passes T] [--spp N]
        [--strata-x NX] [--train-steps S] [--learning-rate R] [--guide-bounces B]
    python -m yar_gb300 info SCENE

SCENE is a .yfs flat scene (the reference's pbrt-v3 loader and kd-tree
builder flattened by the reference harness: `yar_ref flatten scene.pbrt
scene.yfs`, or FlatScene.write from the generators) or a built-in generator:
large, room.  Options mirror the reference's RAY (--spp rounds up
to a perfect square as RAY does; --seedoffset offsets the pixel streams).
The EXR carries YAR's attributes with yar_render_device = gpu.
"""
import argparse
import math
import sys

from . import exr, native, scenes
from .scene import FlatScene


def load(name):
    if name == "large":
        return scenes.large_scene()
    if name == "room":
        return scenes.hard_lighting_room()
    return FlatScene.read(name)


def main(argv=None):
    p = argparse.ArgumentParser(prog="python -m yar_gb300")
    sub = p.add_subparsers(dest="cmd", required=True)
    for name in ("render", "guided", "info"):
        q = sub.add_parser(name)
        q.add_argument("scene")
        if name == "info":
            continue
        q.add_argument("--out", required=True)
        q.add_argument("--compress", action="store_true", help="ZIP-compressed EXR")
        q.add_argument("--device", type=int, default=0)
        q.add_argument("--resolution", default=None, help="WxH: render the whole image at this size")
        if name == "render":
            q.add_argument("--spp", type=int, default=0, help="samples per pixel (rounded up to k*k)")
            q.add_argument("--seedoffset", type=int, default=None)
            q.add_argument("--traversal", choices=["auto", "p64", "p128", "per-ray", "per-ray-vote"], default="auto")
            q.add_argument("--repeat", type=int, default=1,
                           help="render this many times (the first render of a scene times the traversal "
                                "kernels; later ones drive their bounces from the device); the last is written")
        else:
            q.add_argument("--passes", type=int, default=256)
            q.add_argument("--guide-fraction", type=float, default=0.7)
            q.add_argument("--train-passes", type=int, default=64)
            q.add_argument("--time-budget", type=float, default=0.0)
            q.add_argument("--spp", type=int, default=0,
                           help="stratified form: after the training passes, this many samples per pixel")
            q.add_argument("--strata-x", type=int, default=0,
                           help="stratified form: columns of the strata grid (default ceil(sqrt(spp)))")
            q.add_argument("--train-steps", type=int, default=8, help="optimizer steps per training pass")
            q.add_argument("--learning-rate", type=float, default=2e-3)
            q.add_argument("--guide-bounces", type=int, default=0,
                           help="stratified form: guide the first this many vertices of each path (0: all)")
    a = p.parse_args(argv)
    s = load(a.scene)
    if getattr(a, "resolution", None):
        rw, rh = (int(v) for v in a.resolution.lower().split("x"))
        s.config["render_region"] = (0, 0, rw, rh)
        s.camera["image_extent"] = (rw, rh)
    region = s.config["render_region"]
    w, h = int(region[2] - region[0]), int(region[3] - region[1])
    if a.cmd == "info":
        print("%s: %d meshes, %d objects, %d triangles, %dx%d, %dx%d spp, maxdepth %d" % (
            a.scene, len(s.meshes), len(s.objects), s.triangle_count, w, h, s.config["x_pixel_sample_count"],
            s.config["y_pixel_sample_count"], s.config["max_light_bounces"]))
        return 0
    kernels = {"auto": native.TRAVERSAL_AUTO, "p64": native.TRAVERSAL_PERSISTENT_64,
               "p128": native.TRAVERSAL_PERSISTENT_128, "per-ray": native.TRAVERSAL_PER_RAY,
               "per-ray-vote": native.TRAVERSAL_PER_RAY_VOTE}
    ctx = native.Context(a.device, traversal_kernel=kernels[getattr(a, "traversal", "auto")])
    if a.cmd == "render":
        if a.spp:
            k = int(math.ceil(math.sqrt(a.spp)))
            s.config["x_pixel_sample_count"] = s.config["y_pixel_sample_count"] = k
        if a.seedoffset is not None:
            s.config["rng_seed_offset"] = a.seedoffset
        ctx.upload_scene(s)
        for _ in range(max(1, a.repeat)):
            img, st = ctx.render(w, h)
        spp = int(s.config["x_pixel_sample_count"] * s.config["y_pixel_sample_count"])
        attrs = exr.yar_attributes(spp=spp, variance=st.variance, input_file=a.scene, device="gpu")
        print("rendered %dx%d at %d spp in %.3f s (%.1f M paths/s), variance %.6g" % (
            w, h, spp, st.seconds, st.paths / st.seconds / 1e6, st.variance))
    else:
        ctx.upload_scene(s)
        img, _, st = ctx.guided_render(w, h, passes=a.passes, guide_fraction=a.guide_fraction,
                                       train_passes=a.train_passes, time_budget=a.time_budget,
                                       samples_per_pixel=a.spp, strata_x=a.strata_x, train_steps=a.train_steps,
                                       learning_rate=a.learning_rate, guide_bounces=a.guide_bounces)
        if a.spp:  # nx x ny strata, nx = strata_x or ceil(sqrt(spp)), ny = ceil(spp / nx)
            nx = a.strata_x or int(math.ceil(math.sqrt(a.spp)))
            spp = nx * ((a.spp + nx - 1) // nx)
        else:
            spp = st.passes
        attrs = exr.yar_attributes(spp=spp, input_file=a.scene, device="gpu")
        print("rendered %dx%d, %s in %.3f s (training %.3f s)" % (
            w, h, ("%d guided samples per pixel after %d training passes" % (spp, st.passes)) if a.spp
            else "%d guided passes" % st.passes, st.seconds, st.train_seconds))
    exr.write_exr(a.out, img, a.compress, attrs)
    ctx.close()
    print("wrote", a.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
