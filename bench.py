"""Ray-cast benchmark of the GB300 path: extend (closest-hit) + shadow (any-hit).

Workload (the ray-cast kernel bench): seeded fBm terrain of 1024 x 1024 cells
(2,097,152 FP32 triangles, 6 octaves, amplitude 0.1) plus 64 icospheres
(subdivision 4, 5,120 triangles each) = 2,424,832 triangles, kd-trees built by
the reference builder's algorithm; 16,777,216 closest-hit rays with origins
uniform in the scene box and directions uniform on the sphere, and
16,777,216 shadow rays with tmax = U[0,1] x |scene diagonal|.

One step = one extend launch over the 16M rays + one shadow launch over the
16M shadow rays.  metric = Mrays/s over both ray kinds.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun every rank runs the same workload on its own GPU (replicas,
weak scaling, no data-path collective); value = all ranks' rays / max time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))  # the checker: CPU-baseline leg only

METRIC = "Mrays/s (closest-hit + any-hit, ray-cast kernel bench)"
UNIT = "Mrays/s"
GRID, SPHERES, LEVEL = 1024, 64, 4
N_RAYS = 16 * 1024 * 1024
SEED = 1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--rays", type=int, default=N_RAYS)
    p.add_argument("--grid", type=int, default=GRID)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-render", action="store_true", help="skip the C1 render figures")
    p.add_argument("--workload", default="raycast",
                   choices=["raycast", "render-c1", "render-c3", "guided", "batch", "guide-mlp"],
                   help="render-c1 / render-c3 print a separate line for the C1 or the large (C3) render")
    return p.parse_args()


def max_over_ranks(pg, seconds, device):
    """The slowest rank's time (the job's time) under torchrun; unchanged on one process."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def workload(grid):
    from yar_gb300 import scenes
    t0 = time.time()
    s = scenes.raycast_scene(seed=SEED, grid=grid, spheres=SPHERES, level=LEVEL, build=False)
    t1 = time.time()
    s.build_kdtrees()
    t2 = time.time()
    return s, {"generate_s": round(t1 - t0, 3), "kdtree_build_s": round(t2 - t1, 3)}


def rays_for(s, n):
    from yar_gb300 import scenes
    lo, hi = scenes.scene_box(s)
    return scenes.random_rays(lo, hi, n, SEED + 100), scenes.random_shadow_rays(lo, hi, n, SEED + 200)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ algorithmic bytes
def algorithmic_bytes(s, rays, shadow, sample=65536):
    """Per-ray bytes of the traversal in the reference's visit order, counted by
    the oracle on a sample of the same batches:
      closest: 32 (ray) + 20 (hit) + 8*nodes + 4*leaf index words + 48*triangles + 96*object visits
      any:     32 (ray) + 1 (bit)  + the same traversal terms
    (48 B per triangle = 12 B indices + 36 B vertices; 96 B per object record)."""
    import oracle
    idx = np.linspace(0, rays.shape[0] - 1, sample).astype(np.int64)
    _, _, _, _, st = oracle.cast_closest(s, rays[idx], with_stats=True)
    _, st2 = oracle.cast_any(s, shadow[idx], with_stats=True)
    w = np.array([8, 4, 48, 96], np.float64)
    closest = 52.0 + (st.astype(np.float64) @ w).mean()
    anyhit = 33.0 + (st2.astype(np.float64) @ w).mean()
    return closest, anyhit, st.mean(0).tolist(), st2.mean(0).tolist()


def profile_traffic():
    """DRAM bytes per extend launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "extend_raycast_c2.md")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ------------------------------------------------------------------ CPU baselines and parity
def reference_cast_sample(s, rays, shadow, n_sample, threads):
    """The reference's KdTree::intersect / intersect_any (oracle/_ref) on host
    cores over the first n_sample rays of each batch: (closest results,
    occlusion, seconds)."""
    import oracle
    idx = slice(0, n_sample)
    (out_c, info_c) = oracle.ref_cast(s, rays[idx], threads=threads)
    (occ, info_a) = oracle.ref_cast(s, shadow[idx], any_hit=True, threads=threads)
    return out_c, occ, info_c["seconds"] + info_a["seconds"]


def port_cast_rate(s, rays, shadow, n_sample):
    import oracle
    idx = slice(0, n_sample)
    t0 = time.perf_counter()
    oracle.cast_closest(s, rays[idx])
    oracle.cast_any(s, shadow[idx])
    seconds = time.perf_counter() - t0
    return 2 * n_sample / seconds / 1e6, seconds


def cpu_baseline_and_expected(s, rays, shadow):
    """The CPU baseline (the reference's KdTree on all host threads over the
    first 2M + 2M rays, or the oracle's C port on one thread over 256K + 256K
    when the reference is not built) and its outputs, which are the expected
    results of the GPU on those rays."""
    import oracle
    threads = os.cpu_count() or 1
    if oracle.have_reference():
        n = min(rays.shape[0], 1 << 21)
        out_c, occ, sec = reference_cast_sample(s, rays, shadow, n, threads)
        base = {"value": round(2 * n / sec / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "reference",
                "sample": "%d closest + %d any-hit rays of the same batches, reference KdTree::intersect/"
                          "intersect_any on %d threads, %.2f s" % (n, n, threads, sec)}
        return base, out_c, occ, "reference KdTree::intersect / intersect_any"
    n = min(rays.shape[0], 1 << 18)
    t0 = time.perf_counter()
    out_c = oracle.cast_closest(s, rays[:n])
    occ = oracle.cast_any(s, shadow[:n])
    sec = time.perf_counter() - t0
    base = {"value": round(2 * n / sec / 1e6, 3), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d closest + %d any-hit rays of the same batches, oracle C port, 1 thread, %.2f s"
                      % (n, n, sec)}
    return base, out_c, occ, "oracle C restatement"


def cast_parity(got_c, got_occ, want_c, want_occ, source):
    """Bit-for-bit comparison of closest hits (t, triangle, object,
    barycentrics) and occlusion."""
    t, prim, obj, bary = got_c
    wt, wprim, wobj, wbary = want_c
    n = len(wt)
    bad_t = int(np.count_nonzero(t[:n].view(np.uint32) != wt.view(np.uint32)))
    bad_prim = int(np.count_nonzero(prim[:n] != wprim))
    bad_obj = int(np.count_nonzero(obj[:n] != wobj))
    bad_bary = int(np.count_nonzero(bary[:n].view(np.uint32) != wbary.view(np.uint32)))
    bad_occ = int(np.count_nonzero(got_occ[:len(want_occ)] != want_occ))
    ok = bad_t == 0 and bad_prim == 0 and bad_obj == 0 and bad_bary == 0 and bad_occ == 0
    return {"ok": ok, "against": source, "closest_rays": n, "any_rays": len(want_occ),
            "mismatches": {"t": bad_t, "triangle": bad_prim, "object": bad_obj, "barycentrics": bad_bary,
                           "occluded": bad_occ},
            "bar": "bit-identical t, triangle, object, barycentrics and occlusion"}


def builder_parity(s):
    """The product builder's node arrays and bounds against the reference
    builder's on the same scene, word for word."""
    import oracle
    if not oracle.have_reference():
        return {"ok": None, "skipped": "reference not built"}
    t0 = time.time()
    ref, info = oracle.ref_build(s, os.cpu_count() or 1)
    bad = [i for i, (m, r) in enumerate(zip(s.meshes, ref.meshes))
           if not (np.array_equal(np.asarray(m.nodes).view(np.uint32), np.asarray(r.nodes).view(np.uint32)) and
                   np.array_equal(np.asarray(m.bounds).view(np.uint32), np.asarray(r.bounds).view(np.uint32)))]
    scene_ok = (np.array_equal(np.asarray(s.scene_nodes).view(np.uint32), np.asarray(ref.scene_nodes).view(np.uint32))
                and np.array_equal(np.asarray(s.scene_bounds).view(np.uint32),
                                   np.asarray(ref.scene_bounds).view(np.uint32)))
    words = sum(np.asarray(m.nodes).size for m in s.meshes) + np.asarray(s.scene_nodes).size
    return {"ok": (not bad) and scene_ok and len(ref.meshes) == len(s.meshes), "meshes": len(s.meshes),
            "node_words": int(words), "meshes_differing": bad[:8], "scene_tree_identical": bool(scene_ok),
            "reference_build_s": round(info["mesh_build_seconds"] + info["scene_build_seconds"], 3),
            "seconds": round(time.time() - t0, 2), "bar": "word-identical node arrays and bounds"}


def image_parity(img, var, ref, ref_var, bit_equal_min=0.90, mean_rel=1e-4, var_rel=1e-5):
    """The render bars: share of bit-identical pixels, mean relative error of
    the image, relative error of the variance."""
    same = float(np.all(img.view(np.uint32) == ref.view(np.uint32), axis=2).mean())
    rel = float(np.abs(img.astype(np.float64) - ref).sum() / max(float(np.abs(ref.astype(np.float64)).sum()), 1e-30))
    vrel = abs(var - ref_var) / ref_var if ref_var else abs(var - ref_var)
    ok = same >= bit_equal_min and rel < mean_rel and vrel <= var_rel
    return {"ok": bool(ok), "bit_identical_pixels": round(same, 5), "mean_relative_error": rel,
            "variance_relative_error": vrel,
            "bar": ">= %.0f%% bit-identical pixels, mean relative error < %g, variance within %g"
                   % (100 * bit_equal_min, mean_rel, var_rel)}


def product_library_mapped():
    """True when this process has the product library (libyar_gb300.so) mapped."""
    try:
        with open("/proc/self/maps") as f:
            return any("libyar_gb300" in ln for ln in f)
    except OSError:
        return False


def run_reference(args, rank, world, pg):
    """The reference's own ray-cast path on the host cores, on the same workload
    as the GPU arm: the scene generated by the same seeded generator, its
    kd-trees built by the reference builder (build_triangle_mesh_kdtree /
    build_scene_kdtree), and each step one KdTree::intersect batch over all
    closest-hit rays and one KdTree::intersect_any batch over all shadow rays on
    every host thread.  The product library is never loaded in this process."""
    if rank != 0:
        return
    import oracle
    from yar_gb300 import scenes
    threads = os.cpu_count() or 1
    t0 = time.time()
    s = scenes.raycast_scene(seed=SEED, grid=args.grid, spheres=SPHERES, level=LEVEL, build=False)
    gen = time.time() - t0
    if oracle.have_reference():
        built, binfo = oracle.ref_build(s, threads)
        rays, shadow = rays_for(built, args.rays)
        info = oracle.ref_bench_cast(built, rays, shadow, warmup=args.warmup, steps=args.steps, threads=threads)
        secs = [c + a for c, a in info["steps"]]
        kind, cores, n = "reference", threads, args.rays
        setup = {"generate_s": round(gen, 3), "reference_kdtree_build_s": round(binfo["mesh_build_seconds"] +
                                                                              binfo["scene_build_seconds"], 3)}
        sample = "%d closest + %d any-hit rays per step (the whole batches), reference KdTree on %d threads" % (
            n, n, cores)
    else:  # the oracle's C restatement, one thread, on a bounded sample of the batches
        s.build_kdtrees()
        rays, shadow = rays_for(s, args.rays)
        n = min(args.rays, 1 << 18)
        for _ in range(args.warmup):
            port_cast_rate(s, rays, shadow, min(n, 1 << 12))
        secs = [port_cast_rate(s, rays, shadow, n)[1] for _ in range(args.steps)]
        kind, cores = "port", 1
        setup = {"generate_s": round(gen, 3)}
        sample = "%d closest + %d any-hit rays per step, oracle C port, 1 thread" % (n, n)
    ms = 1000 * statistics.median(secs)
    value = 2 * n / (ms * 1e-3) / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm terrain + icospheres, seed %d)" % SEED,
            "config": raycast_config(s.triangle_count, args.rays, 1, args.grid),
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup": setup,
            "product_library_loaded": product_library_mapped()}
    print(json.dumps(line), flush=True)


def raycast_config(triangles, rays, replicas, grid=GRID):
    return {"workload": "raycast C2: %d tris (%d^2 fBm terrain + 64 icospheres L4), %d closest + %d "
                        "any-hit rays per step" % (triangles, grid, rays, rays),
            "triangles": triangles, "rays": rays, "l2": "inputs larger than L2 (rays 512 MiB per kind)",
            "replicas": replicas}


def run_gb300(args, rank, world, local, pg):
    import torch
    from yar_gb300 import native
    torch.cuda.set_device(local)
    s, setup = workload(args.grid)
    rays, shadow = rays_for(s, args.rays)
    n = args.rays
    ctx = native.Context(local, max_batch_rays=n)
    ctx.upload_scene(s)

    dev = torch.device("cuda", local)
    d_rays = torch.from_numpy(rays).to(dev)
    d_shadow = torch.from_numpy(shadow).to(dev)
    d_t = torch.empty(n, dtype=torch.float32, device=dev)
    d_prim = torch.empty(n, dtype=torch.int32, device=dev)
    d_obj = torch.empty(n, dtype=torch.int32, device=dev)
    d_bary = torch.empty((n, 2), dtype=torch.float32, device=dev)
    d_occ = torch.empty(n, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    def step(times=None):
        ms1 = ctx.cast_closest_device(d_rays.data_ptr(), n, d_t.data_ptr(), d_prim.data_ptr(), d_obj.data_ptr(),
                                      d_bary.data_ptr(), timed=True)
        ms2 = ctx.cast_any_device(d_shadow.data_ptr(), n, d_occ.data_ptr(), timed=True)
        if times is not None:
            times.append((ms1, ms2))

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    kernel_times = []
    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step(kernel_times)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
    barrier()
    elapsed = max_over_ranks(pg, elapsed, dev)
    ms_per_step = 1000 * elapsed / args.steps
    value = world * 2 * n * args.steps / elapsed / 1e6

    # end to end: the C ABI with pinned host buffers, copies inside the timed region
    h_rays = torch.from_numpy(rays).pin_memory()
    h_shadow = torch.from_numpy(shadow).pin_memory()
    h_t = torch.empty(n, dtype=torch.float32).pin_memory()
    h_prim = torch.empty(n, dtype=torch.int32).pin_memory()
    h_obj = torch.empty(n, dtype=torch.int32).pin_memory()
    h_bary = torch.empty((n, 2), dtype=torch.float32).pin_memory()
    h_occ = torch.empty(n, dtype=torch.uint8).pin_memory()
    hits = native.HitSoa(h_t.data_ptr(), h_prim.data_ptr(), h_obj.data_ptr(), h_bary.data_ptr())
    import ctypes as C

    # the box's pinned host <-> device copy bandwidth (512 MiB each way, best of 3):
    # the end-to-end figure overlaps these copies with the traversal
    def copy_gbs(dst, src):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return round(src.numel() * src.element_size() / best / 1e9, 1)
    host_copy = {"h2d": copy_gbs(d_rays, h_rays), "d2h": copy_gbs(h_rays, d_rays)}

    def e2e_step():
        rc = native.lib().yar_gpu_cast_closest(ctx._h, h_rays.data_ptr(), n, C.byref(hits), native.YAR_BUFFERS_HOST)
        ctx._check(rc, "cast_closest")
        rc = native.lib().yar_gpu_cast_any(ctx._h, h_shadow.data_ptr(), n, h_occ.data_ptr(), native.YAR_BUFFERS_HOST)
        ctx._check(rc, "cast_any")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_elapsed = time.perf_counter() - t0
    barrier()
    e2e_elapsed = max_over_ranks(pg, e2e_elapsed, dev)
    e2e_value = world * 2 * n * args.steps / e2e_elapsed / 1e6
    h2d = 2 * n * 32
    d2h = n * (4 + 4 + 4 + 8) + n

    # correctness spot check of the timed outputs against the host-buffer path
    same = bool(np.array_equal(d_prim[:4096].cpu().numpy().view(np.uint32), h_prim[:4096].numpy().view(np.uint32))
                and np.array_equal(d_occ[:4096].cpu().numpy(), h_occ[:4096].numpy()))

    if rank != 0:
        return
    ext_ms = statistics.median([a for a, b in kernel_times])
    shd_ms = statistics.median([b for a, b in kernel_times])
    bpr_closest, bpr_any, st_c, st_a = algorithmic_bytes(s, rays, shadow)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = bpr_closest * n / (ext_ms * 1e-3) / 1e9
    traffic = profile_traffic()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded fBm terrain + icospheres, seed %d)" % SEED,
        "config": raycast_config(s.triangle_count, n, world, args.grid),
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "pipeline_chunk_rays": 4 << 20, "host_copy_gbs": host_copy},
        "gpu_launches": 2 * args.steps,
        "kernels": {"extend_ms": round(ext_ms, 3), "shadow_ms": round(shd_ms, 3),
                    "extend_mrays_s": round(n / ext_ms / 1e3, 1), "shadow_mrays_s": round(n / shd_ms / 1e3, 1)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_src,
                     "traffic": traffic, "kernel": "extend",
                     "algorithmic_bytes_per_ray": round(bpr_closest, 1),
                     "any_hit_bytes_per_ray": round(bpr_any, 1),
                     "mean_per_ray_closest": dict(zip(["nodes", "leaf_words", "triangles", "objects"],
                                                      [round(x, 2) for x in st_c])),
                     "mean_per_ray_any": dict(zip(["nodes", "leaf_words", "triangles", "objects"],
                                                  [round(x, 2) for x in st_a]))},
        "clocks": clocks.summary(),
        "setup": setup,
        "outputs_consistent": same,
    }
    parity = {}
    if not args.no_cpu_baseline:
        # the reference's results on the first rays of the timed batches are the
        # expected outputs of the last timed step, bit for bit
        base, want_c, want_occ, source = cpu_baseline_and_expected(s, rays, shadow)
        line["cpu_baseline"] = base
        m = len(want_c[0])
        got_c = (d_t[:m].cpu().numpy(), d_prim[:m].cpu().numpy().view(np.uint32),
                 d_obj[:m].cpu().numpy().view(np.uint32), d_bary[:m].cpu().numpy())
        parity["c2_cast"] = cast_parity(got_c, d_occ[:len(want_occ)].cpu().numpy(), want_c, want_occ, source)
        parity["c2_kdtree_build"] = builder_parity(s)
    ctx.close()
    del d_rays, d_shadow, d_t, d_prim, d_obj, d_bary, d_occ
    torch.cuda.empty_cache()
    if not args.no_render:
        with_cpu = not args.no_cpu_baseline
        line["render_c1"] = render_bench("c1", with_cpu=with_cpu)
        line["render_c3"] = render_bench("c3", with_cpu=with_cpu, reps=2)
        for k in ("c1", "c3"):
            if "parity" in line["render_" + k]:
                parity["render_" + k] = line["render_" + k].pop("parity")
        line["batch_c4"] = batch_bench(sequential=False)
        g = guided_bench(with_cpu=with_cpu)
        if g is not None:
            line["guided_c5"] = g
            if "oracle_vs_reference" in g:
                parity["room_oracle"] = g["oracle_vs_reference"]
    if parity:
        parity["ok"] = all(v.get("ok") is not False for v in parity.values() if isinstance(v, dict))
        line["parity"] = parity
    print(json.dumps(line), flush=True)
    if parity and not parity["ok"]:
        sys.exit(3)


# ------------------------------------------------------------------ render path
def c1_scene(width=256, height=256):
    """The Cornell box (5 walls, 2 rotated boxes, a 0.25 x 0.25 light of
    radiance 17) as the reference's loader and builder flattened it, at
    width x height, 16 spp, maxdepth 8, pcg seed offset 1."""
    from yar_gb300.scene import FlatScene
    s = FlatScene.read(os.path.join(ROOT, "tests", "golden", "cornell_c1_64.yfs"))
    s.config["render_region"] = (0, 0, width, height)
    s.camera["image_extent"] = (width, height)
    return s


def render_bench(kind, with_cpu=True, reps=3):
    """GPU render time (yar_gpu_render, best of `reps`) and, when the reference
    is built here, the reference renderer's render_scene time on all host
    threads (C3: at 1 spp, reported as paths/s).  `parity` compares the GPU
    image with the reference's image of the same configuration (C3: both at 1
    spp) under the render bars, and with the oracle's image computed with
    correctly rounded trigonometry (as the device computes it) bit for bit."""
    import oracle
    from yar_gb300 import native, scenes
    if kind == "c1":
        s = c1_scene()
        desc = "C1 Cornell box 256x256, 16 spp, maxdepth 8 (diffuse, 1 quad light)"
    else:
        s = scenes.large_scene(seed=1)
        desc = ("C3 %d triangles, 1920x1080, 64 spp, maxdepth 16, RR from bounce 3, 50%% Lambertian / 50%% GGX, "
                "64 quad lights" % s.triangle_count)
    w = int(s.config["render_region"][2])
    h = int(s.config["render_region"][3])
    ctx = native.Context(0)
    ctx.upload_scene(s)
    best = None
    for _ in range(reps):
        img, st = ctx.render(w, h)
        if best is None or st.seconds < best.seconds:
            best = st
    kernels = ctx.traversal_kernels()
    ctx.close()
    out = {"workload": desc, "gpu_seconds": round(best.seconds, 4), "paths": int(best.paths),
           "gpu_paths_per_s": round(best.paths / best.seconds, 1),
           "gpu_mrays_per_s": round((best.rays_closest + best.rays_any) / best.seconds / 1e6, 2),
           "rays_closest": int(best.rays_closest), "rays_any": int(best.rays_any),
           "kernel_launches": int(best.kernel_launches), "image_mean": float(img.mean()),
           "traversal_kernels": {k: [["-", "p64", "p128", "per_ray", "per_ray_vote"][c] for c in v]
                                 for k, v in kernels.items() if k != "cast"}}
    if not with_cpu:
        return out
    spp = 1 if kind == "c3" else 0
    if spp:  # the GPU image of the compared configuration
        s.config["x_pixel_sample_count"] = 1
        s.config["y_pixel_sample_count"] = 1
        ctx = native.Context(0)
        ctx.upload_scene(s)
        img, st1 = ctx.render(w, h)
        ctx.close()
        var = st1.variance
    else:
        var = best.variance
    parity = {"config": desc if not spp else desc.replace("64 spp", "1 spp")}
    if oracle.have_reference():
        ref, info = oracle.ref_render_flat(s, spp=spp)
        paths = w * h * int(s.config["x_pixel_sample_count"] * s.config["y_pixel_sample_count"])
        out["cpu_reference"] = {"seconds": info["render_seconds"], "threads": info["threads"], "paths": paths,
                                "paths_per_s": round(paths / info["render_seconds"], 1),
                                "sample": "full image" if not spp else "full image at 1 spp"}
        out["speedup_paths_per_s"] = round(out["gpu_paths_per_s"] / out["cpu_reference"]["paths_per_s"], 1)
        parity["vs_reference"] = image_parity(img, var, ref, info["variance"])
    want, want_var = oracle.render(s, correctly_rounded_trig=True)
    same = float(np.all(img.view(np.uint32) == want.view(np.uint32), axis=2).mean())
    parity["vs_oracle_correctly_rounded_trig"] = {
        "ok": bool(same == 1.0 and want_var == var), "bit_identical_pixels": same,
        "variance_identical": bool(want_var == var), "bar": "every pixel and the variance bit-identical"}
    parity["ok"] = all(v["ok"] for k, v in parity.items() if isinstance(v, dict))
    out["parity"] = parity
    return out


GUIDE = dict(guide_fraction=0.7, train_passes=32, train_steps=32, learning_rate=5e-3)  # one-sample passes
# stratified form: settings from a sweep on the room (guide fraction 0.5-0.8, guided bounces 1-3 or all,
# 4-16 training passes, 32-128 Adam steps, learning rate 3e-3-1e-2)
GUIDE_STRATIFIED = dict(guide_fraction=0.6, train_passes=4, train_steps=64, learning_rate=5e-3, guide_bounces=2)


def strata_grids(k):
    """(columns, rows) grids between (k - 1)^2 and k^2 samples (exclusive),
    columns >= rows, aspect at most 4:3, the squarest of each sample count,
    by increasing count; then k x k."""
    best = {}
    for nx in range(k - 4, k + 5):
        for ny in range(max(1, k - 5), nx + 1):
            n = nx * ny
            if (k - 1) ** 2 < n < k * k and 3 * nx <= 4 * ny and (n not in best or nx - ny < best[n][0] - best[n][1]):
                best[n] = (nx, ny)
    return [best[n] for n in sorted(best)] + [(k, k)]


def guided_bench(plain_spp_side=32, offsets=(2, 3, 4), with_cpu=True):
    """The learned proposal on the hard-lighting room against both plain forms,
    all against the committed FP64 plain-mode oracle (tests/golden/room_oracle.npz,
    made by make_room_oracle.py):
      - plain render: yar_gpu_render with the reference's stratified sampler at
        plain_spp_side^2 samples per pixel (1024);
      - plain passes: yar_gpu_guided_render at guide fraction 0, 1024 one-sample
        passes;
      - guided (stratified form of yar_gpu_guided_render: the training passes,
        then the pixel sampler at nx x ny samples per pixel with continuations
        from the trained proposal): for each stream offset, k is raised until
        the k x k render's RMSE is at or below the better plain form's; then
        every near-square grid between (k - 1)^2 and k^2 samples is rendered;
        the smallest grid from which on every larger grid reaches that RMSE is
        rendered once more (the next larger grid while that render misses it:
        the online training makes renders differ run to run), and that
        render's wall time (training included), like the plain render's second
        run, is the measured time to it.
    oracle_vs_reference: the oracle's 64 x 64 tile means against the reference
    CPU renderer's at 16 spp (z-scores from the noise of two reference renders
    with different seed offsets)."""
    path = os.path.join(ROOT, "tests", "golden", "room_oracle.npz")
    if not os.path.exists(path):
        return None
    from yar_gb300 import native, scenes
    z = np.load(path)
    oracle_img = z["image"].astype(np.float64)
    s = scenes.hard_lighting_room()
    w, h = int(s.config["render_region"][2]), int(s.config["render_region"][3])

    def rmse(img):
        return float(np.sqrt(((img.astype(np.float64) - oracle_img) ** 2).mean()))

    # plain render, the reference's sampler: 32 x 32 samples per pixel
    sp = scenes.hard_lighting_room()
    sp.config["x_pixel_sample_count"] = plain_spp_side
    sp.config["y_pixel_sample_count"] = plain_spp_side
    ctx = native.Context(0)
    ctx.upload_scene(sp)
    ctx.render(w, h)  # the first render includes the per-scene traversal-kernel timing
    img_r, st_r = ctx.render(w, h)
    ctx.upload_scene(s)
    # warm-up: kernel loading and the per-scene traversal-kernel timing
    ctx.guided_render(w, h, passes=4, stream_offset=4090)
    ctx.guided_render(w, h, passes=4, train_passes=2, stream_offset=4091, **{k: v for k, v in GUIDE.items()
                                                                           if k != "train_passes"})
    img_p, _, st_p = ctx.guided_render(w, h, passes=plain_spp_side ** 2, stream_offset=1)
    r_r, r_p = rmse(img_r), rmse(img_p)
    target, t_target = min((r_r, st_r.seconds), (r_p, st_p.seconds))
    ctx.guided_render(w, h, samples_per_pixel=16, stream_offset=4092, **GUIDE_STRATIFIED)  # warm-up of the stratified form
    runs = []
    for off in offsets:
        side = 16
        img_g, _, st_g = ctx.guided_render(w, h, samples_per_pixel=side * side, stream_offset=off, **GUIDE_STRATIFIED)
        r_g = rmse(img_g)
        side = max(1, int(np.ceil(side * r_g / target)))  # RMSE ~ 1 / sqrt(spp)
        for _ in range(8):
            img_g, _, st_g = ctx.guided_render(w, h, samples_per_pixel=side * side, stream_offset=off,
                                               **GUIDE_STRATIFIED)
            r_g = rmse(img_g)
            if r_g <= target:
                break
            side += 1
        grids = [(side, side)]
        i = 0
        if r_g <= target and side > 2:
            # the grids below k x k: the smallest from which on all reach the target
            grids = strata_grids(side)
            reached = []
            for nx, ny in grids[:-1]:
                img_2, _, st_2 = ctx.guided_render(w, h, samples_per_pixel=nx * ny, strata_x=nx, stream_offset=off,
                                                   **GUIDE_STRATIFIED)
                reached.append(rmse(img_2) <= target)
            reached.append(True)
            i = len(grids) - 1
            while i > 0 and reached[i - 1]:
                i -= 1
        # timed as the plain render is, on a second render (warm buffers); the
        # training makes renders differ run to run, so a timing run that misses
        # the target moves on to the next larger grid
        grids += [(side + 1, side), (side + 1, side + 1)]
        while True:
            grid = grids[i]
            spp = grid[0] * grid[1]
            img_g, _, st_g = ctx.guided_render(w, h, samples_per_pixel=spp, strata_x=grid[0], stream_offset=off,
                                               **GUIDE_STRATIFIED)
            r_g = rmse(img_g)
            if r_g <= target or i == len(grids) - 1:
                break
            i += 1
        runs.append({"stream_offset": off, "spp": spp, "strata": list(grid), "seconds": round(st_g.seconds, 3),
                     "rmse": r_g, "reached": bool(r_g <= target), "train_passes": int(st_g.passes),
                     "train_seconds": round(st_g.train_seconds, 3)})
    ctx.close()
    times = [r["seconds"] for r in runs if r["reached"]]
    # float16 storage of the oracle: each pixel rounded within 2^-11 relative
    q_bound = float(np.sqrt(((oracle_img * 2.0 ** -11) ** 2).mean()))
    out = {
        "workload": "hard-lighting room: %d triangles, 512x512, maxdepth 12, one 0.1x0.1 light of radiance 1000 0.6 "
                    "above a 0.1x0.1 ceiling opening, GGX metal walls (roughness 0.1-0.3), boxes outside the beam" % s.triangle_count,
        "oracle": "plain mode, %d one-sample passes, FP64 accumulation, stored as float16 (RMSE of the rounding "
                  "at most %.2e)" % (int(z["passes"]), q_bound),
        "plain_render": {"spp": plain_spp_side ** 2, "seconds": round(st_r.seconds, 3), "rmse": r_r,
                         "sampler": "the reference's stratified pixel sampler (yar_gpu_render)"},
        "plain_passes": {"passes": int(st_p.passes), "seconds": round(st_p.seconds, 3), "rmse": r_p,
                         "mrays_per_s": round(st_p.rays / st_p.seconds / 1e6, 1)},
        "target": {"rmse": target, "seconds": round(t_target, 3),
                   "form": "plain_render" if r_r <= r_p else "plain_passes"},
        "guided": {"runs": runs, **GUIDE_STRATIFIED},
        "time_to_plain_rmse": round(statistics.median(times) / t_target, 4) if len(times) == len(runs) else None,
    }
    if with_cpu:
        out["oracle_vs_reference"] = room_oracle_check(s, oracle_img)
    return out


def room_oracle_check(s, oracle_img, spp_side=8, renders=2, tile=64):
    """The room oracle against the reference CPU renderer: `renders` reference
    renders at spp_side^2 samples per pixel with different seed offsets,
    averaged, against the oracle's image mean and 64 x 64 tile means.  The
    bounds are set from the noise of reference renders of this size (measured:
    one 64-spp render is within 0.2% of the oracle's image mean, its tile means
    within 2% rms and 6% at most; heavy-tailed light paths through the ceiling
    opening keep the tile z-scores far from normal at these sample counts)."""
    import oracle
    if not oracle.have_reference():
        return {"ok": None, "skipped": "reference not built"}
    imgs = []
    for off in range(renders):
        r = scenes_copy(s)
        r.config["x_pixel_sample_count"] = spp_side
        r.config["y_pixel_sample_count"] = spp_side
        r.config["rng_seed_offset"] = 7 * off
        img, _ = oracle.ref_render_flat(r)
        imgs.append(img.astype(np.float64))
    ref = np.mean(imgs, axis=0)
    h, w = oracle_img.shape[:2]
    rel = []
    for ty in range(0, h, tile):
        for tx in range(0, w, tile):
            o = oracle_img[ty:ty + tile, tx:tx + tile].mean()
            rel.append((ref[ty:ty + tile, tx:tx + tile].mean() - o) / o)
    rel = np.abs(np.array(rel))
    mean_rel = abs(ref.mean() - oracle_img.mean()) / oracle_img.mean()
    rms = float(np.sqrt((rel ** 2).mean()))
    return {"ok": bool(mean_rel < 5e-3 and rms < 0.03 and rel.max() < 0.08),
            "reference_spp": renders * spp_side ** 2, "image_mean_relative_difference": round(float(mean_rel), 6),
            "tile_relative_difference_rms": round(rms, 5), "tile_relative_difference_max": round(float(rel.max()), 5),
            "tiles": int(rel.size), "bar": "image mean within 0.5%, 64x64 tile means within 3% rms and 8% at most"}


def scenes_copy(s):
    from yar_gb300.scene import FlatScene
    import copy
    c = FlatScene()
    c.__dict__.update({k: copy.deepcopy(v) if k == "config" else v for k, v in s.__dict__.items()})
    return c


def batch_bench(count=64, sequential=True):
    """The batched workload: `count` procedural scenes (scenes.batch_scenes)
    in one yar_gpu_render_batch call; aggregate paths/s over the graph's GPU
    makespan and per-scene completion percentiles.  sequential: also render
    the scenes one after another through yar_gpu_render, for the gain."""
    from yar_gb300 import native, scenes
    t0 = time.time()
    flats = scenes.batch_scenes(count=count)
    gen = time.time() - t0
    ctx = native.Context(0)
    imgs, sst, st = ctx.render_batch(flats)
    # the same scenes one after another through yar_gpu_render (host-driven
    # bounces, one scene in flight), for the gain of batching
    seq = 0.0
    for f in (flats if sequential else []):
        ctx.upload_scene(f)
        r = f.config["render_region"]
        _, rs = ctx.render(int(r[2] - r[0]), int(r[3] - r[1]))
        seq += rs.seconds
    ctx.close()
    comp = sorted(x.completion_seconds for x in sst)
    pct = lambda q: comp[min(len(comp) - 1, int(round(q * (len(comp) - 1))))]
    tris = sorted(f.triangle_count for f in flats)
    return {
        "workload": "%d scenes: triangles %d..%d (log-uniform 1K-200K), resolutions 128^2..1024^2, spp 4..256 "
                    "(perfect squares), maxdepth 8, 50%% Lambertian / 50%% GGX, 4-16 quad lights"
                    % (count, tris[0], tris[-1]),
        "paths": int(st.paths),
        "gpu_seconds": round(st.gpu_seconds, 4),
        "paths_per_s": round(st.paths / st.gpu_seconds, 1),
        "mrays_per_s": round((st.rays_closest + st.rays_any) / st.gpu_seconds / 1e6, 1),
        "sequential_render_seconds": round(seq, 3) if sequential else None,
        "speedup_vs_sequential": round(seq / st.gpu_seconds, 2) if sequential else None,
        "completion_p50_s": round(pct(0.5), 4),
        "completion_p99_s": round(pct(0.99), 4),
        "autotuner": {"branches": int(st.branches), "chunk_paths": int(st.chunk_paths),
                      "traversal_kernels": {k: sum(1 for x in sst if tuple(x.traversal_kernel) == v)
                                            for k, v in (("p64/p64", (1, 1)), ("per_ray/per_ray", (3, 3)),
                                                         ("per_ray_vote/per_ray_vote", (4, 4)))}},
        "host_seconds": {"generate_and_build": round(gen, 2), "upload": round(st.upload_seconds, 2),
                         "tune": round(st.tune_seconds, 2), "capture": round(st.capture_seconds, 2)},
        "image_mean": float(np.mean([i.mean() for i in imgs])),
    }


def guide_mlp_bench(n_infer=1 << 20, n_train=1 << 18, reps=20):
    """The learned proposal's tensor-core kernels alone: inference of n_infer
    rows and one Adam step over n_train rows through the C ABI (each call
    synchronises; host-timed over `reps` calls, so launch and synchronisation
    overhead is included), against the measured dense bf16 peak."""
    import torch
    from yar_gb300 import native
    box = (-1.0, 0.0, -1.0, 1.0, 2.0, 1.0)
    g = torch.Generator(device="cuda").manual_seed(5)

    def rows(n, width):
        r = torch.zeros((n, width), device="cuda")
        r[:, 0:3] = torch.rand((n, 3), device="cuda", generator=g) * torch.tensor([2.0, 2.0, 2.0], device="cuda") + \
            torch.tensor(box[:3], device="cuda")
        for c in (3, 6) + ((9,) if width == 16 else ()):
            v = torch.randn((n, 3), device="cuda", generator=g)
            r[:, c:c + 3] = v / v.norm(dim=1, keepdim=True)
        if width == 16:
            r[:, 12] = torch.rand(n, device="cuda", generator=g)
        return r

    ctx = native.Context(0)
    q, s = rows(n_infer, 12), rows(n_train, 16)
    lobes = torch.empty((n_infer, 40), device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        ctx.guide_infer(q.data_ptr(), n_infer, box, lobes.data_ptr())
        ctx.guide_train_step(s.data_ptr(), n_train, box, 1.0 / n_train, 1e-4)
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.guide_infer(q.data_ptr(), n_infer, box, lobes.data_ptr())
    t_inf = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.guide_train_step(s.data_ptr(), n_train, box, 1.0 / n_train, 1e-4)
    t_tr = (time.perf_counter() - t0) / reps
    ctx.close()
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("bf16_tflops", 1900.0)
        src = "measured"
    except (OSError, ValueError):
        peak, src = 1900.0, "fallback"
    f_inf = 2 * (64 * 128 + 3 * 64 * 64)             # MMA flops per row: 4 layers
    f_tr = f_inf + 2 * 3 * 64 * 64 + f_inf           # + input gradients of layers 4..2 + weight gradients
    return {
        "inference": {"rows": n_infer, "ms": round(1e3 * t_inf, 3), "rows_per_s": round(n_infer / t_inf, 1),
                      "tflops": round(f_inf * n_infer / t_inf / 1e12, 2),
                      "frac_of_peak": round(f_inf * n_infer / t_inf / 1e12 / peak, 4)},
        "train_step": {"rows": n_train, "ms": round(1e3 * t_tr, 3), "rows_per_s": round(n_train / t_tr, 1),
                       "tflops": round(f_tr * n_train / t_tr / 1e12, 2),
                       "frac_of_peak": round(f_tr * n_train / t_tr / 1e12 / peak, 4)},
        "peak_bf16_tflops": peak, "peak_source": src,
        "flops_per_row": {"inference": f_inf, "train": f_tr},
    }


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    try:
        if args.workload == "guide-mlp":
            if rank == 0:
                m = guide_mlp_bench()
                print(json.dumps({"metric": "guide network rows/s (tcgen05 BF16 MLP inference)", "impl": args.impl,
                                  "value": m["inference"]["rows_per_s"], "unit": "rows/s", "higher_is_better": True,
                                  "guide_mlp": m}), flush=True)
        elif args.workload == "batch":
            if rank == 0:
                b = batch_bench()
                print(json.dumps({"metric": "paths/s (batched render, one graph launch)", "impl": args.impl,
                                  "value": b["paths_per_s"], "unit": "paths/s", "higher_is_better": True,
                                  "batch": b}), flush=True)
        elif args.workload == "guided":
            if rank == 0:
                g = guided_bench(with_cpu=not args.no_cpu_baseline)
                print(json.dumps({"metric": "time to the plain render's RMSE vs FP64 oracle, guided / plain",
                                  "impl": args.impl, "value": None if g is None else g["time_to_plain_rmse"],
                                  "unit": "ratio", "higher_is_better": False, "guided": g}), flush=True)
        elif args.workload in ("render-c1", "render-c3"):
            if rank == 0:
                kind = args.workload[-2:]
                r = render_bench(kind, with_cpu=not args.no_cpu_baseline, reps=2 if kind == "c3" else 3)
                print(json.dumps({"metric": "paths/s (%s wavefront render)" % kind.upper(), "value": r["gpu_paths_per_s"],
                                  "unit": "paths/s", "higher_is_better": True, "impl": args.impl, "render": r}),
                      flush=True)
        elif args.impl == "reference":
            run_reference(args, rank, world, pg)
        else:
            run_gb300(args, rank, world, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    main()
