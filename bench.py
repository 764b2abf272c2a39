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


# ------------------------------------------------------------------ CPU baselines
def reference_cast_rate(s, rays, shadow, n_sample, threads):
    """The reference's KdTree::intersect / intersect_any (oracle/_ref) on host cores."""
    import oracle
    idx = slice(0, n_sample)
    (_, info_c) = oracle.ref_cast(s, rays[idx], threads=threads)
    (_, info_a) = oracle.ref_cast(s, shadow[idx], any_hit=True, threads=threads)
    seconds = info_c["seconds"] + info_a["seconds"]
    return 2 * n_sample / seconds / 1e6, seconds


def port_cast_rate(s, rays, shadow, n_sample):
    import oracle
    idx = slice(0, n_sample)
    t0 = time.perf_counter()
    oracle.cast_closest(s, rays[idx])
    oracle.cast_any(s, shadow[idx])
    seconds = time.perf_counter() - t0
    return 2 * n_sample / seconds / 1e6, seconds


def cpu_baseline(s, rays, shadow):
    import oracle
    threads = os.cpu_count() or 1
    if oracle.have_reference():
        n = min(rays.shape[0], 1 << 21)
        rate, sec = reference_cast_rate(s, rays, shadow, n, threads)
        return {"value": round(rate, 3), "unit": UNIT, "cores": threads, "kind": "reference",
                "sample": "%d closest + %d any-hit rays of the same batches, reference KdTree::intersect/"
                          "intersect_any on %d threads, %.2f s" % (n, n, threads, sec)}
    n = min(rays.shape[0], 1 << 18)
    rate, sec = port_cast_rate(s, rays, shadow, n)
    return {"value": round(rate, 3), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d closest + %d any-hit rays of the same batches, oracle C port, 1 thread, %.2f s"
                      % (n, n, sec)}


# ------------------------------------------------------------------ arms
def run_reference(args, rank, world, pg):
    if rank != 0:
        return
    s, setup = workload(args.grid)
    rays, shadow = rays_for(s, args.rays)
    import oracle
    threads = os.cpu_count() or 1
    have_ref = oracle.have_reference()
    n = min(args.rays, (1 << 21) if have_ref else (1 << 18))
    for _ in range(args.warmup):
        if have_ref:
            reference_cast_rate(s, rays, shadow, min(n, 1 << 16), threads)
        else:
            port_cast_rate(s, rays, shadow, min(n, 1 << 12))
    rates, secs = [], []
    for _ in range(args.steps):
        if have_ref:
            r, sec = reference_cast_rate(s, rays, shadow, n, threads)
        else:
            r, sec = port_cast_rate(s, rays, shadow, n)
        rates.append(r)
        secs.append(sec)
    value = statistics.median(rates)
    kind = "reference" if have_ref else "port"
    cores = threads if have_ref else 1
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000 * statistics.median(secs), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm terrain + icospheres, seed %d)" % SEED,
            "config": {"workload": "raycast C2: %d tris, %d closest + %d any-hit rays; each step a sample of %d+%d"
                                   % (s.triangle_count, args.rays, args.rays, n, n),
                       "triangles": s.triangle_count, "rays": args.rays},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": "%d closest + %d any-hit rays per step on %d host threads" % (n, n, cores)},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
        "config": {"workload": "raycast C2: %d tris (1024^2 fBm terrain + 64 icospheres L4), %d closest + %d "
                               "any-hit rays per step" % (s.triangle_count, n, n),
                   "triangles": s.triangle_count, "rays": n, "l2": "inputs larger than L2 (rays 512 MiB per kind)",
                   "replicas": world},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
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
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s, rays, shadow)
    ctx.close()
    if not args.no_render:
        line["render_c1"] = render_bench("c1", with_cpu=not args.no_cpu_baseline)
        g = guided_bench()
        if g is not None:
            line["guided_c5"] = g
    print(json.dumps(line), flush=True)


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
    threads (C3: at 1 spp, reported as paths/s)."""
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
           "traversal_kernels": {k: [["-", "p64", "p128", "per_ray"][c] for c in v]
                                 for k, v in kernels.items() if k != "cast"}}
    if with_cpu and oracle.have_reference():
        spp = 1 if kind == "c3" else 0
        _, info = oracle.ref_render_flat(s, spp=spp)
        paths = w * h * (1 if spp else int(s.config["x_pixel_sample_count"] * s.config["y_pixel_sample_count"]))
        out["cpu_reference"] = {"seconds": info["render_seconds"], "threads": info["threads"], "paths": paths,
                                "paths_per_s": round(paths / info["render_seconds"], 1),
                                "sample": "full image" if not spp else "full image at 1 spp"}
        out["speedup_paths_per_s"] = round(out["gpu_paths_per_s"] / out["cpu_reference"]["paths_per_s"], 1)
    return out


GUIDE = dict(guide_fraction=0.7, train_passes=32, train_steps=32, learning_rate=5e-3)


def guided_bench(plain_passes=1024):
    """Equal-time RMSE of the guided render against the plain one on the
    hard-lighting room, both against the committed FP64 plain-mode oracle
    (tests/golden/room_oracle.npz, made by make_room_oracle.py).  The plain
    render's time for `plain_passes` one-sample passes is the budget given to
    the guided render (training included)."""
    path = os.path.join(ROOT, "tests", "golden", "room_oracle.npz")
    if not os.path.exists(path):
        return None
    from yar_gb300 import native, scenes
    z = np.load(path)
    oracle = z["image"].astype(np.float64)
    s = scenes.hard_lighting_room()
    w, h = int(s.config["render_region"][2]), int(s.config["render_region"][3])
    ctx = native.Context(0)
    ctx.upload_scene(s)
    # warm-up: kernel loading and the per-scene traversal-kernel timing
    ctx.guided_render(w, h, passes=4, stream_offset=4090)
    ctx.guided_render(w, h, passes=4, train_passes=2, stream_offset=4091, **{k: v for k, v in GUIDE.items()
                                                                           if k != "train_passes"})

    def rmse(img):
        return float(np.sqrt(((img.astype(np.float64) - oracle) ** 2).mean()))

    img_p, _, st_p = ctx.guided_render(w, h, passes=plain_passes, stream_offset=1)
    budget = st_p.seconds
    img_g, _, st_g = ctx.guided_render(w, h, passes=1 << 24, stream_offset=2, time_budget=budget, **GUIDE)
    ctx.close()
    r_p, r_g = rmse(img_p), rmse(img_g)
    return {
        "workload": "hard-lighting room: %d triangles, 512x512, maxdepth 12, one 0.1x0.1 light of radiance 1000 0.6 "
                    "above a 0.1x0.1 ceiling opening, GGX metal walls (roughness 0.1-0.3), boxes outside the beam" % s.triangle_count,
        "oracle": "plain mode, %d one-sample passes, FP64 accumulation" % int(z["passes"]),
        "plain": {"passes": int(st_p.passes), "seconds": round(st_p.seconds, 3), "rmse": r_p,
                  "mrays_per_s": round(st_p.rays / st_p.seconds / 1e6, 1)},
        "guided": {"passes": int(st_g.passes), "seconds": round(st_g.seconds, 3), "rmse": r_g,
                   "train_seconds": round(st_g.train_seconds, 3), "train_samples": int(st_g.train_samples),
                   "mrays_per_s": round(st_g.rays / st_g.seconds / 1e6, 1), **GUIDE},
        "rmse_ratio_equal_time": round(r_g / r_p, 4),
        # RMSE falls as time^-1/2: time the guided render needs for the plain render's RMSE, relative
        "time_ratio_equal_rmse": round((r_g / r_p) ** 2, 4),
    }


def batch_bench(count=64):
    """The batched workload: `count` procedural scenes (scenes.batch_scenes)
    in one yar_gpu_render_batch call; aggregate paths/s over the graph's GPU
    makespan and per-scene completion percentiles."""
    from yar_gb300 import native, scenes
    t0 = time.time()
    flats = scenes.batch_scenes(count=count)
    gen = time.time() - t0
    ctx = native.Context(0)
    imgs, sst, st = ctx.render_batch(flats)
    # the same scenes one after another through yar_gpu_render (host-driven
    # bounces, one scene in flight), for the gain of batching
    seq = 0.0
    for f in flats:
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
        "sequential_render_seconds": round(seq, 3),
        "speedup_vs_sequential": round(seq / st.gpu_seconds, 2),
        "completion_p50_s": round(pct(0.5), 4),
        "completion_p99_s": round(pct(0.99), 4),
        "autotuner": {"branches": int(st.branches), "chunk_paths": int(st.chunk_paths),
                      "traversal_kernels": {k: sum(1 for x in sst if tuple(x.traversal_kernel) == v)
                                            for k, v in (("p64/p64", (1, 1)), ("per_ray/per_ray", (3, 3)))}},
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
                g = guided_bench()
                print(json.dumps({"metric": "equal-time RMSE vs FP64 oracle, guided / plain", "impl": args.impl,
                                  "value": None if g is None else g["rmse_ratio_equal_time"],
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
