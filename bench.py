"""Benchmark of the GB300 ray path (plain GPU path, one frame per step).

Workload (default "mixed"): the partitioned mixed scene -- a 512^3 fp32
Gaussian-blob volume (64 blobs) in 2x2x2 brick partitions plus 4M spheres of
radius 0.002 (half uniform, half in 32 clusters), 2048x2048, one directional
light, shadows plus 4 AO rays per surface hit, rays handed between partition
queues on the device.  Other workloads: "volume" (256^3, 1024x1024, 0.5-voxel
steps, alpha 0.99) and "triangles" (9 displaced spheres, ~197k triangles,
512x512, shadows).  All inputs are seeded synthetic data.

metric value: rays traced per second (primary + shadow + AO rays of a frame
divided by the frame's device time), whole job over N GPUs; frames are
independent replicas on every GPU ("replicas only": the path is a
single-GPU frame, no collective).  --impl reference times the CPU
restatement of Galaxy's path (oracle/, the only CPU implementation of the
path that builds here) on the host cores, on a bounded band of image rows.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s + p50/p99 frame latency: served vs plain GPU path at RMSE≤1e-3"


def make_workload(name):
    from galaxy_gb300 import scenes
    if name == "mixed":
        cam, vis = scenes.mixed_scene()
        cfg = {"workload": "partitioned mixed scene: 512^3 fp32 blob volume in 2x2x2 bricks + 4M spheres r=0.002, "
                           "2048x2048, shadows + 4 AO rays per hit",
               "image": [2048, 2048], "volume": [512, 512, 512], "spheres": 4_000_000, "partitions": [2, 2, 2],
               "ao_rays": 4, "shadows": True}
    elif name == "volume":
        cam, vis = scenes.volume_scene()
        cfg = {"workload": "volume: 256^3 fp32 blob volume, 1024x1024, 0.5-voxel steps, early termination 0.99",
               "image": [1024, 1024], "volume": [256, 256, 256]}
    elif name == "triangles":
        cam, vis = scenes.triangle_spheres_scene()
        cfg = {"workload": "triangles: 9 displaced UV spheres (~197k triangles), 512x512, directional light, shadows",
               "image": [512, 512], "triangles": int(len(vis.operators[0].dataset.indices))}
    else:
        raise SystemExit("unknown workload " + name)
    return cam, vis, cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(g):
    """Algorithmic bytes of one generation's kernel: 64 B per queue record
    read and written, 128 B per BVH8 node line, 48 B per triangle and 16 B
    per sphere tested, 4 B per volume sample read (march positions in clear
    bricks read no voxels and are left out), 32 B per framebuffer
    contribution (read + write of fp32 RGBA)."""
    return (64 * g["rays_in"] + 64 * g["enqueued"] + 128 * g["nodes"] + 48 * g["tri_tests"] +
            16 * g["sph_tests"] + 4 * (g["samples"] - g.get("samples_skipped", 0)) + 32 * g["terminated"])


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(cam, vis, target_s=15.0, threads=None):
    """The oracle (CPU restatement of Galaxy's path) on a band of image rows
    around the middle of the image, sized to about target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    from galaxy_gb300 import scene as S
    threads = threads or os.cpu_count() or 1
    L = S.resolve_lights(vis.lighting, cam)
    t0 = time.time()
    osc = O.OracleScene(vis)
    setup = time.time() - t0
    mid = cam.height // 2
    rows = max(4, threads)
    # probe band, then size the sample to target_s
    r0 = mid - rows // 2
    t0 = time.time()
    _, c = osc.render(cam, L, nthreads=threads, rows=(r0, r0 + rows))
    dt = max(time.time() - t0, 1e-3)
    rows2 = int(min(cam.height, max(rows, rows * target_s / dt)))
    r0 = max(0, mid - rows2 // 2)
    t0 = time.time()
    _, c = osc.render(cam, L, nthreads=threads, rows=(r0, r0 + rows2))
    dt = time.time() - t0
    rays = c["primary"] + c["shadow"] + c["ao"]
    return {"value": rays / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": "rows %d-%d of %dx%d (%d rays, %.1f s; scene set-up %.1f s excluded)" % (
                r0, r0 + rows2, cam.width, cam.height, rays, dt, setup), "seconds": dt}, osc, L


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    rank, world, local = dist_setup(args.gpus)
    if rank != 0:
        return
    cam, vis, cfg = make_workload(args.workload)
    threads = os.cpu_count() or 1
    per_step = max(2.0, 90.0 / max(1, args.steps + args.warmup))
    # the first call sizes the row band; every step then renders that band
    base, osc, L = cpu_baseline(cam, vis, target_s=per_step, threads=threads)
    band = [int(x) for x in base["sample"].split()[1].split("-")]
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.time()
        _, c = osc.render(cam, L, nthreads=threads, rows=(band[0], band[1]))
        dt = time.time() - t0
        if i >= args.warmup:
            vals.append((c["primary"] + c["shadow"] + c["ao"]) / dt)
            secs.append(dt)
    v = float(np.median(vals))
    base["seconds"] = float(np.median(secs))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["seconds"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "rays/s", "cores": threads, "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving workload: Poisson arrivals over two resident scenes (the
    partitioned mixed scene and a 10M-triangle displaced-sphere mesh); each
    request a random camera on a sphere around the scene and a random light
    direction, image side log-uniform in [256, 4096].  The requests are
    served by the continuous-batching loop and, separately, one at a time
    through the plain path; both report rays/s and p50/p95/p99 latency."""
    import copy
    import torch
    from galaxy_gb300 import gpu, scenes, serve
    from galaxy_gb300 import scene as S
    torch.cuda.set_device(0)
    gpu.init(0)
    cam_m, vis_m = scenes.mixed_scene()
    mesh = scenes.displaced_sphere_mesh(10_000_000)
    L = S.Lighting()
    L.lights, L.types, L.shadows, L.n_ao, L.ao_radius = [(-0.577, -0.577, -0.577)], [0], True, 2, 0.05
    vis_t = S.Visualization([S.TrianglesVis(mesh, colormap=scenes.COOLWARM)], L, box=(0, 0, 0, 1, 1, 1))
    t0 = time.time()
    table = {"mixed": gpu.Scene(vis_m), "mesh": gpu.Scene(vis_t)}
    commit_s = time.time() - t0
    viss = {"mixed": vis_m, "mesh": vis_t}
    lo, hi = args.side_min, args.side_max

    def make(rng, rid, arrival, key, side):
        th, ph = rng.uniform(0.2, 1.3), rng.uniform(0, 2 * np.pi)
        dist = rng.uniform(1.6, 3.0)
        eye = (0.5 + dist * np.sin(th) * np.cos(ph), 0.5 + dist * np.cos(th), 0.5 + dist * np.sin(th) * np.sin(ph))
        cam = S.Camera(eye, (0.5 - eye[0], 0.5 - eye[1], 0.5 - eye[2]), (0, 1, 0), 35.0, side, side)
        lit = copy.copy(viss[key].lighting)
        d = rng.normal(size=3)
        d = -np.abs(d) / np.linalg.norm(d)
        lit.lights, lit.types = [tuple(float(x) for x in d)], [0]
        return serve.Request(rid, arrival, key, cam, S.resolve_lights(lit, cam).c())

    reqs = serve.poisson_requests(args.rate, args.requests, ["mixed", "mesh"], make, side_range=(lo, hi))
    # warm-up (not timed): one small request of each scene on both paths
    warm = [make(np.random.default_rng(1), i, 0.0, k, 256) for i, k in enumerate(["mixed", "mesh"])]
    serve.serve_plain(table, [copy.copy(w) for w in warm])
    slot_pixels = hi * hi
    srv = serve.Server(table, n_slots=args.slots, slot_pixels=slot_pixels, max_jobs=64, max_shadow=1, max_ao=4,
                       fb_budget=16 << 30, use_graph=True, cooperative=args.coop)
    srv.run([copy.copy(w) for w in warm])
    served_reqs = [copy.copy(r) for r in reqs]
    plain_reqs = [copy.copy(r) for r in reqs]
    served = srv.run(served_reqs, time_limit=args.time_limit)
    srv.release()
    torch.cuda.synchronize()
    plain = serve.serve_plain(table, plain_reqs, time_limit=args.time_limit)
    # served vs plain images on a sample of the requests (same camera/light)
    rmse = 0.0
    chk = gpu.Batch(slot_pixels, 8, 1, 4)
    for r in reqs[: min(6, len(reqs))]:
        fa = torch.zeros((r.camera.height, r.camera.width, 4), device="cuda")
        fb_ = torch.zeros_like(fa)
        torch.cuda.synchronize()
        chk.submit([(table[r.scene], r.camera, r.lighting, fa.data_ptr())], use_graph=True, cooperative=args.coop)
        chk.wait(120000)
        table[r.scene].render(r.camera, r.lighting, fb_.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        rmse = max(rmse, float(torch.sqrt(torch.mean((fa[..., :3] - fb_[..., :3]) ** 2)).item()))
    chk.release()
    out = {"metric": METRIC, "value": served["rays_per_s"], "unit": "rays/s", "n_gpus": 1,
           "steps": args.requests, "warmup": len(warm), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": "serving: Poisson %.0f req/s over the partitioned mixed scene and a 10M-triangle "
                                  "mesh, random camera + light per request, image side log-uniform %d..%d"
                                  % (args.rate, lo, hi), "rate": args.rate, "requests": args.requests,
                      "slots": args.slots, "slot_pixels": slot_pixels},
           "served": served, "plain": plain,
           "served_over_plain_rays_per_s": served["rays_per_s"] / max(1e-9, plain["rays_per_s"]),
           "latency_ms": {k: served.get(k + "_ms") for k in ("p50", "p95", "p99")},
           "rmse_served_vs_plain": rmse,
           "scene_commit_s": commit_s}
    print(json.dumps(out), flush=True)


def run_batch(args):
    """Batching workload: 64 render jobs at once over the three plain
    scenes (200k-triangle spheres, 256^3 volume, partitioned mixed scene),
    image side log-uniform in [128, 2048], camera on a sphere of radius
    U[4, 12] around the scene centre (in units of the triangle scene; the
    unit-cube scenes scale it by 1/4), 0-2 shadow/AO levels (none / shadows
    / shadows + 4 AO).  The jobs go through the batching loop (same-scene
    jobs packed into CUDA-graph batch submissions on several slot streams,
    larger frames alone) and, separately, one at a time through the plain
    path; both report rays/s and per-job latency."""
    import copy
    import torch
    from galaxy_gb300 import gpu, scenes, serve
    from galaxy_gb300 import scene as S
    torch.cuda.set_device(0)
    gpu.init(0)
    c0, c1, c2 = scenes.triangle_spheres_scene(), scenes.volume_scene(), scenes.mixed_scene()
    viss = {"triangles": c0[1], "volume": c1[1], "mixed": c2[1]}
    geom = {"triangles": ((0.0, 0.0, 0.0), 1.0), "volume": ((0.5, 0.5, 0.5), 0.25), "mixed": ((0.5, 0.5, 0.5), 0.25)}
    t0 = time.time()
    table = {k: gpu.Scene(v) for k, v in viss.items()}
    commit_s = time.time() - t0
    rng = np.random.Generator(np.random.Philox(11))

    def make(rid, side=None):
        key = ["triangles", "volume", "mixed"][int(rng.integers(0, 3))]
        if side is None:
            side = int(round(np.exp(rng.uniform(np.log(128), np.log(2048)))))
        (cx, cy, cz), scale = geom[key]
        th, ph = rng.uniform(0.3, 2.8), rng.uniform(0, 2 * np.pi)
        rad = rng.uniform(4.0, 12.0) * scale
        eye = (cx + rad * np.sin(th) * np.cos(ph), cy + rad * np.cos(th), cz + rad * np.sin(th) * np.sin(ph))
        cam = S.Camera(eye, (cx - eye[0], cy - eye[1], cz - eye[2]), (0, 1, 0), 45.0, side, side)
        lit = copy.copy(viss[key].lighting)
        level = int(rng.integers(0, 3))
        lit.lights, lit.types = [(-0.577, -0.577, -0.577)], [0]
        lit.shadows, lit.n_ao = level >= 1, (4 if level == 2 else 0)
        lit.ao_radius = 0.1 * scale * 4
        return serve.Request(rid, 0.0, key, cam, S.resolve_lights(lit, cam).c())

    jobs = [make(j) for j in range(args.jobs)]
    warm = [make(1000 + j, 256) for j in range(6)]
    slot_pixels = 2048 * 2048
    n_slots = max(args.slots, 4)   # 4-8 slot streams measured alike (1.60-1.62x), 2 slower (1.52x)
    srv = serve.Server(table, n_slots=n_slots, slot_pixels=slot_pixels, max_jobs=64, max_shadow=1, max_ao=4,
                       fb_budget=16 << 30, use_graph=True, small_pixels=1 << 20, small_batch_pixels=4 << 20)
    serve.serve_plain(table, [copy.copy(w) for w in warm])
    srv.run([copy.copy(w) for w in warm])
    batched = srv.run([copy.copy(r) for r in jobs], time_limit=args.time_limit)
    srv.release()
    torch.cuda.synchronize()
    plain = serve.serve_plain(table, [copy.copy(r) for r in jobs], time_limit=args.time_limit)
    out = {"metric": "rays/s: batched vs plain GPU path (64 uneven jobs)", "value": batched["rays_per_s"],
           "unit": "rays/s", "n_gpus": 1, "steps": args.jobs, "warmup": len(warm), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": "batching: %d jobs over the triangle, volume and mixed scenes, image side "
                                  "log-uniform 128..2048, 0-2 shadow/AO levels" % args.jobs,
                      "slots": n_slots, "slot_pixels": slot_pixels, "pixels": int(sum(r.pixels for r in jobs))},
           "batched": batched, "plain": plain,
           "batched_over_plain_rays_per_s": batched["rays_per_s"] / max(1e-9, plain["rays_per_s"]),
           "latency_ms": {k: batched.get(k + "_ms") for k in ("p50", "p95", "p99")},
           "scene_commit_s": commit_s}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed", choices=["mixed", "volume", "triangles"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--image", type=int, default=0, help="override the image side (smaller profiling cases)")
    ap.add_argument("--mode", default="frame", choices=["frame", "serve", "batch"])
    ap.add_argument("--jobs", type=int, default=64, help="batch mode: number of render jobs")
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--side-min", type=int, default=256)
    ap.add_argument("--side-max", type=int, default=4096)
    ap.add_argument("--time-limit", type=float, default=120.0)
    ap.add_argument("--coop", action="store_true", help="serve with cooperative single-launch batches")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the autotuner (occupancy, grid size, split tracing) before timing")
    ap.add_argument("--tune", default="", help="fixed tuning 'blocks_per_sm,grid_per_sm,split' (implies --no-autotune)")
    ap.add_argument("--leaf-max", type=int, default=0, help="primitives per BVH8 leaf (1-4; 0: library default)")
    ap.add_argument("--trav-steps", type=int, default=0, help="node visits per refill round (0: library default)")
    ap.add_argument("--march-steps", type=int, default=0, help="samples per refill round (0: library default)")
    ap.add_argument("--skip-clear", type=int, default=-1,
                    help="empty-space skipping flags at scene commit: 1 on, 0 off (-1: library default)")
    ap.add_argument("--skip-mode", type=int, default=-1,
                    help="clear-brick skipping bits: 1 camera-ray runs, 2 shadow/AO skipping, 4 shadow/AO runs "
                         "(-1: library default)")
    ap.add_argument("--bvh", default="", help="BVH binary tree: 'lbvh' (radix tree), 'sah' (binned-SAH top over "
                                                "radix clusters of 256) or 'sah:C' (clusters of C); default: library")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "serve":
        return run_serve(args)
    if args.mode == "batch":
        return run_batch(args)
    args.warmup = max(3, args.warmup)

    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from galaxy_gb300 import _abi as A
    from galaxy_gb300 import autotune
    from galaxy_gb300 import gpu
    from galaxy_gb300 import scene as S

    cam, vis, cfg = make_workload(args.workload)
    if args.bvh:
        gpu.set_tuning(gpu.TUNE_BVH_SAH, 0 if args.bvh == "lbvh" else
                       (int(args.bvh.split(":")[1]) if ":" in args.bvh else 1))
    if args.leaf_max:
        gpu.set_tuning(gpu.TUNE_LEAF_MAX, args.leaf_max)
    if args.skip_clear >= 0:
        gpu.set_tuning(gpu.TUNE_SKIP_CLEAR, args.skip_clear)
    if args.trav_steps:
        gpu.set_tuning(gpu.TUNE_TRAV_STEPS, args.trav_steps)
    if args.march_steps:
        gpu.set_tuning(gpu.TUNE_MARCH_STEPS, args.march_steps)
    if args.skip_mode >= 0:
        gpu.set_tuning(gpu.TUNE_SKIP_MODE, args.skip_mode)
    cfg = dict(cfg, bvh_sah_clusters=gpu.get_tuning(gpu.TUNE_BVH_SAH), leaf_max=gpu.get_tuning(gpu.TUNE_LEAF_MAX),
               skip_clear=gpu.get_tuning(gpu.TUNE_SKIP_CLEAR),
               trav_steps=gpu.get_tuning(gpu.TUNE_TRAV_STEPS), march_steps=gpu.get_tuning(gpu.TUNE_MARCH_STEPS))
    if args.image:
        cam.width = cam.height = args.image
        cfg = dict(cfg, image=[args.image, args.image], workload=cfg["workload"] + " (image %d^2)" % args.image)
    gpu.init(local)
    L = S.resolve_lights(vis.lighting, cam)
    cam_c = cam.c()
    bvh_tuning = None
    t0 = time.time()
    if args.autotune and not args.tune and not args.bvh:
        # scene-level knob first: radix-tree BVH or binned-SAH top over clusters of 64
        sc, v, bvh_out = autotune.tune_bvh(vis, cam_c, L, values=(0, 64))
        bvh_tuning = {"bvh_sah_clusters": v, "ms_per_frame": dict(bvh_out)}
        cfg = dict(cfg, bvh_sah_clusters=v)
    else:
        sc = gpu.Scene(vis)
    commit_s = time.time() - t0
    stream = torch.cuda.current_stream()
    fb = torch.zeros((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")

    def frame():
        fb.zero_()
        sc.render(cam_c, L, fb.data_ptr(), stream.cuda_stream)

    tuning = None
    if args.tune:
        vals = [int(x) for x in args.tune.split(",")] + [1]
        gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, vals[0])
        gpu.set_tuning(gpu.TUNE_GRID_PER_SM, vals[1])
        gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, vals[2])
        gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, vals[3])
    elif args.autotune:
        tuning = autotune.tune(sc, cam_c, L, frames=4)
    sc.set_profiling(True)
    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    c = sc.counters()
    rays_per_frame = c["primary_rays"] + c["shadow_rays"] + c["ao_rays"]

    # ---- timed region: K frames, per-frame events, clocks sampled
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    gen_ms, gen_bytes = {}, {}
    launches = 0
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        frame()
        ev[k][1].record(stream)
        gens = sc.generations()
        launches += len(gens)
        for g in gens:
            gen_ms.setdefault(g["kind"], []).append(g["ms"])
            gen_bytes.setdefault(g["kind"], []).append(algorithmic_bytes(g))
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    sc_last_gens = sc.generations()
    total_ms = t_start.elapsed_time(t_end)
    frame_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = allreduce_max(total_ms, world)
    value = rays_per_frame * args.steps * world / (total_ms / 1e3)

    # ---- end to end through the host-framebuffer C ABI call
    host_fb = torch.empty((cam.height, cam.width, 4), dtype=torch.float32, pin_memory=True).numpy()
    sc.set_profiling(False)
    sc.render_host(cam_c, L, out=host_fb, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sc.render_host(cam_c, L, out=host_fb, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e2e_s = allreduce_max(time.perf_counter() - t0, world)
    e2e = {"value": rays_per_frame * e2e_steps * world / e2e_s, "unit": "rays/s",
           "h2d_bytes_per_step": int(ctypes_size(A.gxy_camera) + ctypes_size(A.gxy_lighting)),
           "d2h_bytes_per_step": int(host_fb.nbytes)}

    # ---- roofline of the dominant kernel (largest share of device time);
    # achieved = algorithmic bytes of its launches / their event time
    dom = max(gen_ms, key=lambda g: sum(gen_ms[g]))
    dom_ms = float(np.mean(gen_ms[dom]))
    dom_bytes = float(np.mean(gen_bytes[dom]))
    peak, peak_kind = measured_peaks()
    achieved = sum(gen_bytes[dom]) / (sum(gen_ms[dom]) / 1e3) / 1e9
    share = sum(gen_ms[dom]) / max(1e-9, sum(sum(v) for v in gen_ms.values()))
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic_%s.json" % args.workload)
    if os.path.exists(tf):
        t = json.load(open(tf))
        traffic = t.get("bytes_per_launch")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": peak_kind,
            "kernel": ["k_cam_query" if gpu.get_tuning(gpu.TUNE_SPLIT_PRIMARY) else "k_primary<camera>",
                       "k_primary<queue>",
                       "k_sec_query" if gpu.get_tuning(gpu.TUNE_SPLIT_SECONDARY) else "k_secondary",
                       "k_sec_march", "k_prim_march"][dom],
            "kernel_ms": dom_ms, "algorithmic_bytes": dom_bytes, "share_of_frame_kernel_time": share}

    out = {"metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": dict(cfg, l2="inputs larger than L2 (volume 512 MiB + spheres)" if args.workload == "mixed"
                          else "L2 not flushed; working set may be L2-resident", parallelism="replicas"),
           "latency_ms": {"p50": float(np.percentile(frame_ms, 50)), "p95": float(np.percentile(frame_ms, 95)),
                          "p99": float(np.percentile(frame_ms, 99))},
           "rays_per_frame": rays_per_frame,
           "rays": {"primary": c["primary_rays"], "shadow": c["shadow_rays"], "ao": c["ao_rays"],
                    "segments": c["segments"], "handoffs": c["handoffs"], "generations": c["bounces"],
                    "samples": c["samples"], "samples_skipped": c["samples_skipped"], "bvh_nodes": c["nodes"],
                    "prim_tests": c["prim_tests"]},
           "generations": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in g.items()}
                           for g in sc_last_gens],
           "scene_commit_s": commit_s, "bvh": sc.bvh_info(),
           "gpu_launches": launches, "roofline": roof, "e2e": e2e, "clocks": clk,
           "tuning": dict(tuning if tuning else {"best": autotune.current()}, bvh=bvh_tuning)}
    if rank == 0 and not args.no_cpu_baseline:
        base, _, _ = cpu_baseline(cam, vis, target_s=args.cpu_seconds)
        base.pop("seconds", None)
        out["cpu_baseline"] = base
    if rank == 0:
        print(json.dumps(out), flush=True)


def ctypes_size(t):
    import ctypes
    return ctypes.sizeof(t)


if __name__ == "__main__":
    main()
