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


def dram_roofline(frame_traffic, kernel_ms, kernel_bytes, frames, peak):
    """DRAM-measured roofline of the dominant kernel: the DRAM bytes ncu
    measured for its launches of one frame (frame_traffic) over its CUDA-event
    time per frame (kernel_ms: its launch times over `frames` frames).  Both
    are taken per frame, so the figure does not depend on how many launches
    a frame has; bytes_per_launch is the per-launch mean, beside the
    algorithmic bytes (kernel_bytes: per launch, the same launches)."""
    frames = max(1, frames)
    launches = max(1e-9, len(kernel_ms) / frames)
    frame_ms = sum(kernel_ms) / frames
    gbs = frame_traffic / (frame_ms / 1e3) / 1e9
    return {"achieved": gbs, "frac": gbs / peak, "bytes_per_frame": frame_traffic,
            "bytes_per_launch": frame_traffic / launches,
            "traffic_over_algorithmic": frame_traffic / (sum(kernel_bytes) / frames)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(cam, vis, target_s=10.0, threads=None):
    """The oracle (CPU restatement of Galaxy's path) on the host cores:
    whole frames of the workload, repeated until about target_s seconds of
    CPU work.  Returns the baseline record, the oracle scene, the resolved
    lighting and the first frame (the parity reference of the GPU frame)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    from galaxy_gb300 import scene as S
    threads = threads or os.cpu_count() or 1
    L = S.resolve_lights(vis.lighting, cam)
    t0 = time.time()
    osc = O.OracleScene(vis)
    setup = time.time() - t0
    frames, rays, dt, first, counts = 0, 0, 0.0, None, None
    while frames == 0 or (dt < target_s and frames < 50):
        t0 = time.time()
        fb, c = osc.render(cam, L, nthreads=threads)
        dt += time.time() - t0
        if first is None:
            first, counts = fb, c
        frames += 1
        rays += c["primary"] + c["shadow"] + c["ao"]
    return {"value": rays / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": "%d whole %dx%d frame(s), %d rays, %.1f s (scene set-up %.1f s excluded)" % (
                frames, cam.width, cam.height, rays, dt, setup), "seconds": dt / frames,
            "frames": frames}, osc, L, first, counts


PARITY_RMSE = 1e-3      # image RMSE bound of the workloads (RGB, fp32 framebuffer)
PARITY_CH = 2.0 / 255   # per-channel bound, met by 99.9 % of channels


def parity(img, ref, gpu_counts, ref_counts):
    """GPU frame against the oracle frame of the same camera and lighting."""
    d = np.abs(img[..., :3].astype(np.float64) - ref[..., :3].astype(np.float64))
    rmse = float(np.sqrt(np.mean(d ** 2)))
    within = float(np.mean(d <= PARITY_CH))
    q = lambda a: (np.trunc(255.0 * a.astype(np.float32)).astype(np.int64) & 0xff)   # ColorImageWriter bytes
    dq = np.abs(q(img[..., :3]) - q(ref[..., :3]))
    rays = {"gpu": {k: int(gpu_counts[k + "_rays"]) for k in ("primary", "shadow", "ao")},
            "oracle": {k: int(ref_counts[k]) for k in ("primary", "shadow", "ao")}}
    return {"against": "oracle frame of the same camera and lighting (whole image)",
            "rmse": rmse, "max_abs": float(d.max()), "frac_within_2_255": within,
            "png_bytes_equal": float(np.mean(dq == 0)), "png_max_byte_diff": int(dq.max()),
            "rays": rays, "tolerance": {"rmse": PARITY_RMSE, "channel": PARITY_CH, "channel_frac": 0.999},
            "pass": bool(rmse <= PARITY_RMSE and within >= 0.999)}


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
    if args.image:
        cam.width = cam.height = args.image
        cfg = dict(cfg, image=[args.image, args.image], workload=cfg["workload"] + " (image %d^2)" % args.image)
    threads = os.cpu_count() or 1
    # every step renders the whole frame of the workload on all host cores
    base, osc, L, _, _ = cpu_baseline(cam, vis, target_s=0.0, threads=threads)
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.time()
        _, c = osc.render(cam, L, nthreads=threads)
        dt = time.time() - t0
        if i >= args.warmup:
            vals.append((c["primary"] + c["shadow"] + c["ao"]) / dt)
            secs.append(dt)
    v = float(np.median(vals))
    sample = "whole %dx%d frame per step (%d steps, median)" % (cam.width, cam.height, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median(secs)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "rays/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serve_table(vis_m=None, sc_m=None):
    """The serving workload's resident scenes: the partitioned mixed scene
    (committed here unless given) and a 10M-triangle displaced-sphere mesh;
    returns (scene table, visualizations, commit seconds)."""
    from galaxy_gb300 import gpu, scenes
    from galaxy_gb300 import scene as S
    t0 = time.time()
    if vis_m is None:
        vis_m = scenes.mixed_scene()[1]
    mesh = scenes.displaced_sphere_mesh(10_000_000)
    L = S.Lighting()
    L.lights, L.types, L.shadows, L.n_ao, L.ao_radius = [(-0.577, -0.577, -0.577)], [0], True, 2, 0.05
    vis_t = S.Visualization([S.TrianglesVis(mesh, colormap=scenes.COOLWARM)], L, box=(0, 0, 0, 1, 1, 1))
    table = {"mixed": sc_m if sc_m is not None else gpu.Scene(vis_m), "mesh": gpu.Scene(vis_t)}
    return table, {"mixed": vis_m, "mesh": vis_t}, time.time() - t0


def serve_compare(table, viss, rate, n_requests, side_min=256, side_max=4096, slots=3, coop=False,
                  time_limit=120.0, check=6):
    """Poisson arrivals at `rate` over the resident scenes; each request a
    random camera on a sphere around the scene plus, with probability 1/3
    each, a random transfer-function change or a random light direction;
    image side log-uniform in [side_min, side_max].  The requests are served
    by the continuous-batching loop and, separately, one at a time through
    the plain path; both report rays/s and p50/p95/p99 latency, and the
    images of `check` requests are compared between the two paths."""
    import copy
    import torch
    from galaxy_gb300 import gpu, scenes, serve
    from galaxy_gb300 import scene as S

    def random_tf(rng, key):
        if key == "mixed":
            op = copy.copy(viss[key].operators[0])
            a = float(rng.uniform(0.1, 0.5))
            op.opacitymap = [(0.0, 0.0), (a, 0.0), (1.0, float(rng.uniform(0.4, 1.0)))]
            op.colormap = [tuple([c[0]] + list(np.roll(c[1:], int(rng.integers(0, 3))))) for c in op.colormap]
            return [(gpu.VIS_VOLUME, 0, op.tf())]
        op = copy.copy(viss[key].operators[0])
        op.colormap = [(c[0],) + tuple(float(x) for x in rng.uniform(0, 1, 3)) for c in op.colormap]
        return [(gpu.VIS_TRIANGLES, 0, op.tf())]

    def make(rng, rid, arrival, key, side):
        th, ph = rng.uniform(0.2, 1.3), rng.uniform(0, 2 * np.pi)
        dist = rng.uniform(1.6, 3.0)
        eye = (0.5 + dist * np.sin(th) * np.cos(ph), 0.5 + dist * np.cos(th), 0.5 + dist * np.sin(th) * np.sin(ph))
        cam = S.Camera(eye, (0.5 - eye[0], 0.5 - eye[1], 0.5 - eye[2]), (0, 1, 0), 35.0, side, side)
        lit = copy.copy(viss[key].lighting)
        change = int(rng.integers(0, 3))      # 0 camera only, 1 + transfer function, 2 + light
        tf = random_tf(rng, key) if change == 1 else None
        if change == 2:
            d = rng.normal(size=3)
            d = -np.abs(d) / np.linalg.norm(d)
            lit.lights, lit.types = [tuple(float(x) for x in d)], [0]
        return serve.Request(rid, arrival, key, cam, S.resolve_lights(lit, cam).c(), tf=tf)

    defaults = {"mixed": [(gpu.VIS_VOLUME, 0, viss["mixed"].operators[0].tf()),
                          (gpu.VIS_PARTICLES, 0, viss["mixed"].operators[1].tf())],
                "mesh": [(gpu.VIS_TRIANGLES, 0, viss["mesh"].operators[0].tf())]}
    keys = sorted(table)
    reqs = serve.poisson_requests(rate, n_requests, keys, make, side_range=(side_min, side_max))
    # warm-up (not timed): small requests of each scene on both paths, with and without a TF change
    wr = np.random.Generator(np.random.Philox(1))
    warm = [make(wr, 10_000 + i, 0.0, k, 256) for i, k in enumerate(keys * 3)]
    serve.serve_plain(table, [copy.copy(w) for w in warm], default_tfs=defaults)
    slot_pixels = side_max * side_max
    srv = serve.Server(table, n_slots=slots, slot_pixels=slot_pixels, max_jobs=64, max_shadow=1, max_ao=4,
                       fb_budget=16 << 30, use_graph=True, cooperative=coop)
    srv.run([copy.copy(w) for w in warm])
    keep = {r.id for r in reqs if r.camera.width <= 2048}
    keep = set(sorted(keep)[:check])
    served_reqs = [copy.copy(r) for r in reqs]
    plain_reqs = [copy.copy(r) for r in reqs]
    served = srv.run(served_reqs, time_limit=time_limit, keep=keep)
    srv.release()
    torch.cuda.synchronize()
    plain = serve.serve_plain(table, plain_reqs, time_limit=time_limit, keep=keep, default_tfs=defaults)
    rmse, max_abs, checked = 0.0, 0.0, 0
    for a, b in zip(served_reqs, plain_reqs):
        if a.id in keep and a.fb is not None and b.fb is not None:
            d = np.abs(a.fb[..., :3] - b.fb[..., :3])
            rmse = max(rmse, float(np.sqrt(np.mean(d ** 2))))
            max_abs = max(max_abs, float(d.max()))
            checked += 1
    kinds = {"camera": sum(1 for r in reqs if r.tf is None), "transfer_function": sum(1 for r in reqs if r.tf)}
    return {"rate": rate, "requests": n_requests, "slots": slots, "slot_pixels": slot_pixels,
            "side_range": [side_min, side_max], "request_kinds": kinds,
            "served": served, "plain": plain,
            "served_over_plain_rays_per_s": served["rays_per_s"] / max(1e-9, plain["rays_per_s"]),
            "latency_ms": {"served": {k: served.get(k + "_ms") for k in ("p50", "p95", "p99")},
                           "plain": {k: plain.get(k + "_ms") for k in ("p50", "p95", "p99")}},
            "images_served_vs_plain": {"requests": checked, "max_rmse": rmse, "max_abs": max_abs,
                                       "pass": bool(checked > 0 and rmse <= PARITY_RMSE)}}


def run_serve(args):
    """Serving workload (--mode serve): Poisson arrivals over the partitioned
    mixed scene and a 10M-triangle mesh, served by the continuous-batching
    loop and one at a time through the plain path."""
    import torch
    from galaxy_gb300 import gpu
    torch.cuda.set_device(0)
    gpu.init(0)
    table, viss, commit_s = serve_table()
    res = serve_compare(table, viss, args.rate, args.requests, args.side_min, args.side_max, args.slots,
                        args.coop, args.time_limit)
    served = res["served"]
    out = {"metric": METRIC, "value": served["rays_per_s"], "unit": "rays/s", "n_gpus": 1,
           "steps": args.requests, "warmup": 6, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": "serving: Poisson %.0f req/s over the partitioned mixed scene and a 10M-triangle "
                                  "mesh, random camera + transfer-function or light change per request, image side "
                                  "log-uniform %d..%d" % (args.rate, args.side_min, args.side_max),
                      "rate": args.rate, "requests": args.requests, "slots": args.slots},
           "served_vs_plain": res, "scene_commit_s": commit_s}
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
    n_slots = args.batch_slots
    small, small_batch = args.small_pixels, args.small_batch_pixels
    srv = serve.Server(table, n_slots=n_slots, slot_pixels=max(slot_pixels, small_batch), max_jobs=64, max_shadow=1,
                       max_ao=4, fb_budget=16 << 30, use_graph=True, small_pixels=small,
                       small_batch_pixels=small_batch)
    serve.serve_plain(table, [copy.copy(w) for w in warm])
    srv.run([copy.copy(w) for w in warm])
    batched = srv.run([copy.copy(r) for r in jobs], time_limit=args.time_limit)
    srv.release()
    torch.cuda.synchronize()
    plain = serve.serve_plain(table, [copy.copy(r) for r in jobs], time_limit=args.time_limit)
    single = single_launch(table, jobs)
    chosen = "packed" if batched["rays_per_s"] >= single["rays_per_s"] else "single_launch"
    best = batched if chosen == "packed" else single
    out = {"metric": "rays/s: batched vs plain GPU path (64 uneven jobs)", "value": best["rays_per_s"],
           "unit": "rays/s", "n_gpus": 1, "steps": args.jobs, "warmup": len(warm), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": "batching: %d jobs over the triangle, volume and mixed scenes, image side "
                                  "log-uniform 128..2048, 0-2 shadow/AO levels" % args.jobs,
                      "slots": n_slots, "slot_pixels": max(slot_pixels, small_batch), "small_pixels": small,
                      "small_batch_pixels": small_batch, "pixels": int(sum(r.pixels for r in jobs))},
           "batched": batched, "single_launch": single, "plain": plain, "chosen": chosen,
           "batched_over_plain_rays_per_s": best["rays_per_s"] / max(1e-9, plain["rays_per_s"]),
           "latency_ms": {k: best.get(k + "_ms") for k in ("p50", "p95", "p99")},
           "scene_commit_s": commit_s}
    print(json.dumps(out), flush=True)


def single_launch(table, jobs, repeats=3):
    """All jobs in ONE batch submission: one wavefront launch per generation
    over every job's rays (jobs of the three scenes together), replayed as a
    CUDA graph; framebuffers cleared and the graph run `repeats` times, the
    median makespan kept.  Every job completes with the submission."""
    import torch
    from galaxy_gb300 import gpu
    pix = sum(r.pixels for r in jobs)
    b = gpu.Batch(max_pixels=pix, max_jobs=len(jobs), max_shadow=1, max_ao=4)
    fbs = [torch.zeros((r.camera.height, r.camera.width, 4), device="cuda") for r in jobs]
    spec = [(table[r.scene], r.camera, r.lighting, fb.data_ptr()) for r, fb in zip(jobs, fbs)]
    times = []
    for k in range(repeats + 1):
        for fb in fbs:
            fb.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.submit(spec, use_graph=True)
        b.wait(600000)
        dt = time.perf_counter() - t0
        if k:
            times.append(dt)
    c = b.counters()
    b.release()
    rays = c["primary_rays"] + c["shadow_rays"] + c["ao_rays"]
    ms = float(np.median(times))
    return {"requests": len(jobs), "completed": len(jobs), "makespan_s": ms, "rays": float(rays),
            "rays_per_s": rays / ms, "p50_ms": ms * 1e3, "p95_ms": ms * 1e3, "p99_ms": ms * 1e3,
            "generations": c["bounces"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed", choices=["mixed", "volume", "triangles"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--image", type=int, default=0, help="override the image side (smaller profiling cases)")
    ap.add_argument("--mode", default="frame", choices=["frame", "serve", "batch"])
    ap.add_argument("--jobs", type=int, default=64, help="batch mode: number of render jobs")
    # packing measured best of 3/1M/4M, 4/4M/16M, 3/4M/64M, 8/1M/4M, 6/256k/2M (1.55-1.72x)
    ap.add_argument("--batch-slots", type=int, default=3, help="batch mode: slot streams")
    ap.add_argument("--small-pixels", type=int, default=4 << 20,
                    help="batch mode: jobs up to this many pixels are packed together")
    ap.add_argument("--small-batch-pixels", type=int, default=64 << 20,
                    help="batch mode: pixels per packed submission")
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--side-min", type=int, default=256)
    ap.add_argument("--side-max", type=int, default=4096)
    ap.add_argument("--time-limit", type=float, default=120.0)
    ap.add_argument("--coop", action="store_true", help="serve with cooperative single-launch batches")
    ap.add_argument("--serve-rate", type=float, default=800.0,
                    help="frame mode: arrival rate of the bounded served-vs-plain comparison")
    ap.add_argument("--serve-requests", type=int, default=60,
                    help="frame mode: requests of the served-vs-plain comparison (0: skip it)")
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
    sc.set_profiling(False)
    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    c = sc.counters()
    rays_per_frame = c["primary_rays"] + c["shadow_rays"] + c["ao_rays"]

    # ---- timed region: K frames, per-frame events, clocks sampled; the
    # per-launch statistics are off here (their event records and reads
    # would be timed too) and are taken over K more frames below
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        frame()
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)

    # ---- per-launch device time and counters of K profiled frames (events
    # around every launch on its stream): the roofline's kernel time
    sc.set_profiling(True)
    frame()
    torch.cuda.synchronize()
    gen_ms, gen_bytes = {}, {}
    launches = 0
    for k in range(args.steps):
        frame()
        gens = sc.generations()
        launches += len(gens)
        for g in gens:
            # launches of handed-off primaries run on a side stream beside
            # the shadow/AO passes; their event time includes waiting for
            # SMs, so they are reported but not ranked for the roofline
            if g["kind"] in (1, 5) or (g["kind"] == 4 and g["generation"] > 0):
                continue
            gen_ms.setdefault(g["kind"], []).append(g["ms"])
            gen_bytes.setdefault(g["kind"], []).append(algorithmic_bytes(g))
    torch.cuda.synchronize()
    sc_last_gens = sc.generations()
    sc.set_profiling(False)
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
    share = sum(gen_ms[dom]) / max(1e-9, sum(sum(v) for v in gen_ms.values()))   # of the main stream's kernel time
    # measured DRAM traffic of the dominant kernel (ncu, profiles/): the
    # fraction of HBM bandwidth it actually moves, beside the model's
    traffic, dram, binding = None, None, None
    tf = os.path.join(ROOT, "profiles", "traffic_%s.json" % args.workload)
    if os.path.exists(tf) and not args.image:
        t = json.load(open(tf))
        frame_traffic = t.get("bytes_per_frame")
        binding = t.get("binding")
        if frame_traffic:
            dram = dram_roofline(frame_traffic, gen_ms[dom], gen_bytes[dom], args.steps, peak)
            dram["measured_at"] = t.get("measured_at")
            traffic = dram["bytes_per_launch"]   # per launch, like `achieved`
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "dram": dram, "binding": binding, "peak_source": peak_kind,
            "model": "algorithmic bytes (64 B per record read and written, 128 B per node line, 16 B per sphere "
                     "and 48 B per triangle tested, 4 B per voxel sample read, 32 B per pixel update) over "
                     "the kernel's CUDA-event time; most node and voxel bytes are L1/L2 hits (dram.frac is the "
                     "DRAM-measured fraction)",
            "kernel": ["k_cam_query" if gpu.get_tuning(gpu.TUNE_SPLIT_PRIMARY) else "k_primary<camera>",
                       "k_primary<queue>",
                       "k_sec_query" if gpu.get_tuning(gpu.TUNE_SPLIT_SECONDARY) else "k_secondary",
                       "k_sec_march", "k_prim_march", "k_prim_query"][dom],
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
    # ---- the metric's served-vs-plain comparison (bounded serving run over
    # this scene and a 10M-triangle mesh)
    if rank == 0 and args.workload == "mixed" and args.serve_requests > 0 and not args.image:
        table, viss, _ = serve_table(vis_m=vis, sc_m=sc)
        out["served_vs_plain"] = serve_compare(table, viss, args.serve_rate, args.serve_requests)
        table["mesh"].release()
        del table
    parity_ok = True
    if rank == 0 and not args.no_cpu_baseline:
        base, _, _, ref_img, ref_counts = cpu_baseline(cam, vis, target_s=args.cpu_seconds)
        base.pop("seconds", None)
        out["cpu_baseline"] = base
        # the last end-to-end frame (host framebuffer) against the oracle's
        out["parity"] = parity(host_fb, ref_img, c, ref_counts)
        parity_ok = out["parity"]["pass"]
    if rank == 0:
        print(json.dumps(out), flush=True)
    if not parity_ok:
        sys.exit("parity failed: GPU frame differs from the oracle frame beyond the stated tolerance")


def ctypes_size(t):
    import ctypes
    return ctypes.sizeof(t)


if __name__ == "__main__":
    main()
