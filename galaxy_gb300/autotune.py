"""Autotuner for the wavefront kernels.

Measures a short run of real frames of the caller's scene per candidate
setting and keeps the fastest, one knob at a time (coordinate descent,
repeated while a pass still changes something):

  * register budget / occupancy: the frame kernels compiled for 2 resident
    blocks per SM (128 registers, no spills) or 3 (80 registers, some
    spills to L1-resident local memory; the refill queries then run at 4);
  * grid-stride grid size: 8, 16 or 32 blocks per SM;
  * split shadow/AO tracing: one combined kernel, or a query pass plus a
    march pass whose lanes refill from the march queue (volume scenes);
  * split camera-ray tracing, likewise;
  * camera-ray traversal per thread (per-lane refill) or per warp (one
    shared traversal for an 8x4 pixel tile);
  * shadow/AO traversal per thread (per-lane refill) or per warp (one
    shared traversal for 32 consecutive queue records);
  * traversal round of the refill queries: BVH8 node visits per refill
    round;
  * queue chunk of the shadow/AO query: records a block takes from the ray
    queue at once (1k-64k; as needed when 0);
  * march tiling: volume samples per refill round of the march passes;
  * clear-brick skipping: fast runs in the camera-ray march, skipping (and
    fast runs) in the shadow/AO march, the occlusion shortcut of the
    shadow/AO query.

tune_bvh() picks the scene-level BVH builder (radix tree, or a binned-SAH
top over radix-tree clusters) by committing the scene with each.

Frames are timed with CUDA events on the render stream after one warm-up
frame per setting.  The result can be cached in a JSON file keyed by GPU
name and workload.
"""
import json
import os

from . import gpu

KNOBS = (
    ("blocks_per_sm", gpu.TUNE_BLOCKS_PER_SM, (2, 3)),
    ("grid_per_sm", gpu.TUNE_GRID_PER_SM, (8, 16, 32)),
    ("split", gpu.TUNE_SPLIT_SECONDARY, (0, 1)),
    ("split_primary", gpu.TUNE_SPLIT_PRIMARY, (0, 1)),
    ("camera_packet", gpu.TUNE_CAMERA_PACKET, (0, 1)),
    ("sec_packet", gpu.TUNE_SEC_PACKET, (0, 1)),
    ("trav_steps", gpu.TUNE_TRAV_STEPS, (4, 8, 16)),
    ("queue_chunk", gpu.TUNE_QUEUE_CHUNK, (0, 1024, 4096, 16384, 65536)),
    ("march_steps", gpu.TUNE_MARCH_STEPS, (8, 16, 32, 64)),
    ("skip_mode", gpu.TUNE_SKIP_MODE, (0, 1, 3, 7, 9, 11)),
    ("runahead", gpu.TUNE_RUNAHEAD, (1, 2, 4, 8)),
    ("query_blocks", gpu.TUNE_QUERY_BLOCKS, (3, 4)),
    ("pmarch_blocks", gpu.TUNE_PMARCH_BLOCKS, (2, 3)),
    ("pquery_blocks", gpu.TUNE_PQUERY_BLOCKS, (2, 4)),
    ("continue", gpu.TUNE_CONTINUE, (0, 1)),
)


def current():
    return {name: gpu.get_tuning(knob) for name, knob, _ in KNOBS}


def apply(setting):
    for name, knob, _ in KNOBS:
        if name in setting:
            gpu.set_tuning(knob, int(setting[name]))


def descend(measure, start, knobs=KNOBS, passes=2, min_gain=0.0):
    """Coordinate descent: from the setting `start` (knob name -> value),
    try every other value of one knob at a time, keep a change when
    measure(setting) -- a time, lower is better -- improves by more than the
    fraction `min_gain` (a change within timing noise is not taken), and
    repeat the sweep while a pass still changes something (at most `passes`
    sweeps).  Each distinct setting is measured once.  Returns (best
    setting, its time, [setting with ms_per_frame, ...] in measurement
    order)."""
    measured = {}
    results = []

    def cost(setting):
        key = tuple(sorted(setting.items()))
        if key not in measured:
            measured[key] = measure(setting)
            results.append(dict(setting, ms_per_frame=measured[key]))
        return measured[key]

    best = dict(start)
    best_ms = cost(best)
    for _ in range(passes):
        changed = False
        for name, _, values in knobs:
            for v in values:
                if v == best[name]:
                    continue
                cand = dict(best, **{name: v})
                ms = cost(cand)
                if ms < best_ms * (1.0 - min_gain):
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    return best, best_ms, results


def tune(scene, camera, lighting, frames=3, passes=2, knobs=KNOBS, verbose=False, target_ms=30.0, min_gain=0.005):
    """descend() over real frames of the caller's scene, timed with CUDA
    events on the render stream after one warm-up frame per setting; leaves
    the library set to the best setting.  Each setting is timed over at
    least `frames` frames and at least `target_ms` of rendering (short
    frames are dominated by launch and host gaps, so a few of them time
    noise), a change is kept only when it gains more than `min_gain`, and
    the winner is timed once more against the starting setting over twice
    the frames before it is kept."""
    import math
    import torch
    stream = torch.cuda.current_stream()
    cam = camera.c() if hasattr(camera, "c") else camera
    fb = torch.zeros((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")

    def timed(setting, n):
        apply(setting)
        fb.zero_()
        scene.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fb.zero_()
            scene.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    start = current()
    n_frames = max(1, frames, int(math.ceil(target_ms / max(timed(start, frames), 1e-3))))

    def measure(setting):
        ms = timed(setting, n_frames)
        if verbose:
            print("autotune", dict(setting, ms_per_frame=ms), flush=True)
        return ms

    best, best_ms, results = descend(measure, start, knobs, passes, min_gain)
    if best != start:
        ms_best, ms_start = timed(best, 2 * n_frames), timed(start, 2 * n_frames)
        if ms_start <= ms_best:
            best, best_ms = start, ms_start
        else:
            best_ms = ms_best
    apply(best)
    return {"best": dict(best, ms_per_frame=best_ms), "frames_per_setting": n_frames, "candidates": results}


def tune_bvh(vis, camera, lighting, values=(0, 64), frames=2, verbose=False):
    """Scene-level knob: commit `vis` once per BVH binary-tree builder
    (GXY_TUNE_BVH_SAH: 0 radix tree, C > 1 binned-SAH top over clusters of C
    primitives), time a few frames of each and keep the faster scene.
    Returns (scene, value, [(value, ms), ...])."""
    import torch
    stream = torch.cuda.current_stream()
    cam = camera.c() if hasattr(camera, "c") else camera
    fb = torch.zeros((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
    best, best_ms, out = None, float("inf"), []
    for v in values:
        gpu.set_tuning(gpu.TUNE_BVH_SAH, v)
        sc = gpu.Scene(vis)
        sc.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(frames):
            fb.zero_()
            sc.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / frames
        out.append((v, ms))
        if verbose:
            print("autotune bvh", v, ms, flush=True)
        if ms < best_ms:
            if best is not None:
                best[0].release()
            best, best_ms = (sc, v), ms
        else:
            sc.release()
    gpu.set_tuning(gpu.TUNE_BVH_SAH, best[1])
    return best[0], best[1], out


def cache_key(workload):
    import torch
    return "%s|%s" % (torch.cuda.get_device_name(0), workload)


def load(path, workload):
    if not os.path.exists(path):
        return None
    d = json.load(open(path)).get(cache_key(workload))
    if d:
        apply(d)
    return d


def save(path, workload, best):
    d = json.load(open(path)) if os.path.exists(path) else {}
    d[cache_key(workload)] = best
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    json.dump(d, open(path, "w"), indent=1)
