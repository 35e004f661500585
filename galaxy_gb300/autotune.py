"""Autotuner for the wavefront kernels.

Measures a short run of real frames of the caller's scene for each
candidate setting and keeps the fastest:

  * register budget / occupancy: the frame kernels compiled for 2 resident
    blocks per SM (128 registers, no spills) or 3 (80 registers, some
    spills to L1-resident local memory);
  * grid-stride grid size: 4, 8 or 16 blocks per SM (a smaller grid keeps
    rays of a block spatially closer; a larger one balances the tail);
  * split shadow/AO tracing: one combined kernel, or a query pass plus a
    march pass whose lanes refill from the march queue (volume scenes);
  * split camera-ray tracing, likewise.

Frames are timed with CUDA events on the render stream after one warm-up
frame per setting.  The result can be cached in a JSON file keyed by GPU
name and workload.
"""
import json
import os

from . import gpu


def tune(scene, camera, lighting, frames=3, blocks_per_sm=(2, 3), grid_per_sm=(8, 16, 32), split=(0, 1),
         split_primary=(0, 1), verbose=False):
    import torch
    stream = torch.cuda.current_stream()
    cam = camera.c() if hasattr(camera, "c") else camera
    fb = torch.zeros((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
    results = []
    combos = [(mb, gp, sp, pp) for mb in blocks_per_sm for gp in grid_per_sm for sp in split for pp in split_primary]
    for mb, gp, sp, pp in combos:
        if True:
            gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, mb)
            gpu.set_tuning(gpu.TUNE_GRID_PER_SM, gp)
            gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, sp)
            gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, pp)
            fb.zero_()
            scene.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(frames):
                fb.zero_()
                scene.render(cam, lighting, fb.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / frames
            results.append({"blocks_per_sm": mb, "grid_per_sm": gp, "split": sp, "split_primary": pp,
                            "ms_per_frame": ms})
            if verbose:
                print("autotune", results[-1], flush=True)
    best = min(results, key=lambda r: r["ms_per_frame"])
    gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, best["blocks_per_sm"])
    gpu.set_tuning(gpu.TUNE_GRID_PER_SM, best["grid_per_sm"])
    gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, best["split"])
    gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, best["split_primary"])
    return {"best": best, "candidates": results}


def cache_key(workload):
    import torch
    return "%s|%s" % (torch.cuda.get_device_name(0), workload)


def load(path, workload):
    if not os.path.exists(path):
        return None
    d = json.load(open(path)).get(cache_key(workload))
    if d:
        gpu.set_tuning(gpu.TUNE_BLOCKS_PER_SM, d["blocks_per_sm"])
        gpu.set_tuning(gpu.TUNE_GRID_PER_SM, d["grid_per_sm"])
        gpu.set_tuning(gpu.TUNE_SPLIT_SECONDARY, d.get("split", 1))
        gpu.set_tuning(gpu.TUNE_SPLIT_PRIMARY, d.get("split_primary", 1))
    return d


def save(path, workload, best):
    d = json.load(open(path)) if os.path.exists(path) else {}
    d[cache_key(workload)] = best
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    json.dump(d, open(path, "w"), indent=1)
