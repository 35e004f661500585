"""Continuous-batching request loop over device-resident scenes.

This plays the role of Galaxy's serving front ends -- ViewerClientServer's
`render` command (src/multiserver/ViewerClientServer.cpp:62-253, pixels
returned per ServerRendering::AddLocalPixels, ServerRendering.cpp:45-66) and
GuiClientServer's `gui::render` (src/guiserver/GuiClientServer.cpp:375-407)
-- without their socket transport: a request names a resident scene and
carries a camera, a light change or a transfer-function change, and an
image size.  The loop itself is the library's C++ worker (gxy_server_*,
csrc/server.cu); it

  * admits waiting requests whenever a batch slot is free and the
    framebuffers fit the HBM budget (admission control; a request too large
    for any slot is refused),
  * packs the admitted requests of one scene into one persistent wavefront
    launch on that slot's stream, so several batches -- requests that
    arrived while others were already on the GPU -- overlap on the device,
  * polls the slots and records each request's latency (arrival ->
    framebuffer complete on the device); the client takes the image.

A request that changes a transfer function renders through a view of its
scene (gxy_gpu_scene_view: the datasets and BVH shared, the transfer
functions its own) taken from a small pool per scene, so requests with
different transfer functions are on the GPU at once while the resident
scene keeps its own.

serve_plain() serves the same requests one at a time through the plain
single-frame path (gxy_gpu_render) for comparison, changing the resident
scene's transfer functions in place (gxy_gpu_scene_set_tf) as a viewer's
json command does.  CommandSession reads a
viewer client's command lines (json / window / render / renderMany ...) and
streams each frame's pixels back as AddLocalPixels messages.
"""
import math
import time

import numpy as np

from . import _abi as A
from . import gpu
from . import scene as S


class Request:
    __slots__ = ("id", "arrival", "scene", "camera", "lighting", "pixels", "fb", "t_submit", "t_done", "rays",
                 "refused", "tf")

    def __init__(self, rid, arrival, scene, camera, lighting, tf=None):
        self.id = rid
        self.arrival = arrival
        self.scene = scene          # key into the scene table
        self.camera = camera        # scene.Camera
        self.lighting = lighting    # gxy_lighting (resolved)
        self.tf = tf                # None, or [(vis kind, operator index, gxy_tf), ...]
        self.pixels = camera.width * camera.height
        self.fb = None
        self.t_submit = None
        self.t_done = None
        self.rays = 0
        self.refused = False


class Server:
    """Continuous batching over resident scenes: the library's C++ request
    loop (gxy_server_*, gpu.NativeServer) does the admission, packing and
    completion; run() replays requests at their arrival times and collects
    latency and rays.  Admission policy: requests up to `small_pixels` are
    "small" and are packed together (same scene, FIFO) up to
    `small_batch_pixels` per launch; a larger request runs in a slot of its
    own.  The oldest waiting request goes first, except that small requests
    may pass a large one that has waited less than `big_wait_s`; requests
    are admitted while their framebuffers fit `fb_budget` bytes."""

    def __init__(self, scenes, n_slots=4, slot_pixels=8 << 20, max_jobs=64, max_shadow=1, max_ao=4,
                 fb_budget=8 << 30, use_graph=True, keep_results=False, cooperative=False,
                 small_pixels=1 << 20, small_batch_pixels=4 << 20, big_wait_s=0.05, max_views=16):
        self.scenes = scenes
        self.keep_results = keep_results
        self.slot_pixels = slot_pixels
        self.max_views = max_views
        self.views = {}             # scene key -> [[view, id of its last request], ...]
        self.native = gpu.NativeServer(n_slots, slot_pixels, max_jobs, max_shadow, max_ao, fb_budget,
                                       small_pixels, small_batch_pixels, big_wait_s, use_graph, cooperative)

    def release(self):
        self.native.release()
        for pool in self.views.values():
            for v in pool:
                v[0].release()
        self.views = {}

    def _view(self, key):
        """A view of scene `key` whose last request has finished (a new one
        while the pool is below max_views)."""
        pool = self.views.setdefault(key, [])
        while True:
            for v in pool:
                if v[1] is None or self.native.poll(v[1]):
                    return v
            if len(pool) < self.max_views:
                pool.append([self.scenes[key].view(), None])
                return pool[-1]
            time.sleep(50e-6)

    def run(self, requests, time_limit=120.0, keep=None):
        """Submit `requests` (sorted by arrival, seconds from start) in real
        time, wait for all, and return the statistics dict; with
        keep_results (or r.id in `keep`) each request's image is left in
        r.fb (host array)."""
        t0 = time.perf_counter()
        submitted = []
        for r in requests:
            now = time.perf_counter() - t0
            if now > time_limit:
                break
            if r.arrival > now:
                time.sleep(r.arrival - now)
            sc, view = self.scenes[r.scene], None
            if r.tf:
                view = self._view(r.scene)
                for kind, index, tf in r.tf:
                    view[0].set_tf(kind, index, tf)
                sc = view[0]
            try:
                rid = self.native.submit(sc, r.camera, r.lighting)
            except gpu.GxyError as e:
                if e.code != A.GXY_ERR_ADMISSION:
                    raise
                r.refused = True
                continue
            if view is not None:
                view[1] = rid
            r.t_submit = time.perf_counter() - t0
            submitted.append((r, rid))
        left = max(1.0, time_limit - (time.perf_counter() - t0))
        self.native.drain(int(left * 1000))
        makespan = time.perf_counter() - t0
        for r, rid in submitted:
            img, lat, rays = self.native.take(rid, image=self.keep_results or (keep is not None and r.id in keep))
            r.t_done = r.t_submit + lat
            r.rays = rays
            r.fb = img
        for pool in self.views.values():
            for v in pool:
                v[1] = None
        return summarize(requests, makespan)


def summarize(requests, makespan, busy_s=None):
    lat = np.array([r.t_done - r.arrival for r in requests if r.t_done is not None])
    rays = sum(r.rays for r in requests if r.t_done is not None)
    out = {"requests": len(requests), "completed": int(len(lat)),
           "refused": int(sum(1 for r in requests if r.refused)), "makespan_s": makespan,
           "rays": float(rays), "rays_per_s": float(rays / makespan) if makespan > 0 else 0.0}
    if busy_s is not None and makespan > 0:
        out["gpu_busy_frac"] = float(busy_s / makespan)   # time with a request on the GPU
    if len(lat):
        out.update(p50_ms=float(np.percentile(lat, 50) * 1e3), p95_ms=float(np.percentile(lat, 95) * 1e3),
                   p99_ms=float(np.percentile(lat, 99) * 1e3), mean_ms=float(lat.mean() * 1e3))
    return out


def serve_plain(scenes, requests, time_limit=120.0, keep=None, default_tfs=None):
    """The same requests, one at a time through the plain single-frame path
    (gxy_gpu_render on torch's current stream), in arrival order.  A request
    with transfer functions sets them on the resident scene first
    (gxy_gpu_scene_set_tf); the next request without any restores
    default_tfs[key] (the committed ones).  Images of requests whose id is in
    `keep` are left in r.fb (host array)."""
    import torch
    t0 = time.perf_counter()
    stream = torch.cuda.current_stream()
    changed = {}
    for r in requests:
        now = time.perf_counter() - t0
        if now > time_limit:
            break
        if r.arrival > now:
            time.sleep(r.arrival - now)
        sc = scenes[r.scene]
        r.t_submit = time.perf_counter() - t0
        if r.tf:
            for kind, index, tf in r.tf:
                sc.set_tf(kind, index, tf, stream.cuda_stream)
            changed[r.scene] = True
        elif changed.get(r.scene):
            for kind, index, tf in (default_tfs or {}).get(r.scene, []):
                sc.set_tf(kind, index, tf, stream.cuda_stream)
            changed[r.scene] = False
        fb = torch.zeros((r.camera.height, r.camera.width, 4), dtype=torch.float32, device="cuda")
        sc.render(r.camera, r.lighting, fb.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        r.t_done = time.perf_counter() - t0
        c = sc.counters()
        r.rays = c["primary_rays"] + c["shadow_rays"] + c["ao_rays"]
        if keep is not None and r.id in keep:
            r.fb = fb.cpu().numpy()
        del fb
    for key, ch in changed.items():
        if ch:
            for kind, index, tf in (default_tfs or {}).get(key, []):
                scenes[key].set_tf(kind, index, tf, stream.cuda_stream)
    busy = sum(r.t_done - r.t_submit for r in requests if r.t_done is not None)
    return summarize(requests, time.perf_counter() - t0, busy)


def poisson_requests(rate, count, scene_keys, make_request, seed=7, side_range=(256, 4096)):
    """Poisson arrivals at `rate` per second; image side log-uniform in
    side_range; make_request(rng, rid, arrival, scene_key, side) builds one
    request (random camera, light or transfer-function change)."""
    rng = np.random.Generator(np.random.Philox(seed))
    t = 0.0
    out = []
    lo, hi = math.log(side_range[0]), math.log(side_range[1])
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        side = int(round(math.exp(rng.uniform(lo, hi))))
        key = scene_keys[int(rng.integers(0, len(scene_keys)))]
        out.append(make_request(rng, rid, t, key, side))
    return out


# ------------------------------------------------------- command protocol
PIXEL_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("r", "<f4"), ("g", "<f4"), ("b", "<f4"), ("o", "<f4")])


class CommandSession:
    """One viewer client's command stream, as ViewerClientServer::handle
    (multiserver/ViewerClientServer.cpp:62-253) reads it, over the resident
    device path (no sockets here: a front end passes each received line to
    handle() and sends back the reply and the pixel messages).

    Commands: "json <document>" with any of Datasets, Visualization, Camera,
    Renderer (loaded and committed in that order; error replies as Galaxy
    words them), "window <w> <h>", "commit", "render", "renderMany <n>",
    "permute_pixels on|off" and "max_rays_per_packet <n>" (accepted; the
    device path renders whole frames, so they change nothing).  handle()
    returns (handled, reply); an unknown command is (False, None).

    Each rendered frame is sent as ServerRendering::AddLocalPixels messages
    (ServerRendering.cpp:45-66): on_pixels(n, frame, sender, pixels), pixels
    a PIXEL_DTYPE array (x, y, r, g, b, o) of the frame's non-zero pixels,
    in chunks of `chunk`."""

    def __init__(self, base_dir=".", on_pixels=None, chunk=1 << 16, partitions=(1, 1, 1), render_fn=None):
        self.base_dir = base_dir
        self.on_pixels = on_pixels
        self.chunk = int(chunk)
        self.partitions = partitions
        self.render_fn = render_fn
        self.datasets = {}
        self.visualization = None
        self.camera = None
        self.epsilon = 0.001
        self.scene = None
        self.frame = 0
        self.permute = True
        self.max_rays_per_packet = 0

    def _commit(self):
        self.scene = None
        if self.visualization is not None:
            self.scene = gpu.Scene(self.visualization)

    def handle(self, line):
        import json
        parts = line.strip().split(None, 1)
        if not parts:
            return False, None
        cmd, rest = parts[0], (parts[1] if len(parts) > 1 else "")
        if cmd == "permute_pixels":
            if rest.strip() in ("", "on"):
                self.permute = True
            elif rest.strip() == "off":
                self.permute = False
            else:
                return True, "error permute_pixels needs on or off"
            return True, "ok"
        if cmd == "max_rays_per_packet":
            try:
                self.max_rays_per_packet = int(rest.split()[0])
            except (ValueError, IndexError):
                return True, "error max_rays_per_packet needs an integer"
            return True, "ok"
        if cmd == "commit":
            self._commit()
            return True, "ok"
        if cmd == "json":
            try:
                doc = json.loads(rest)
            except ValueError:
                return True, "error parsing json command"
            if "Datasets" in doc:
                try:
                    self.datasets.update(S.datasets_from_json(doc, self.base_dir))
                except (ValueError, OSError, KeyError):
                    return True, "error loading datasets from json command"
            if "Renderer" in doc:
                self.epsilon = S.renderer_epsilon(doc, self.epsilon)
            if "Visualization" in doc:
                try:
                    self.visualization = S.visualization_from_json(doc["Visualization"], self.datasets,
                                                                   self.partitions, self.epsilon)
                except (ValueError, KeyError):
                    return True, "error loading visualization from json command"
                try:
                    self._commit()
                except gpu.GxyError:
                    return True, "error committing visualization from json command"
            if "Camera" in doc:
                try:
                    cam = S.Camera.from_json(doc["Camera"])
                except (ValueError, KeyError):
                    return True, "error loading camera from json command"
                if self.camera is not None and "dimensions" not in doc["Camera"]:
                    cam.width, cam.height = self.camera.width, self.camera.height
                self.camera = cam
            return True, "ok"
        if cmd == "window":
            try:
                w, h = (int(x) for x in rest.split()[:2])
            except ValueError:
                return True, "error window command needs width and height as integers"
            if self.camera is None:
                self.camera = S.Camera((0, 0, 5), (0, 0, -1), (0, 1, 0), 45.0, w, h)
            self.camera.width, self.camera.height = w, h
            return True, "ok"
        if cmd == "render":
            self.render()
            return True, "ok"
        if cmd == "renderMany":
            try:
                n = int(rest.split()[0])
            except (ValueError, IndexError):
                return True, "error renderMany needs a count"
            for _ in range(n):
                self.render()
            return True, "ok"
        return False, None

    def render(self):
        """Render the current camera x visualization and stream its pixels;
        returns the (h, w, 4) framebuffer."""
        if self.scene is None or self.camera is None:
            return None
        L = S.resolve_lights(self.visualization.lighting, self.camera)
        if self.render_fn is not None:
            fb = self.render_fn(self.scene, self.camera, L)
        else:
            fb = self.scene.render_host(self.camera, L)
        frame = self.frame
        self.frame += 1
        if self.on_pixels is not None:
            ys, xs = np.nonzero(np.any(fb != 0, axis=2))
            px = np.empty(len(xs), PIXEL_DTYPE)
            px["x"], px["y"] = xs, ys
            v = fb[ys, xs]
            px["r"], px["g"], px["b"], px["o"] = v[:, 0], v[:, 1], v[:, 2], v[:, 3]
            for k in range(0, len(px), self.chunk):
                part = px[k:k + self.chunk]
                self.on_pixels(len(part), frame, 0, part)
        return fb
