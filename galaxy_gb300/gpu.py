"""ctypes binding of libgxy_gpu.so (include/gxy_gpu.h).

The GPU library is the only implementation of the ray path in this package:
if it is missing or fails to load, every call raises -- there is no CPU
fallback.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgxy_gpu.so")
_lib = None
_initialised = False


class GxyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gxy error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libgxy_gpu.so (built by galaxy_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgxy_gpu.so is not built (%s); run galaxy_gb300.build.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    sig = {
        "gxy_gpu_init": [C.c_int, C.c_size_t],
        "gxy_gpu_shutdown": [],
        "gxy_gpu_last_error": [C.c_char_p, C.c_int],
        "gxy_gpu_hbm_in_use": [C.POINTER(C.c_size_t)],
        "gxy_gpu_scene_commit": [C.POINTER(A.gxy_scene_desc), C.POINTER(vp)],
        "gxy_gpu_scene_release": [vp],
        "gxy_gpu_scene_set_tf": [vp, C.c_int, C.c_int, C.POINTER(A.gxy_tf), vp],
        "gxy_gpu_scene_view": [vp, C.POINTER(vp)],
        "gxy_gpu_scene_partition_info": [vp, C.c_int, C.POINTER(A.gxy_partition_info)],
        "gxy_gpu_scene_bvh_info": [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(C.c_double)],
        "gxy_scene_partition_layout": [C.POINTER(A.gxy_scene_desc), C.c_int, C.POINTER(A.gxy_partition_info)],
        "gxy_resolve_lights": [C.POINTER(A.gxy_lighting), C.POINTER(A.gxy_camera), C.POINTER(A.gxy_lighting)],
        "gxy_gpu_render": [vp, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_lighting), vp, vp],
        "gxy_gpu_render_host": [vp, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_lighting), A.f32p, vp],
        "gxy_gpu_query_counters": [vp, C.POINTER(A.gxy_counters)],
        "gxy_gpu_query_counters_ex": [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)],
        "gxy_gpu_generate_initial_rays": [vp, C.c_int, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_raylist),
                                          C.POINTER(i32)],
        "gxy_gpu_trace_raylist": [vp, C.c_int, C.POINTER(A.gxy_lighting), C.POINTER(A.gxy_raylist),
                                  C.POINTER(A.gxy_raylist), C.POINTER(i32)],
        "gxy_gpu_set_profiling": [vp, C.c_int],
        "gxy_gpu_query_generations": [vp, C.POINTER(A.gxy_generation_stats), C.c_int, C.POINTER(i32)],
        "gxy_gpu_batch_create": [C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(vp)],
        "gxy_gpu_batch_release": [vp],
        "gxy_gpu_batch_submit": [vp, C.POINTER(A.gxy_job), C.c_int, C.c_int],
        "gxy_gpu_batch_poll": [vp, C.POINTER(C.c_int)],
        "gxy_gpu_batch_wait": [vp, C.c_int],
        "gxy_gpu_batch_counters": [vp, C.POINTER(A.gxy_counters)],
        "gxy_gpu_batch_stream": [vp, C.POINTER(vp)],
        "gxy_gpu_set_tuning": [C.c_int, C.c_int],
        "gxy_tf_clear_below": [C.POINTER(A.gxy_tf), C.POINTER(C.c_float)],
        "gxy_gpu_get_tuning": [C.c_int, C.POINTER(C.c_int)],
        "gxy_gpu_classify": [C.POINTER(A.gxy_raylist)],
        "gxy_gpu_assign_destinations": [vp, C.c_int, C.POINTER(A.gxy_raylist)],
        "gxy_gpu_accumulate_terminated": [C.POINTER(A.gxy_raylist), A.f32p, C.c_int, C.c_int],
        "gxy_server_create": [C.POINTER(A.gxy_server_config), C.POINTER(vp)],
        "gxy_server_release": [vp],
        "gxy_server_submit": [vp, vp, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_lighting), C.POINTER(i64)],
        "gxy_server_poll": [vp, i64, C.POINTER(C.c_int)],
        "gxy_server_drain": [vp, C.c_int],
        "gxy_server_cancel": [vp, i64, C.POINTER(C.c_int)],
        "gxy_server_take": [vp, i64, A.f32p, C.POINTER(C.c_double), C.POINTER(i64)],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = L
    return L


def check(rc):
    if rc != A.GXY_OK:
        buf = C.create_string_buffer(1024)
        lib().gxy_gpu_last_error(buf, 1024)
        raise GxyError(rc, buf.value.decode(errors="replace"))
    return rc


def init(device=0, hbm_budget=0):
    global _initialised
    check(lib().gxy_gpu_init(device, hbm_budget))
    _initialised = True


def ensure_init():
    if not _initialised:
        init()


def hbm_in_use():
    v = C.c_size_t(0)
    check(lib().gxy_gpu_hbm_in_use(C.byref(v)))
    return v.value


TUNE_BLOCKS_PER_SM = 1
TUNE_GRID_PER_SM = 2
TUNE_SPLIT_SECONDARY = 3
TUNE_SPLIT_PRIMARY = 4
TUNE_BVH_SAH = 5
TUNE_LEAF_MAX = 6
TUNE_TRAV_STEPS = 7
TUNE_MARCH_STEPS = 8
TUNE_CAMERA_PACKET = 9
TUNE_SKIP_CLEAR = 10
TUNE_SKIP_MODE = 11
TUNE_CARRY_HITS = 13
TUNE_QUEUE_LIMIT = 14
TUNE_QUEUE_CHUNK = 15
TUNE_SPLIT_HANDOFF = 16
TUNE_SEC_PACKET = 17
TUNE_BVH_COLLAPSE = 18
TUNE_RUNAHEAD = 19
TUNE_QUERY_BLOCKS = 20
TUNE_PMARCH_BLOCKS = 21
TUNE_PQUERY_BLOCKS = 22
TUNE_CONTINUE = 23


def set_tuning(knob, value):
    check(lib().gxy_gpu_set_tuning(int(knob), int(value)))


def tf_clear_below(tf):
    """Zero-opacity threshold of a gxy_tf (host only; see gxy_gpu.h)."""
    t = C.c_float()
    check(lib().gxy_tf_clear_below(C.byref(tf), C.byref(t)))
    return t.value


def get_tuning(knob):
    v = C.c_int(0)
    check(lib().gxy_gpu_get_tuning(int(knob), C.byref(v)))
    return v.value


def partition_layout(vis, p):
    """Brick p's boxes and neighbours for a Visualization (host only)."""
    d = vis.desc()
    pi = A.gxy_partition_info()
    check(lib().gxy_scene_partition_layout(C.byref(d), p, C.byref(pi)))
    return pi


def resolve_lights(lighting, camera):
    """Rendering::resolve_lights through the C ABI; returns a gxy_lighting."""
    out = A.gxy_lighting()
    L = lighting.c() if hasattr(lighting, "c") else lighting
    cam = camera.c() if hasattr(camera, "c") else camera
    check(lib().gxy_resolve_lights(C.byref(L), C.byref(cam), C.byref(out)))
    return out


VIS_VOLUME, VIS_TRIANGLES, VIS_PARTICLES, VIS_PATHLINES = 0, 1, 2, 3


class Scene:
    """A committed Visualization on the device (gxy_gpu_scene_commit), or a
    view of one (Scene.view())."""

    def __init__(self, vis=None, _handle=None, _base=None):
        ensure_init()
        if _handle is not None:
            self.desc = _base.desc
            self.h = _handle
            return
        self.desc = vis.desc()
        h = C.c_void_p()
        check(lib().gxy_gpu_scene_commit(C.byref(self.desc), C.byref(h)))
        self.h = h

    def view(self):
        """A second handle sharing this scene's datasets and BVH, with its own
        transfer functions (gxy_gpu_scene_view)."""
        h = C.c_void_p()
        check(lib().gxy_gpu_scene_view(self.h, C.byref(h)))
        return Scene(_handle=h, _base=self)

    def set_tf(self, kind, index, tf, stream=None):
        """Replace the transfer function (a gxy_tf, or a MappedVis whose tf()
        gives one) of operator `index` of `kind` (VIS_VOLUME ...)."""
        t = tf.tf() if hasattr(tf, "tf") else tf
        check(lib().gxy_gpu_scene_set_tf(self.h, int(kind), int(index), C.byref(t), C.c_void_p(stream or 0)))

    def release(self):
        if getattr(self, "h", None) and self.h.value:
            lib().gxy_gpu_scene_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def partition_info(self, p):
        pi = A.gxy_partition_info()
        check(lib().gxy_gpu_scene_partition_info(self.h, p, C.byref(pi)))
        return pi

    def bvh_info(self):
        n, s, ms = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().gxy_gpu_scene_bvh_info(self.h, C.byref(n), C.byref(s), C.byref(ms)))
        return {"nodes": n.value, "prim_refs": s.value, "build_ms": ms.value}

    def render(self, camera, lighting, fb_ptr, stream=None):
        """Device framebuffer (pointer) path; contributions are added."""
        cam = camera.c() if hasattr(camera, "c") else camera
        L = lighting if isinstance(lighting, A.gxy_lighting) else lighting.c()
        check(lib().gxy_gpu_render(self.h, C.byref(cam), C.byref(L), C.c_void_p(fb_ptr),
                                   C.c_void_p(stream or 0)))

    def render_host(self, camera, lighting, out=None, stream=None):
        """Host framebuffer path: returns (height, width, 4) float32."""
        cam = camera.c() if hasattr(camera, "c") else camera
        L = lighting if isinstance(lighting, A.gxy_lighting) else lighting.c()
        if out is None:
            out = np.zeros((cam.height, cam.width, 4), np.float32)
        check(lib().gxy_gpu_render_host(self.h, C.byref(cam), C.byref(L), A.fptr(out), C.c_void_p(stream or 0)))
        return out

    def counters(self):
        c = A.gxy_counters()
        check(lib().gxy_gpu_query_counters(self.h, C.byref(c)))
        d = {f: getattr(c, f) for f, _ in A.gxy_counters._fields_}
        t, s, e = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().gxy_gpu_query_counters_ex(self.h, C.byref(t), C.byref(s), C.byref(e)))
        d.update(tri_tests=t.value, sph_tests=s.value, enqueued=e.value)
        return d

    def set_profiling(self, on=True):
        check(lib().gxy_gpu_set_profiling(self.h, 1 if on else 0))

    def generations(self):
        """Per-generation kernel time and counters of the last render
        (recorded while profiling is on)."""
        buf = (A.gxy_generation_stats * 256)()
        n = C.c_int32(0)
        check(lib().gxy_gpu_query_generations(self.h, buf, 256, C.byref(n)))
        return [{f: getattr(buf[i], f) for f, _ in A.gxy_generation_stats._fields_} for i in range(min(n.value, 256))]

    # ---- RayList drop-in
    def generate_initial_rays(self, p, camera, capacity=None):
        cam = camera.c() if hasattr(camera, "c") else camera
        out = A.RayListArrays(capacity or cam.width * cam.height)
        n = C.c_int32(0)
        rl = out.c()
        check(lib().gxy_gpu_generate_initial_rays(self.h, p, C.byref(cam), C.byref(rl), C.byref(n)))
        return out.truncate(n.value)

    def trace(self, p, lighting, rays, capacity=None):
        """TraceRays::Trace on a copy of `rays`: returns (traced, secondary)."""
        rin = rays.copy()
        L = lighting if isinstance(lighting, A.gxy_lighting) else lighting.c()
        cap = capacity if capacity is not None else max(1, rays.n * 40)
        out = A.RayListArrays(cap)
        n = C.c_int32(0)
        ci, co = rin.c(), out.c()
        check(lib().gxy_gpu_trace_raylist(self.h, p, C.byref(L), C.byref(ci), C.byref(co), C.byref(n)))
        return rin, out.truncate(n.value)

    def assign_destinations(self, p, rays):
        r = rays.copy()
        c = r.c()
        check(lib().gxy_gpu_assign_destinations(self.h, p, C.byref(c)))
        return r


def classify(rays):
    r = rays.copy()
    c = r.c()
    check(lib().gxy_gpu_classify(C.byref(c)))
    return r


def accumulate_terminated(rays, fb):
    c = rays.c()
    h, w, _ = fb.shape
    check(lib().gxy_gpu_accumulate_terminated(C.byref(c), A.fptr(fb), w, h))
    return fb


class Batch:
    """A batch slot (gxy_gpu_batch_create): device queues for up to
    max_pixels camera rays, a job table and its own CUDA stream.  submit()
    renders many jobs -- (scene, camera, lighting, device framebuffer) -- in
    one persistent wavefront launch; poll()/wait() report completion."""

    def __init__(self, max_pixels, max_jobs=64, max_shadow=1, max_ao=4):
        ensure_init()
        h = C.c_void_p()
        check(lib().gxy_gpu_batch_create(int(max_pixels), int(max_jobs), int(max_shadow), int(max_ao), C.byref(h)))
        self.h = h
        self.max_pixels, self.max_jobs, self.max_shadow, self.max_ao = max_pixels, max_jobs, max_shadow, max_ao
        self._keep = None

    def release(self):
        if getattr(self, "h", None) and self.h.value:
            lib().gxy_gpu_batch_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @property
    def stream(self):
        s = C.c_void_p()
        check(lib().gxy_gpu_batch_stream(self.h, C.byref(s)))
        return s.value

    def submit(self, jobs, use_graph=False, cooperative=False):
        """jobs: list of (Scene, camera, gxy_lighting, device fb pointer).
        use_graph: replay the submission as a CUDA graph; cooperative: run
        every generation in one cooperative launch (else one launch per
        generation, so slots on different streams overlap)."""
        arr = (A.gxy_job * len(jobs))()
        for i, (sc, cam, L, fb) in enumerate(jobs):
            arr[i].scene = sc.h.value
            arr[i].camera = cam.c() if hasattr(cam, "c") else cam
            arr[i].lighting = L if isinstance(L, A.gxy_lighting) else L.c()
            arr[i].fb_rgba = fb
        self._keep = (arr, jobs)
        flags = (1 if use_graph else 0) | (2 if cooperative else 0)
        check(lib().gxy_gpu_batch_submit(self.h, arr, len(jobs), flags))

    def poll(self):
        d = C.c_int(0)
        check(lib().gxy_gpu_batch_poll(self.h, C.byref(d)))
        return bool(d.value)

    def wait(self, timeout_ms=60000):
        check(lib().gxy_gpu_batch_wait(self.h, int(timeout_ms)))

    def counters(self):
        c = A.gxy_counters()
        check(lib().gxy_gpu_batch_counters(self.h, C.byref(c)))
        return {f: getattr(c, f) for f, _ in A.gxy_counters._fields_}


class NativeServer:
    """The library's continuous-batching request loop (gxy_server_*): a C++
    worker thread admits submitted requests into batch slots under a
    framebuffer budget and completes them by polling."""

    def __init__(self, n_slots=4, slot_pixels=8 << 20, max_jobs=64, max_shadow=1, max_ao=4, fb_budget=8 << 30,
                 small_pixels=1 << 20, small_batch_pixels=4 << 20, big_wait_s=0.05, use_graph=True,
                 cooperative=False):
        ensure_init()
        cfg = A.gxy_server_config(n_slots=n_slots, slot_pixels=int(slot_pixels), max_jobs=max_jobs,
                                  max_shadow=max_shadow, max_ao=max_ao, fb_budget_bytes=int(fb_budget),
                                  small_pixels=int(small_pixels), small_batch_pixels=int(small_batch_pixels),
                                  big_wait_s=float(big_wait_s), use_graph=1 if use_graph else 0,
                                  cooperative=1 if cooperative else 0)
        h = C.c_void_p()
        check(lib().gxy_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._sizes = {}

    def release(self):
        if getattr(self, "h", None) and self.h.value:
            lib().gxy_server_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def submit(self, scene, camera, lighting):
        cam = camera.c() if hasattr(camera, "c") else camera
        L = lighting if isinstance(lighting, A.gxy_lighting) else lighting.c()
        rid = C.c_int64(0)
        check(lib().gxy_server_submit(self.h, scene.h, C.byref(cam), C.byref(L), C.byref(rid)))
        self._sizes[rid.value] = (cam.height, cam.width)
        return rid.value

    def poll(self, rid):
        d = C.c_int(0)
        check(lib().gxy_server_poll(self.h, int(rid), C.byref(d)))
        return bool(d.value)

    def cancel(self, rid):
        """Cancel a request; returns True if it was already running."""
        w = C.c_int(0)
        check(lib().gxy_server_cancel(self.h, int(rid), C.byref(w)))
        return bool(w.value)

    def drain(self, timeout_ms=600000):
        check(lib().gxy_server_drain(self.h, int(timeout_ms)))

    def take(self, rid, image=True):
        """(rgba or None, latency seconds, rays) of a finished request."""
        h, w = self._sizes.pop(rid)
        out = np.zeros((h, w, 4), np.float32) if image else None
        lat, rays = C.c_double(0), C.c_int64(0)
        check(lib().gxy_server_take(self.h, int(rid), A.fptr(out) if image else None, C.byref(lat), C.byref(rays)))
        return out, lat.value, rays.value
