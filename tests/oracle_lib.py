"""ctypes loader for the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: the oracle is the parity checker, never the product.
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from galaxy_gb300 import _abi as A  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as ob  # oracle/build.py
        path = ob.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.oracle_scene_create.restype = vp
        L.oracle_scene_create.argtypes = [C.POINTER(A.gxy_scene_desc)]
        L.oracle_scene_destroy.argtypes = [vp]
        L.oracle_partition_info.argtypes = [vp, C.c_int, C.POINTER(A.gxy_partition_info)]
        L.oracle_generate_initial_rays.argtypes = [vp, C.c_int, C.POINTER(A.gxy_camera),
                                                   C.POINTER(A.gxy_raylist), C.POINTER(C.c_int32)]
        L.oracle_trace_raylist.argtypes = [vp, C.c_int, C.POINTER(A.gxy_lighting), C.POINTER(A.gxy_raylist),
                                           C.POINTER(A.gxy_raylist), C.POINTER(C.c_int32)]
        L.oracle_trace_f64.argtypes = [vp, C.c_int, C.POINTER(A.gxy_raylist), C.POINTER(C.c_double)]
        L.oracle_classify.argtypes = [C.POINTER(A.gxy_raylist)]
        L.oracle_assign_destinations.argtypes = [vp, C.c_int, C.POINTER(A.gxy_raylist)]
        L.oracle_accumulate.argtypes = [C.POINTER(A.gxy_raylist), A.f32p, C.c_int, C.c_int]
        L.oracle_render.argtypes = [vp, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_lighting), A.f32p,
                                    C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64)]
        L.oracle_tf_resample.argtypes = [A.f32p, C.c_int, A.f32p, C.c_int, C.c_int, C.c_float, C.c_float,
                                         C.POINTER(A.gxy_tf)]
        L.oracle_ao_tables.argtypes = [A.f32p, A.f32p]
        L.oracle_tf_opacity.restype = C.c_float
        L.oracle_tf_opacity.argtypes = [C.POINTER(A.gxy_tf), C.c_float]
        L.oracle_quantize.argtypes = [A.f32p, C.c_int, C.c_int, C.POINTER(C.c_uint8)]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_set_threads(os.cpu_count() or 1)
        _lib = L
    return _lib


class OracleScene:
    def __init__(self, vis):
        self.desc = vis.desc()
        self.h = lib().oracle_scene_create(C.byref(self.desc))

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_scene_destroy(self.h)
            self.h = None

    def partition_info(self, p):
        pi = A.gxy_partition_info()
        assert lib().oracle_partition_info(self.h, p, C.byref(pi)) == 0
        return pi

    def render(self, cam, lighting, nthreads=8, rows=None):
        c = cam.c()
        L = lighting.c()
        fb = np.zeros((cam.height, cam.width, 4), np.float32)
        cnt = (C.c_int64 * 6)()
        r0, r1 = rows if rows is not None else (0, 0)
        lib().oracle_render(self.h, C.byref(c), C.byref(L), fb.ctypes.data_as(A.f32p), nthreads, r0, r1, cnt)
        return fb, dict(zip(("primary", "shadow", "ao", "segments", "samples", "terminated"), list(cnt)))

    def generate_initial_rays(self, p, cam, capacity=None):
        c = cam.c()
        cap = capacity or cam.width * cam.height
        out = A.RayListArrays(cap)
        n = C.c_int32(0)
        rl = out.c()
        assert lib().oracle_generate_initial_rays(self.h, p, C.byref(c), C.byref(rl), C.byref(n)) == 0
        return out.truncate(n.value)

    def trace(self, p, lighting, rays, capacity=None):
        """TraceRays::Trace on a copy of `rays`: returns (traced, secondary)."""
        rin = rays.copy()
        cap = capacity if capacity is not None else max(1, rays.n * 40)
        out = A.RayListArrays(cap)
        L = lighting.c()
        n = C.c_int32(0)
        ci, co = rin.c(), out.c()
        rc = lib().oracle_trace_raylist(self.h, p, C.byref(L), C.byref(ci), C.byref(co), C.byref(n))
        assert rc == 0, rc
        return rin, out.truncate(n.value)

    def trace_f64(self, p, rays):
        rin = rays.copy()
        res = np.zeros((rays.n, 4), np.float64)
        ci = rin.c()
        lib().oracle_trace_f64(self.h, p, C.byref(ci), res.ctypes.data_as(C.POINTER(C.c_double)))
        return res

    def classify(self, rays):
        r = rays.copy()
        c = r.c()
        lib().oracle_classify(C.byref(c))
        return r

    def assign_destinations(self, p, rays):
        r = rays.copy()
        c = r.c()
        lib().oracle_assign_destinations(self.h, p, C.byref(c))
        return r


def quantize(fb):
    h, w, _ = fb.shape
    out = np.zeros((h, w, 4), np.uint8)
    f = np.ascontiguousarray(fb, np.float32)
    lib().oracle_quantize(f.ctypes.data_as(A.f32p), w, h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def ao_tables():
    u = np.zeros(256, np.float32)
    v = np.zeros(256, np.float32)
    lib().oracle_ao_tables(u.ctypes.data_as(A.f32p), v.ctypes.data_as(A.f32p))
    return u, v
