"""ctypes mirror of the C ABI structs declared in include/gxy_gpu.h.

Only data layout lives here: the scene, camera, lighting and RayList
descriptors Galaxy's ISPC boundary passes (Rays.ih:21-48, Lighting.ih:23-32,
Visualization.ih:30-47, VolumeVis.ih, MappedVis.ih).  Every field matches the
C header one to one; tests/test_abi.py checks the sizes against the compiled
library.
"""
import ctypes as C

import numpy as np

GXY_OK = 0
GXY_ERR_INVALID = -1
GXY_ERR_CUDA = -2
GXY_ERR_OOM = -3
GXY_ERR_OVERFLOW = -4
GXY_ERR_TIMEOUT = -5
GXY_ERR_ADMISSION = -6
GXY_ERR_NOT_INIT = -7
GXY_ERR_CANCELLED = -8

RAY_PRIMARY, RAY_SHADOW, RAY_AO, RAY_EMPTY = 0x1, 0x2, 0x4, 0x8
RAY_SURFACE, RAY_OPAQUE, RAY_BOUNDARY, RAY_TIMEOUT = 0x1, 0x2, 0x4, 0x8
TERMINATED, DROP_ON_FLOOR, KEEP_HERE, UNDETERMINED = -1, -2, -3, -4

TF_SIZE = 256
MAX_LIGHTS = 8
MAX_SLICES = 8
MAX_ISOVALUES = 8
MAX_VOLUMES = 4

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)


class gxy_tf(C.Structure):
    _fields_ = [("colors", C.c_float * (TF_SIZE * 3)),
                ("opacities", C.c_float * TF_SIZE),
                ("range", C.c_float * 2)]


class gxy_volume_vis(C.Structure):
    _fields_ = [("samples", f32p),
                ("counts", C.c_int32 * 3),
                ("origin", C.c_float * 3),
                ("deltas", C.c_float * 3),
                ("tf", gxy_tf),
                ("n_slices", C.c_int32),
                ("slices", (C.c_float * 4) * MAX_SLICES),
                ("n_isovalues", C.c_int32),
                ("isovalues", C.c_float * MAX_ISOVALUES),
                ("volume_render", C.c_int32)]


class gxy_triangles_vis(C.Structure):
    _fields_ = [("vertices", f32p), ("n_vertices", C.c_int64),
                ("indices", i32p), ("n_triangles", C.c_int64),
                ("normals", f32p), ("data", f32p), ("tf", gxy_tf)]


class gxy_particles_vis(C.Structure):
    _fields_ = [("centers", f32p), ("data", f32p), ("n", C.c_int64),
                ("radius0", C.c_float), ("radius1", C.c_float),
                ("value0", C.c_float), ("value1", C.c_float), ("tf", gxy_tf)]


class gxy_pathlines_vis(C.Structure):
    _fields_ = [("vertices", f32p), ("data", f32p), ("n_vertices", C.c_int64),
                ("indices", i32p), ("n_segments", C.c_int64),
                ("radius0", C.c_float), ("radius1", C.c_float),
                ("value0", C.c_float), ("value1", C.c_float), ("tf", gxy_tf)]


class gxy_lighting(C.Structure):
    _fields_ = [("n_lights", C.c_int32),
                ("lights", (C.c_float * 3) * MAX_LIGHTS),
                ("types", C.c_int32 * MAX_LIGHTS),
                ("Ka", C.c_float), ("Kd", C.c_float),
                ("n_ao", C.c_int32), ("ao_radius", C.c_float),
                ("shadows", C.c_int32)]


class gxy_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("dir", C.c_float * 3), ("up", C.c_float * 3),
                ("aov", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class gxy_scene_desc(C.Structure):
    _fields_ = [("n_volumes", C.c_int32), ("volumes", C.POINTER(gxy_volume_vis)),
                ("n_triangle_sets", C.c_int32), ("triangles", C.POINTER(gxy_triangles_vis)),
                ("n_particle_sets", C.c_int32), ("particles", C.POINTER(gxy_particles_vis)),
                ("partitions", C.c_int32 * 3),
                ("has_box", C.c_int32), ("box", C.c_float * 6),
                ("sampling_rate", C.c_float), ("opaque_alpha", C.c_float),
                ("epsilon", C.c_float),
                ("n_pathline_sets", C.c_int32), ("pathlines", C.POINTER(gxy_pathlines_vis)),
                ("n_partition_extents", C.c_int32), ("partition_extents", f32p)]


RAY_FLOAT_FIELDS = ("ox", "oy", "oz", "dx", "dy", "dz", "nx", "ny", "nz", "sample",
                    "r", "g", "b", "o", "sr", "sg", "sb", "so", "t", "tMax")
RAY_INT_FIELDS = ("x", "y", "type", "term", "classification")


class gxy_raylist(C.Structure):
    _fields_ = ([(f, f32p) for f in RAY_FLOAT_FIELDS] +
                [(f, i32p) for f in RAY_INT_FIELDS] + [("n", C.c_int32)])


class gxy_partition_info(C.Structure):
    _fields_ = [("global_box", C.c_float * 6), ("local_box", C.c_float * 6),
                ("neighbors", C.c_int32 * 6), ("n_partitions", C.c_int32)]


class gxy_counters(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "primary_rays", "secondary_rays", "shadow_rays", "ao_rays", "segments",
        "handoffs", "terminated", "dropped", "kept", "bounces", "samples", "nodes",
        "prim_tests")] + [("overflow", C.c_int32), ("bands", C.c_int32), ("samples_skipped", C.c_int64)]


def fptr(a):
    """float32 numpy array -> float* (None for None)."""
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(f32p)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(i32p)


class RayListArrays:
    """Host-side RayList: 20 float32 and 5 int32 numpy arrays of equal length
    (the field set of RayList, Rays.h:43-227), viewable as a gxy_raylist."""

    def __init__(self, n=0, **fields):
        self.n = int(n)
        for f in RAY_FLOAT_FIELDS:
            setattr(self, f, np.zeros(self.n, np.float32))
        for f in RAY_INT_FIELDS:
            setattr(self, f, np.zeros(self.n, np.int32))
        for k, v in fields.items():
            arr = np.ascontiguousarray(v, dtype=np.int32 if k in RAY_INT_FIELDS else np.float32)
            assert arr.shape == (self.n,), k
            setattr(self, k, arr)

    def c(self):
        rl = gxy_raylist()
        for f in RAY_FLOAT_FIELDS:
            setattr(rl, f, fptr(getattr(self, f)))
        for f in RAY_INT_FIELDS:
            setattr(rl, f, iptr(getattr(self, f)))
        rl.n = self.n
        return rl

    def copy(self):
        out = RayListArrays(self.n)
        for f in RAY_FLOAT_FIELDS + RAY_INT_FIELDS:
            setattr(out, f, getattr(self, f).copy())
        return out

    def truncate(self, n):
        out = RayListArrays(n)
        for f in RAY_FLOAT_FIELDS + RAY_INT_FIELDS:
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[:n]))
        return out

    def take(self, idx):
        out = RayListArrays(len(idx))
        for f in RAY_FLOAT_FIELDS + RAY_INT_FIELDS:
            setattr(out, f, np.ascontiguousarray(getattr(self, f)[idx]))
        return out


class gxy_generation_stats(C.Structure):
    _fields_ = [("ms", C.c_double), ("generation", C.c_int32), ("kind", C.c_int32)] + [(n, C.c_int64) for n in (
        "rays_in", "enqueued", "segments", "samples", "nodes", "tri_tests", "sph_tests", "terminated",
        "samples_skipped")] + [("start_ms", C.c_double)]


class gxy_job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", gxy_camera), ("lighting", gxy_lighting),
                ("fb_rgba", C.c_void_p)]


class gxy_server_config(C.Structure):
    _fields_ = [("n_slots", C.c_int32), ("slot_pixels", C.c_int64), ("max_jobs", C.c_int32),
                ("max_shadow", C.c_int32), ("max_ao", C.c_int32), ("fb_budget_bytes", C.c_size_t),
                ("small_pixels", C.c_int64), ("small_batch_pixels", C.c_int64), ("big_wait_s", C.c_double),
                ("use_graph", C.c_int32), ("cooperative", C.c_int32)]
