"""Allocation-free camera rays: gxy_gpu_generate_initial_rays_noalloc.

Some callers may not allocate device memory: a visualization step run in situ
inside a simulation whose own allocator holds the GPU's memory, where a
cudaFree would synchronise the whole device and stall the simulation's
streams.  They pass an output RayList they already hold in memory the GPU can
address (device memory, managed memory or mapped pinned host memory), and the
entry point keeps its scratch in a fixed array inside the library.  These
tests call it through the C ABI and compare its rays with those of
gxy_gpu_generate_initial_rays, bit for bit (the parity tests hold camera rays
to exact equality), on two calls in a row that share the fixed scratch, for
each of the three memory kinds; and check what it refuses.

The file is named to be collected last, so a run that stops at the first
failure has run every other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

from galaxy_gb300 import _abi as A
from galaxy_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from galaxy_gb300 import gpu
    gpu.init(0)
    torch.cuda.set_device(0)
    L = gpu.lib()
    f = L.gxy_gpu_generate_initial_rays_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.POINTER(A.gxy_camera), C.POINTER(A.gxy_raylist),
                  C.POINTER(C.c_int32)]
    f.restype = C.c_int
    return torch, gpu, f


def device_raylist(torch, cap):
    """25 device arrays of `cap` elements, filled with a sentinel so that a
    field the entry point fails to write shows up."""
    arrs = {k: torch.full((cap,), float("nan"), dtype=torch.float32, device="cuda")
            for k in A.RAY_FLOAT_FIELDS}
    arrs.update({k: torch.full((cap,), -7, dtype=torch.int32, device="cuda") for k in A.RAY_INT_FIELDS})
    rl = A.gxy_raylist()
    for k in A.RAY_FLOAT_FIELDS:
        setattr(rl, k, C.cast(C.c_void_p(arrs[k].data_ptr()), A.f32p))
    for k in A.RAY_INT_FIELDS:
        setattr(rl, k, C.cast(C.c_void_p(arrs[k].data_ptr()), A.i32p))
    rl.n = cap
    return arrs, rl


def cudart():
    """The CUDA runtime the library links (same instance, so its managed and
    mapped pinned allocations are the ones the library's checks see)."""
    rt = C.CDLL("libcudart.so.13")
    rt.cudaMallocManaged.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_uint]
    rt.cudaHostAlloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_uint]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaFreeHost.argtypes = [C.c_void_p]
    rt.cudaDeviceSynchronize.argtypes = []
    return rt


class HostVisibleRayList:
    """25 arrays of `cap` records in managed memory (kind "managed") or in
    mapped pinned host memory (kind "pinned"), filled with a sentinel."""

    def __init__(self, kind, cap):
        self.rt = cudart()
        self.kind = kind
        self.ptrs = []
        self.arrs = {}
        rl = A.gxy_raylist()
        for k in A.RAY_FLOAT_FIELDS + A.RAY_INT_FIELDS:
            p = C.c_void_p()
            if kind == "managed":
                assert self.rt.cudaMallocManaged(C.byref(p), cap * 4, 1) == 0   # cudaMemAttachGlobal
            else:
                assert self.rt.cudaHostAlloc(C.byref(p), cap * 4, 2) == 0       # cudaHostAllocMapped
            self.ptrs.append(p.value)
            isf = k in A.RAY_FLOAT_FIELDS
            a = np.ctypeslib.as_array(C.cast(p, A.f32p if isf else A.i32p), (cap,))
            a[:] = np.nan if isf else -7
            self.arrs[k] = a
            setattr(rl, k, C.cast(p, A.f32p if isf else A.i32p))
        rl.n = cap
        self.rl = rl

    def free(self):
        self.rt.cudaDeviceSynchronize()
        for p in self.ptrs:
            (self.rt.cudaFree if self.kind == "managed" else self.rt.cudaFreeHost)(C.c_void_p(p))
        self.ptrs = []


def call_noalloc(gpu, f, scene, part, cam, rl):
    n = C.c_int32(-1)
    rc = f(scene.h, part, C.byref(cam), C.byref(rl), C.byref(n))
    return rc, n.value


def assert_same_rays(arrs, ref, n):
    assert ref.n == n
    for k in A.RAY_FLOAT_FIELDS + A.RAY_INT_FIELDS:
        got = arrs[k][:n]
        got = got.cpu().numpy() if hasattr(got, "cpu") else np.array(got)
        want = getattr(ref, k)
        assert got.dtype == want.dtype, k
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), k


def test_noalloc_matches_allocating_entry_point_twice(env):
    torch, gpu, f = env
    cam_a, vis = scenes.mixed_scene(n=64, n_spheres=4000, width=160, height=120, partitions=(2, 2, 1))
    scene = gpu.Scene(vis)
    cap = 160 * 120
    arrs, rl = device_raylist(torch, cap)
    # first call: partition 1 of a 160x120 image; second call: a smaller
    # 96x72 image of another partition, so the shared scratch still holds
    # the longer first call's flags and offsets beyond the second's pixels
    cam_b = scenes.mixed_scene(n=64, n_spheres=4000, width=96, height=72, partitions=(2, 2, 1))[0]
    cases = [(1, cam_a.c()), (2, cam_b.c())]
    for i, (part, cam) in enumerate(cases):
        ref = scene.generate_initial_rays(part, cam)
        assert ref.n > 0
        hbm0 = gpu.hbm_in_use()
        free0 = torch.cuda.mem_get_info(0)[0] if i else None
        rc, n = call_noalloc(gpu, f, scene, part, cam, rl)
        assert rc == A.GXY_OK, rc
        torch.cuda.synchronize()
        assert gpu.hbm_in_use() == hbm0
        if i:   # everything the call uses was loaded by the first call
            assert torch.cuda.mem_get_info(0)[0] == free0
        assert_same_rays(arrs, ref, n)
    del scene


def test_noalloc_refuses_what_it_cannot_do(env):
    torch, gpu, f = env
    cam, vis = scenes.mixed_scene(n=32, n_spheres=500, width=64, height=48, partitions=(1, 1, 1))
    scene = gpu.Scene(vis)
    arrs, rl = device_raylist(torch, 64 * 48)
    # above the fixed scratch's pixel limit
    big = cam.c()
    big.width, big.height = 1025, 1024
    rc, _ = call_noalloc(gpu, f, scene, 0, big, rl)
    assert rc == A.GXY_ERR_INVALID
    buf = C.create_string_buffer(512)
    gpu.lib().gxy_gpu_last_error(buf, 512)
    assert b"1048576" in buf.value
    # output too small: the ray count is reported, nothing is written
    ref = scene.generate_initial_rays(0, cam.c())
    assert ref.n > 10
    small = A.gxy_raylist.from_buffer_copy(rl)
    small.n = 10
    rc, n = call_noalloc(gpu, f, scene, 0, cam.c(), small)
    assert rc == A.GXY_ERR_OVERFLOW and n == ref.n
    assert torch.isnan(arrs["ox"]).all()
    # host memory the GPU was not given is refused before any launch
    host = A.RayListArrays(64 * 48)
    hrl = host.c()
    rc, _ = call_noalloc(gpu, f, scene, 0, cam.c(), hrl)
    assert rc == A.GXY_ERR_INVALID
    # the entry point still works after the refusals
    rc, n = call_noalloc(gpu, f, scene, 0, cam.c(), rl)
    assert rc == A.GXY_OK
    assert_same_rays(arrs, ref, n)
    del scene


@pytest.mark.parametrize("kind", ["managed", "pinned"])
def test_noalloc_host_visible_memory_twice(env, kind):
    """The two other memory kinds the entry point accepts: managed memory
    and mapped pinned host memory, two calls in a row, bit for bit."""
    torch, gpu, f = env
    cam_a, vis = scenes.mixed_scene(n=64, n_spheres=4000, width=128, height=96, partitions=(2, 1, 1))
    cam_b = scenes.mixed_scene(n=64, n_spheres=4000, width=80, height=64, partitions=(2, 1, 1))[0]
    scene = gpu.Scene(vis)
    out = HostVisibleRayList(kind, 128 * 96)
    try:
        for part, cam in ((0, cam_a.c()), (1, cam_b.c())):
            ref = scene.generate_initial_rays(part, cam)
            assert ref.n > 0
            rc, n = call_noalloc(gpu, f, scene, part, cam, out.rl)
            assert rc == A.GXY_OK, rc
            assert_same_rays(out.arrs, ref, n)
    finally:
        out.free()
    del scene


def test_noalloc_refuses_capacity_beyond_the_arrays(env):
    """A capacity larger than the caller's arrays is refused before anything
    is written: the whole range must lie inside one allocation (arrays of
    their own cudaMalloc here; a caching allocator's tensors lie inside its
    larger segments, which is all the check can see)."""
    torch, gpu, f = env
    cam, vis = scenes.mixed_scene(n=32, n_spheres=500, width=64, height=48, partitions=(1, 1, 1))
    scene = gpu.Scene(vis)
    rt = cudart()
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    cap = 64
    sentinel = np.full(cap, np.nan, np.float32)
    ptrs = []
    rl = A.gxy_raylist()
    try:
        for k in A.RAY_FLOAT_FIELDS + A.RAY_INT_FIELDS:
            p = C.c_void_p()
            assert rt.cudaMalloc(C.byref(p), cap * 4) == 0
            assert rt.cudaMemcpy(p, sentinel.ctypes.data, cap * 4, 1) == 0   # host to device
            ptrs.append(p)
            setattr(rl, k, C.cast(p, A.f32p if k in A.RAY_FLOAT_FIELDS else A.i32p))
        rl.n = 64 * 48
        rc, _ = call_noalloc(gpu, f, scene, 0, cam.c(), rl)
        assert rc == A.GXY_ERR_INVALID
        back = np.zeros(cap, np.float32)
        assert rt.cudaMemcpy(back.ctypes.data, ptrs[0], cap * 4, 2) == 0     # device to host
        assert np.isnan(back).all()
        # the same arrays with their true capacity are accepted
        rl.n = cap
        rc, n = call_noalloc(gpu, f, scene, 0, cam.c(), rl)
        assert rc in (A.GXY_OK, A.GXY_ERR_OVERFLOW)
    finally:
        rt.cudaDeviceSynchronize()
        for p in ptrs:
            rt.cudaFree(p)
    del scene
