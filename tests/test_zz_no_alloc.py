"""Allocation-free camera rays: gxy_gpu_generate_initial_rays_noalloc.

Some callers may not allocate device memory: a visualization step run in situ
inside a simulation whose own allocator holds the GPU's memory, where a
cudaFree would synchronise the whole device and stall the simulation's
streams.  They pass an output RayList they already hold in device memory, and
the entry point keeps its scratch in a fixed array inside the library.  These
tests call it through the C ABI and compare its rays with those of
gxy_gpu_generate_initial_rays, bit for bit (the parity tests hold camera rays
to exact equality), on two calls in a row that share the fixed scratch.

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


def call_noalloc(gpu, f, scene, part, cam, rl):
    n = C.c_int32(-1)
    rc = f(scene.h, part, C.byref(cam), C.byref(rl), C.byref(n))
    return rc, n.value


def assert_same_rays(arrs, ref, n):
    assert ref.n == n
    for k in A.RAY_FLOAT_FIELDS + A.RAY_INT_FIELDS:
        got = arrs[k][:n].cpu().numpy()
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
