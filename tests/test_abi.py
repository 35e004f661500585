"""The C ABI library loads without a GPU and exports every entry point that
include/gxy_gpu.h declares; the ctypes struct mirror matches the header."""
import ctypes as C
import os
import re

from galaxy_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gxy_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(gxy_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    from galaxy_gb300 import build, gpu
    build.build()
    lib = C.CDLL(gpu.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes():
    # sizes of the C structs as laid out by the C compiler for this header
    assert C.sizeof(A.gxy_tf) == 4 * (768 + 256 + 2)
    assert C.sizeof(A.gxy_raylist) == 25 * C.sizeof(C.c_void_p) + 8
    assert C.sizeof(A.gxy_lighting) == 4 + 8 * 12 + 8 * 4 + 4 * 5
    assert C.sizeof(A.gxy_camera) == 10 * 4 + 8


def test_gpu_calls_fail_cleanly_without_init_or_device():
    from galaxy_gb300 import gpu
    lib = gpu.lib()
    buf = C.create_string_buffer(256)
    assert lib.gxy_gpu_last_error(buf, 256) == 0
    # a scene commit before gxy_gpu_init is refused, not crashed
    d = A.gxy_scene_desc()
    h = C.c_void_p()
    if not gpu._initialised:
        assert lib.gxy_gpu_scene_commit(C.byref(d), C.byref(h)) == A.GXY_ERR_NOT_INIT
