"""The C ABI library loads without a GPU and exports every entry point that
include/gxy_gpu.h declares; the ctypes struct mirrors have the header's
layout."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

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


MIRRORED = ("gxy_tf", "gxy_volume_vis", "gxy_triangles_vis", "gxy_particles_vis", "gxy_pathlines_vis",
            "gxy_lighting", "gxy_camera", "gxy_scene_desc", "gxy_raylist", "gxy_partition_info", "gxy_counters",
            "gxy_generation_stats", "gxy_job", "gxy_server_config")


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler
    gives the header's struct (a C program built against the header prints
    them)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gxy_gpu.h"', "int main(void) {"]
    for name in MIRRORED:
        st = getattr(A, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in st._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)]).decode().splitlines() if line)
    for name in MIRRORED:
        st = getattr(A, name)
        assert int(got[name]) == C.sizeof(st), name
        for f, _ in st._fields_:
            assert int(got["%s.%s" % (name, f)]) == getattr(st, f).offset, (name, f)


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
