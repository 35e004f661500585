"""Build libgxy_gpu.so (the CUDA kernels and the C ABI) for sm_103a, and the
C++ host layer over it (libgxy_host.so and the gxywriter program).

nvcc compiles each .cu in parallel, then links one shared library into
galaxy_gb300/_build/; g++ then builds the host layer (host/*.cpp, no CUDA
headers) against include/gxy_gpu.h and that library.  Device code is built with -fmad=false so its
rounding is the one the ray-path semantics state (the BVH box test uses
explicit fused multiply-adds); host code with -ffp-contract=off for the
same reason on aarch64 hosts, where contraction is the default.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgxy_gpu.so")
SOURCES = ["render.cu", "bvh.cu", "server.cu"]
HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(OUT_DIR, "libgxy_host.so")
GXYWRITER = os.path.join(OUT_DIR, "gxywriter")
HEADERS = ["gxy_dev.cuh", "gxy_host.h", "trace.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include")]


def _stale(out, deps):
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "gxy_gpu.h")]
    objs, jobs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc()] + flags() + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    build_host(force, verbose)
    return LIB


def _cuda_lib_dir():
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path()))), "lib64")


def nvcc_path():
    import shutil
    c = nvcc()
    return c if os.path.sep in c else (shutil.which(c) or "/usr/local/cuda/bin/nvcc")


def build_host(force=False, verbose=False):
    """The C++ host layer: libgxy_host.so and gxywriter, linked to
    libgxy_gpu.so (found beside them at run time)."""
    srcs = [os.path.join(HOST, "galaxy_host.cpp")]
    deps = srcs + [os.path.join(HOST, h) for h in ("galaxy_host.hpp", "json.hpp")] + \
        [os.path.join(HERE, "..", "include", "gxy_gpu.h"), LIB]
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + HOST]
    link = ["-L" + OUT_DIR, "-lgxy_gpu", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath-link," + _cuda_lib_dir(),
            "-Wl,-rpath," + _cuda_lib_dir()]
    for out, extra, flags in ((HOST_LIB, [], ["-shared"]), (GXYWRITER, [os.path.join(HOST, "gxywriter.cpp")], [])):
        if not force and not _stale(out, deps + extra):
            continue
        tmp = out + ".tmp%d" % os.getpid()
        cmd = cxx + flags + ["-o", tmp] + srcs + extra + link
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(tmp, out)
    return HOST_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
