"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle is a plain C++ restatement of Galaxy's ray path used only as the
parity checker; see gxy_oracle.cpp.  No -march flags (the same source builds
on x86-64 and aarch64) and no fused multiply-add (-ffp-contract=off).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "gxy_oracle.cpp")
    hdr = os.path.join(HERE, "..", "include", "gxy_gpu.h")
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
           "-o", tmp, src, "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
