"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle is a plain C++ restatement of Galaxy's ray path used only as the
parity checker and the timed CPU baseline; see gxy_oracle.cpp.  -O3 lets the
compiler vectorise with the ISA baseline of the host (SSE2 on x86-64, NEON on
aarch64); no -march flags, so the same source builds and gives the same
results on both, and no fused multiply-add (-ffp-contract=off), so the
optimisation level changes no result.
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
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
           "-o", tmp, src, "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
