"""ORACLE build recipe (test infrastructure only).

Compiles the CPU restatement (oracle.cpp, binary32 without FMA contraction) and its
binary64 denoiser (oracle64.cpp) into oracle/_build/libvlt_oracle.so with g++
(OpenMP). The reference's own shaders, compiled as C++ against an HLSL vocabulary
header, are built separately by oracle/ref_build.py into oracle/_ref/ (only where
the reference tree is present); they pin this restatement.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libvlt_oracle.so")
SRCS = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle64.cpp")]
DEPS = SRCS + [os.path.join(HERE, "omath.hpp"), os.path.join(os.path.dirname(HERE), "include", "vlt.h")]
FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(verbose=False, force=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in DEPS):
        return OUT
    cmd = [os.environ.get("CXX", "g++")] + FLAGS + SRCS + ["-o", OUT]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s%s" % (r.stdout, r.stderr))
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
