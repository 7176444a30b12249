"""ORACLE build recipe (test infrastructure only).

Compiles the CPU restatement (oracle.cpp, binary32 without FMA contraction), its
binary64 denoiser (oracle64.cpp) and the binary64 replay of the float forms' whole
back end (oracle64r.cpp) into oracle/_build/libvlt_oracle.so with g++ (OpenMP). The reference's own shaders, compiled as C++ against an HLSL vocabulary
header, are built separately by oracle/ref_build.py into oracle/_ref/ (only where
the reference tree is present); they pin this restatement.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libvlt_oracle.so")
SRCS = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle64.cpp"), os.path.join(HERE, "oracle64r.cpp")]
DEPS = SRCS + [os.path.join(HERE, "omath.hpp"), os.path.join(HERE, "oracle64r.hpp"),
               os.path.join(os.path.dirname(HERE), "include", "vlt.h")]
FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


# The synthetic scene generator's host path, compiled from the product's source
# without CUDA: the CPU benchmark of the oracle synthesises its inputs with it, so that
# its process never loads the product library.
SCENE_SRC = os.path.join(os.path.dirname(HERE), "violet_gb300", "csrc", "scene.cu")
SCENE_OUT = os.path.join(HERE, "_build", "libvlt_scene_host.so")
SCENE_DEPS = [SCENE_SRC] + [os.path.join(os.path.dirname(HERE), "violet_gb300", "csrc", h)
                            for h in ("scene_gen.cuh", "vlt_math.cuh")] + [
    os.path.join(os.path.dirname(HERE), "include", h) for h in ("vlt.h", "vlt_scene.h")]


def build_scene_host(verbose=False, force=False):
    os.makedirs(os.path.dirname(SCENE_OUT), exist_ok=True)
    if not force and os.path.exists(SCENE_OUT) and all(
            os.path.getmtime(d) <= os.path.getmtime(SCENE_OUT) for d in SCENE_DEPS):
        return SCENE_OUT
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-x", "c++", "-DVLT_SCENE_HOST_ONLY", SCENE_SRC, "-o", SCENE_OUT, "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host scene build failed:\n%s%s" % (r.stdout, r.stderr))
    return SCENE_OUT


def build(verbose=False, force=False):
    build_scene_host(verbose, force)
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
