"""Builds libvlt.so (the CUDA kernels + C ABI) for sm_103a, in-tree.

Each translation unit is compiled in parallel with nvcc; the product numeric
contract needs --fmad=false (no FMA contraction in device code) and
-ffp-contract=off for host code, so kernel results match the CPU restatement
bit for bit.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvlt.so")

SOURCES = ["restir.cu", "denoise.cu", "denoise_f32.cu", "hashgrid.cu", "trace.cu", "post.cu", "scene.cu", "launch.cu", "api.cu", "batch.cu", "server.cu"]
HEADERS = ["vlt_math.cuh", "vlt_device.cuh", "vlt_launch.cuh", "vlt_internal.h", "brdf.cuh", "scene_gen.cuh", "trace.cuh",
           "hashgrid.cuh", "vlt_compact.cuh"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = os.path.join(os.path.dirname(HERE), "include")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(inc, h) for h in ("vlt.h", "vlt_scene.h")]

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        if force or _newer(o, [s] + hdrs):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _newer(LIB, objs):
        cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
