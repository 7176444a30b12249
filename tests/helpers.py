"""Shared test helpers: host<->device copies through the CUDA runtime, frame upload."""
import ctypes as C

import numpy as np

import violet_gb300 as vg

_cudart = None


def cudart():
    global _cudart
    if _cudart is None:
        _cudart = C.CDLL("libcudart.so.13")
    return _cudart


def d2h(ptr, nbytes, dtype=np.uint8):
    out = np.empty(nbytes, np.uint8)
    if nbytes:
        rc = cudart().cudaMemcpy(C.c_void_p(out.ctypes.data), C.c_void_p(ptr), C.c_size_t(nbytes), 2)
        assert rc == 0, "cudaMemcpy D2H failed (%d)" % rc
    return out.view(dtype)


def h2d(ptr, arr):
    arr = np.ascontiguousarray(arr)
    rc = cudart().cudaMemcpy(C.c_void_p(ptr), C.c_void_p(arr.ctypes.data), C.c_size_t(arr.nbytes), 1)
    assert rc == 0, "cudaMemcpy H2D failed (%d)" % rc


def dev_zeros(nbytes):
    import torch

    return torch.zeros(max(int(nbytes), 16), dtype=torch.uint8, device="cuda")


def upload(host):
    """Host frame dict (numpy) -> device frame dict (torch uint8 tensors)."""
    import torch

    return {k: torch.from_numpy(np.ascontiguousarray(v).view(np.uint8)).cuda() for k, v in host.items()}


def to_np(t, dtype):
    return t.cpu().numpy().view(dtype)


def float_bits_equal(a, b):
    """Bitwise equality of float32 arrays, treating every NaN as equal."""
    a = np.asarray(a).view(np.uint32)
    b = np.asarray(b).view(np.uint32)
    na = (a & 0x7FFFFFFF) > 0x7F800000
    nb = (b & 0x7FFFFFFF) > 0x7F800000
    return bool(np.all((a == b) | (na & nb)))


def first_mismatch(a, b, width=None, rec=1):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    idx = np.nonzero(a != b)[0]
    if idx.size == 0:
        return None
    i = int(idx[0])
    px = i // rec
    where = (px % width, px // width) if width else px
    return "%d mismatching words; first at word %d (pixel %s): got 0x%08x expected 0x%08x" % (
        idx.size, i, where, int(a[i]), int(b[i]))


def rel_l2(got, exp):
    """||got - exp|| / ||exp|| over the finite entries, and whether the NaN/inf
    patterns agree (both must be non-finite at the same places)."""
    got = np.asarray(got, np.float64).reshape(-1)
    exp = np.asarray(exp, np.float64).reshape(-1)
    fg, fe = np.isfinite(got), np.isfinite(exp)
    same_pattern = bool(np.array_equal(fg, fe))
    m = fg & fe
    den = float(np.sqrt(np.sum(exp[m] ** 2)))
    num = float(np.sqrt(np.sum((got[m] - exp[m]) ** 2)))
    return (num / den if den > 0 else num), same_pattern


def first_float_mismatch(a, b, width=None, rec=1):
    """first_mismatch over float32 words, treating any two NaNs as equal."""
    a = np.asarray(a).reshape(-1).view(np.uint32)
    b = np.asarray(b).reshape(-1).view(np.uint32)
    na = (a & 0x7FFFFFFF) > 0x7F800000
    nb = (b & 0x7FFFFFFF) > 0x7F800000
    bad = (a != b) & ~(na & nb)
    if not bad.any():
        return None
    return first_mismatch(np.where(bad, a, 0), np.where(bad, b, 0), width, rec)


def ref_golden_cases():
    """The cases of tests/golden/ref_passes.npz (made from the reference's own shaders
    by tests/golden/make_ref_golden.py): a list of (pass name, args, expected outputs);
    args are (kind, value) with kind in fp, params, in, out, inout, u32, i32, f32, none."""
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_passes.npz")
    z = np.load(path)
    man = json.loads(bytes(z["manifest"]).decode())
    out = []
    for c in man["cases"]:
        args = [(k, z[v] if k in ("fp", "params", "in", "out", "inout") else v) for k, v in c["args"]]
        out.append((c["pass"], args, [z[k] for k in c["expect"]]))
    return out


def call_with_args(fn, args, arrays_in, fp_type, params_type):
    """Calls fn with the fixture args; `arrays_in(kind, ndarray)` turns an array argument
    into a pointer (and keeps whatever it allocates). Returns the ctypes call list."""
    call, keep = [], []
    for kind, v in args:
        if kind == "fp":
            s = fp_type.from_buffer_copy(v.tobytes())
            keep.append(s)
            call.append(C.byref(s))
        elif kind == "params":
            s = params_type.from_buffer_copy(v.tobytes())
            keep.append(s)
            call.append(C.byref(s))
        elif kind in ("in", "out", "inout"):
            call.append(arrays_in(kind, v))
        elif kind == "u32":
            call.append(C.c_uint32(v))
        elif kind == "i32":
            call.append(C.c_int32(v))
        elif kind == "f32":
            call.append(C.c_float(v))
        else:
            call.append(None)
    return call, keep
