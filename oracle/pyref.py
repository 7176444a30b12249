"""ORACLE — test infrastructure only: ctypes front end of oracle/_ref/libvlt_ref.so,
the reference's own HLSL shaders compiled as C++ (oracle/ref_build.py).

lib() returns None where the reference tree is absent (the library cannot be built
there); callers skip.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref_build as _build  # noqa: E402
from violet_gb300 import _ffi  # noqa: E402  (struct layouts of include/vlt.h only)

P = C.c_void_p
U32 = C.c_uint32
FP = C.POINTER(_ffi.FrameParams)

SIGS = {
    "vltr_jenkins_hash": (None, [P, P, U32]),
    "vltr_lcg_sequence": (None, [U32, U32, U32, U32, P, P]),
    "vltr_xxhash32": (U32, [P, U32]),
    "vltr_oct_encode": (None, [P, P, P, U32]),
    "vltr_oct_decode": (None, [P, P, P, P, U32]),
    "vltr_reservoir_simple": (None, [P, P, P, P, P, U32]),
    "vltr_hit_pos_normal": (None, [P, P, P, P, P, U32]),
    "vltr_vertex_key": (None, [P, P, P, U32]),
    "vltr_gbuffer_decode": (None, [P, P, U32]),
}

_lib = None
_tried = False


def lib():
    global _lib, _tried
    if _lib is None and not _tried:
        _tried = True
        path = _build.build()
        if path is None:
            return None
        L = C.CDLL(path)
        for k, (r, a) in SIGS.items():
            if hasattr(L, k):
                f = getattr(L, k)
                f.restype = r
                f.argtypes = a
        _lib = L
    return _lib


def ptr(a):
    if a is None:
        return None
    assert isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"], "host arrays must be contiguous numpy arrays"
    return a.ctypes.data
