"""ORACLE — test infrastructure only: the synthetic scene generator's host path
(oracle/_build/libvlt_scene_host.so, the product's generator source compiled without
CUDA), with the same API as violet_gb300.Scene's host methods. The CPU benchmark uses
it so that its process loads the oracle's libraries only."""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build as _build  # noqa: E402
from violet_gb300 import _ffi  # noqa: E402  (struct layouts of include/vlt.h only)

# Frame input buffers (element type, elements per pixel), as violet_gb300.FRAME_BUFFERS.
FRAME_BUFFERS = {
    "depth": (np.float32, 1),
    "gbuffer": (np.uint32, 4),
    "diff_hit_pos_normal": (np.uint32, 2),
    "diff_hit_radiance": (np.uint32, 1),
    "diff_source_pdf": (np.float32, 1),
    "spec_hit_pos": (np.float32, 4),
    "spec_hit_radiance": (np.uint32, 1),
    "shadow_mask": (np.uint8, 1),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_scene_host())
        L.vlt_scene_desc_default.restype = None
        L.vlt_scene_desc_default.argtypes = [C.POINTER(_ffi.SceneDesc), C.c_uint64, C.c_uint32, C.c_uint32]
        L.vlt_scene_frame_params.restype = C.c_int
        L.vlt_scene_frame_params.argtypes = [C.POINTER(_ffi.SceneDesc), C.c_uint32, C.POINTER(_ffi.FrameParams)]
        L.vlt_scene_generate_host.restype = C.c_int
        L.vlt_scene_generate_host.argtypes = [C.POINTER(_ffi.SceneDesc), C.c_uint32, C.POINTER(_ffi.SceneFrame)]
        _lib = L
    return _lib


class Scene:
    def __init__(self, seed, width, height, disocclusion_frac=0.0, camera_speed=0.01, jitter_cycle=8):
        self.desc = _ffi.SceneDesc()
        lib().vlt_scene_desc_default(C.byref(self.desc), int(seed), int(width), int(height))
        self.desc.disocclusion_frac = float(disocclusion_frac)
        self.desc.camera_speed = float(camera_speed)
        self.desc.jitter_cycle = int(jitter_cycle)
        self.width, self.height = int(width), int(height)

    def frame_params(self, frame):
        fp = _ffi.FrameParams()
        rc = lib().vlt_scene_frame_params(C.byref(self.desc), int(frame), C.byref(fp))
        assert rc == 0, "vlt_scene_frame_params failed"
        return fp

    def generate_host(self, frame):
        n = self.width * self.height
        bufs = {k: np.zeros(n * c, dtype=dt) for k, (dt, c) in FRAME_BUFFERS.items()}
        f = _ffi.SceneFrame()
        for k, v in bufs.items():
            setattr(f, k, v.ctypes.data)
        rc = lib().vlt_scene_generate_host(C.byref(self.desc), int(frame), C.byref(f))
        assert rc == 0, "vlt_scene_generate_host failed"
        return bufs
