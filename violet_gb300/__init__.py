"""violet_gb300 — GB300-native per-pixel lighting back end of violet.

ReSTIR GI temporal/spatial reservoir resampling (indirect diffuse and specular),
the ReLAX/SVGF denoiser and the spatial-hash-grid radiance-cache update, as sm_103a
CUDA kernels behind the C ABI of include/vlt.h. This package is a thin Python
front end over that ABI (ctypes); device memory is handed over as raw pointers
(torch tensors are only used as allocations). There is no CPU fallback: if
libvlt.so is missing or no GPU is present, calls raise.
"""
from . import _ffi
from ._ffi import VltError, FrameParams, Params, SceneDesc  # noqa: F401
from .renderer import Context, View, FrameBinding, FrameSequence, Batch, Server, Scene, params_reference, params_plain, FRAME_BUFFERS  # noqa: F401,E501


def lib():
    """The loaded libvlt.so (ctypes.CDLL)."""
    return _ffi.load()
