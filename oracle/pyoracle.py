"""ORACLE — test infrastructure only: ctypes front end of libvlt_oracle.so.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; the
product (violet_gb300) never imports it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build as _build  # noqa: E402
from violet_gb300 import _ffi  # noqa: E402  (struct layouts of include/vlt.h only)

P = C.c_void_p
U32 = C.c_uint32
FP = C.POINTER(_ffi.FrameParams)
PP = C.POINTER(_ffi.Params)

SIGS = {
    "vlto_set_threads": (None, [C.c_int]),
    "vlto_get_threads": (C.c_int, []),
    "vlto_view_create": (P, [U32, U32, PP]),
    "vlto_view_create_form": (P, [U32, U32, PP, C.c_int]),
    "vlto64_create": (P, [U32, U32, PP]),
    "vlto64_destroy": (None, [P]),
    "vlto64_frame": (None, [P, FP, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                             C.c_void_p, C.c_void_p]),
    "vlto_view_destroy": (None, [P]),
    "vlto_view_set_atrous_reference_weights": (None, [P, C.c_int]),
    "vlto_view_enable_fp64": (C.c_int, [P]),
    "vlto_view_fp64_buffer": (U32, [P, C.c_char_p, P, C.c_size_t]),
    "vlto_view_fp64_flips": (C.c_int64, [P]),
    "vlto_view_fp64_flips_by_pass": (C.c_uint32, [P, P]),
    "vlto_frame_run": (None, [P, C.POINTER(_ffi.FrameInputs), C.POINTER(_ffi.FrameOutputs)]),
    "vlto_view_buffer": (P, [P, C.c_char_p, C.POINTER(C.c_size_t)]),
    "vlto_ao_gen": (None, [FP, U32, U32, P, P, P, P, U32, U32, C.c_float]),
    "vlto_ao_filter": (None, [U32, U32, P, P, P]),
    "vlto_ind_diff_temporal_resample": (None, [FP, U32, U32, PP, P, P, P, P, P, P, P, U32, U32, U32]),
    "vlto_ind_diff_spatial_resample": (None, [FP, U32, U32, PP, P, P, P, P, P, P, U32]),
    "vlto_ind_spec_temporal_resample": (None, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, P, P, U32, U32]),
    "vlto_ind_spec_spatial_resample": (None, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, U32]),
    "vlto_denoise_temporal": (None, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, U32, U32]),
    "vlto_denoise_disocclusion_fix": (None, [U32, U32, P, P, P, P, P, P, P]),
    "vlto_denoise_fast_history_clamp": (None, [U32, U32, P, P]),
    "vlto_denoise_spatial_fallback": (None, [U32, U32, P, P, P, P, P, P, P]),
    "vlto_denoise_atrous": (None, [U32, U32, P, P, P, P, P, P, C.c_int]),
    "vlto_frame_trace": (None, [P, C.POINTER(_ffi.FrameInputs), P, P, P, P]),
    "vlto_cache_ray_capacity": (U32, [P]),
    "vlto_final_lighting": (None, [C.c_int, FP, U32, U32, P, P, P, P, C.c_int, P]),
    "vlto_temporal_aa": (None, [C.c_int, FP, U32, U32, P, P, P, U32, P]),
    "vlto_hg_decay": (None, [U32, P, P]),
    "vlto_hg_visualize": (None, [FP, U32, U32, U32, U32, P, P, P, U32, P]),
    "vlto_hg_emit_queries": (None, [FP, U32, U32, U32, U32, U32, P, P, P, P, P]),
    "vlto_hg_query_select": (None, [U32, U32, P, P, P, P, U32]),
    "vlto_hg_query_compact": (None, [U32, U32, P, P, P, P]),
    "vlto_hg_update": (None, [P, P, P, P, P, P]),
    "vlto_hg_find": (None, [FP, U32, U32, P, U32, P, P, P, P]),
    "vlto_math": (None, [C.c_int, P, P, U32]),
    "vlto_codec": (None, [C.c_int, P, P, U32]),
    "vlto_oct": (None, [P, P, P, P, U32]),
    "vlto_lcg_sequence": (None, [U32, U32, U32, U32, P, P]),
    "vlto_xxhash32": (U32, [P, U32]),
    "vlto_oct_decode": (None, [P, P, P, P, U32]),
    "vlto_hit_pos_normal": (None, [P, P, P, P, P, U32]),
    "vlto_vertex_key": (None, [P, P, P, U32]),
    "vlto_gbuffer_decode": (None, [P, P, U32]),
    "vlto_reservoir_encode": (U32, [U32, C.c_float]),
    "vlto_reservoir_decode": (None, [U32, C.POINTER(U32), C.POINTER(C.c_float)]),
}

MATH = {"exp2": 0, "exp": 1, "log2": 2, "sin": 3, "cos": 4, "exp2_fma": 5, "exp2_fma_full": 6, "f16_pair": 7}
CODEC = {"f32tof16": 0, "f16tof32": 1, "uf11": 2, "uf10": 3, "uf11_to_f32": 4, "jenkins": 5, "xorshift": 6,
         "xxh1": 7, "xxh3": 8}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        for k, (r, a) in SIGS.items():
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


def set_threads(n):
    lib().vlto_set_threads(int(n))


def threads():
    return int(lib().vlto_get_threads())


def math(fn, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().vlto_math(MATH[fn], ptr(x), ptr(y), x.size)
    return y


def codec(fn, x):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    y = np.empty_like(x)
    lib().vlto_codec(CODEC[fn], ptr(x), ptr(y), x.size)
    return y


class OracleView:
    """CPU restatement of one view (the same buffer names as violet_gb300.View)."""

    def __init__(self, width, height, params, form="ref"):
        self.width, self.height = int(width), int(height)
        self.params = params
        self.form = form
        self.handle = lib().vlto_view_create_form(self.width, self.height, C.byref(params), _ffi.FORMS[form])

    def _inputs(self, frame_params, frame_index, inputs):
        fi = _ffi.FrameInputs()
        fi.params = C.pointer(frame_params)
        fi.frame_index = int(frame_index) & 0xFFFFFFFF
        for k in ("depth", "gbuffer", "diff_hit_pos_normal", "diff_hit_radiance", "diff_source_pdf", "spec_hit_pos",
                  "spec_hit_radiance", "shadow_mask", "cache_hits", "diffuse_hits", "spec_validate_hits"):
            setattr(fi, k, ptr(inputs.get(k)))
        return fi

    def trace(self, frame_params, frame_index, inputs):
        """Traced mode, phase one: returns (rays dict of float32 arrays, counts dict)."""
        fi = self._inputs(frame_params, frame_index, inputs)
        n = self.width * self.height
        nq = int(lib().vlto_cache_ray_capacity(self.handle))
        rays = {"cache": np.zeros(8 * max(nq, 1), np.float32), "diffuse": np.zeros(8 * n, np.float32),
                "spec_validate": np.zeros(8 * n, np.float32)}
        counts = np.zeros(4, np.uint32)
        lib().vlto_frame_trace(self.handle, C.byref(fi), ptr(rays["cache"]), ptr(rays["diffuse"]),
                               ptr(rays["spec_validate"]), ptr(counts))
        return rays, {"cache": int(counts[0]), "diffuse": int(counts[1]), "spec_validate": int(counts[2]),
                      "diffuse_kind": int(counts[3])}

    def run(self, frame_params, frame_index, inputs, outputs=None):
        fi = self._inputs(frame_params, frame_index, inputs)
        fo = _ffi.FrameOutputs()
        for k in ("diffuse", "specular", "raw_diffuse", "raw_specular", "color", "taa"):
            setattr(fo, k, ptr((outputs or {}).get(k)))
        lib().vlto_frame_run(self.handle, C.byref(fi), C.byref(fo))

    def set_atrous_reference_weights(self, on=True):
        """Float forms: run the a-trous with the reference's edge-stopping formulas
        (svgf.inc.hlsl:60-82, separately rounded) instead of the forms' own
        base-2 / fused-multiply-add evaluation."""
        lib().vlto_view_set_atrous_reference_weights(self.handle, 1 if on else 0)

    def enable_fp64(self):
        """Float forms: from the next frame on, run the binary64 replay of the whole
        back end beside every frame (the float form's decisions replayed)."""
        rc = lib().vlto_view_enable_fp64(self.handle)
        if rc != 0:
            raise ValueError("the binary64 replay needs a float form without traced mode or fast-history clamp")

    def fp64(self, name):
        """The binary64 replay's buffer `name` as a float64 array (pixels, values)."""
        n = self.width * self.height
        k = int(lib().vlto_view_fp64_buffer(self.handle, name.encode(), None, 0))
        if k == 0:
            raise KeyError(name)
        out = np.zeros(n * k, np.float64)
        lib().vlto_view_fp64_buffer(self.handle, name.encode(), out.ctypes.data, out.size)
        return out.reshape(n, k)

    def fp64_flips(self):
        """Decisions of the last frame on which binary64 evaluation would have gone the
        other way (-1: a decision tape overflowed)."""
        return int(lib().vlto_view_fp64_flips(self.handle))

    FLIP_PASSES = ("ao_gen", "ao_filter", "diff_temporal", "diff_spatial", "spec_temporal", "spec_spatial",
                   "denoise")

    def fp64_flips_by_pass(self):
        """The last frame's flips per replayed pass, as {pass: count}."""
        out = np.zeros(len(self.FLIP_PASSES), np.uint64)
        lib().vlto_view_fp64_flips_by_pass(self.handle, out.ctypes.data)
        return {k: int(v) for k, v in zip(self.FLIP_PASSES, out)}

    def form_values(self, name):
        """The float form's own value of a replay buffer `name` (same layout as fp64())."""
        n = self.width * self.height
        f16 = self.form == "f16"
        half = lambda a: a.view(np.float16).astype(np.float64)  # noqa: E731
        if name in ("diff_W", "diff_M"):
            b = self.buffer("diff_reservoir")
            if f16:
                rec = b[: 16 * n].view(np.uint32).reshape(n, 4)
                if name == "diff_W":
                    return rec[:, 3].view(np.float32).astype(np.float64).reshape(n, 1)
                return b[16 * n: 17 * n].astype(np.float64).reshape(n, 1)
            rec = b.view(np.float32).reshape(n, 12)
            if name == "diff_W":
                return rec[:, 3:4].astype(np.float64)
            return rec[:, 7].view(np.uint32).astype(np.float64).reshape(n, 1)
        if name in ("spec_W", "spec_M"):
            rsv = self.buffer("spec_reservoir").view(np.uint32).reshape(n, 2)
            if name == "spec_W":
                return rsv[:, 1].view(np.float32).astype(np.float64).reshape(n, 1)
            return rsv[:, 0].astype(np.float64).reshape(n, 1)
        if name == "ao":
            b = self.buffer("ao_filtered")
            return (half(b) if f16 else b.view(np.float32).astype(np.float64)).reshape(n, 1)
        if name in ("raw_diffuse", "raw_specular", "ray_len"):
            b = self.buffer("raw_specular" if name == "ray_len" else name)
            v = (half(b) if f16 else b.view(np.float32).astype(np.float64)).reshape(n, 4)
            return v[:, 3:4] if name == "ray_len" else v[:, :3]
        if name in ("hist_color", "hist_moments", "variance"):
            b = self.buffer("fallback_record" if name == "variance" else "hist_record")
            v = (half(b) if f16 else b.view(np.float32).astype(np.float64)).reshape(n, 8)
            if name == "hist_color":
                return np.concatenate([v[:, 0:3], v[:, 4:7]], 1)
            aux = v[:, [3, 7]]
            if not f16:
                return aux
            aux = aux * np.abs(aux)  # the FP16 records hold signed square roots
            if name == "hist_moments":  # ... of the variance around the record's colour
                lum = np.array([0.2126, 0.7152, 0.0722])
                aux = aux + np.stack([v[:, 0:3] @ lum, v[:, 4:7] @ lum], 1) ** 2
            return aux
        if name == "hist_len":
            return self.buffer("hist_len").astype(np.float64).reshape(n, 1)
        raise KeyError(name)

    def buffer(self, name, dtype=np.uint8):
        n = C.c_size_t(0)
        p = lib().vlto_view_buffer(self.handle, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        raw = (C.c_uint8 * n.value).from_address(p)
        return np.frombuffer(raw, dtype=np.uint8).copy().view(dtype)

    def close(self):
        if self.handle:
            lib().vlto_view_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Denoiser64:
    """Binary64 denoiser fed with a form's raw lighting (precision reference)."""

    def __init__(self, width, height, params):
        self.width, self.height = int(width), int(height)
        self.params = params
        self.handle = lib().vlto64_create(self.width, self.height, C.byref(params))

    def frame(self, frame_params, host_inputs, diff_rgb, spec_rgb, ray_len, run_denoiser):
        """diff_rgb / spec_rgb: float32 (n, 3); ray_len: float32 (n,). Returns two
        float64 (n, 3) arrays (meaningful when the denoiser ran)."""
        n = self.width * self.height
        d = np.ascontiguousarray(diff_rgb, np.float32)
        s = np.ascontiguousarray(spec_rgb, np.float32)
        r = np.ascontiguousarray(ray_len, np.float32)
        od = np.zeros((n, 3), np.float64)
        os_ = np.zeros((n, 3), np.float64)
        lib().vlto64_frame(self.handle, C.byref(frame_params), ptr(host_inputs["depth"]), ptr(host_inputs["gbuffer"]),
                           ptr(d), ptr(s), ptr(r), 1 if run_denoiser else 0, ptr(od), ptr(os_))
        return od, os_

    def close(self):
        if self.handle:
            lib().vlto64_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
