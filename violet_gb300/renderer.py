"""Python front end of the C ABI: views (RestirRenderer + Denoiser state) and the
synthetic scene.

The call sequence mirrors RestirRenderer::add_passes / Denoiser::add_passes of
crates/violet-restir/src/{restir_renderer.rs,denoising.rs}: one `View.run` per
frame with that frame's G-buffer, candidate samples and FrameParams.
"""
import ctypes as C

import numpy as np

from . import _ffi

# Per-frame input buffers: name -> (numpy dtype, elements per pixel).
FRAME_BUFFERS = {
    "depth": (np.float32, 1),
    "gbuffer": (np.uint32, 4),  # layer-planar: 4 planes of W*H
    "diff_hit_pos_normal": (np.uint32, 2),
    "diff_hit_radiance": (np.uint32, 1),
    "diff_source_pdf": (np.float32, 1),
    "spec_hit_pos": (np.float32, 4),
    "spec_hit_radiance": (np.uint32, 1),
    "shadow_mask": (np.uint8, 1),
}


def params_reference():
    p = _ffi.Params()
    _ffi.load().vlt_params_reference(C.byref(p))
    return p


def params_plain(config):
    p = _ffi.Params()
    _ffi.load().vlt_params_plain(C.byref(p), int(config))
    return p


def _ptr(x):
    """Device/host address of a torch tensor, numpy array, int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError("cannot take the address of %r" % type(x))


class Context:
    def __init__(self, device=0):
        self._lib = _ffi.load()
        h = C.c_void_p()
        _ffi.check(self._lib.vlt_ctx_create(int(device), C.byref(h)), "vlt_ctx_create")
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self._lib.vlt_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _frame_structs(frame_params, frame_index, inputs, outputs):
    fi = _ffi.FrameInputs()
    fi.params = C.pointer(frame_params)
    fi.frame_index = int(frame_index) & 0xFFFFFFFF
    for name in ("depth", "gbuffer", "prev_depth", "prev_gbuffer", "diff_hit_pos_normal", "diff_hit_radiance",
                 "diff_source_pdf", "spec_hit_pos", "spec_hit_radiance", "shadow_mask", "cache_hits", "diffuse_hits",
                 "spec_validate_hits"):
        setattr(fi, name, _ptr(inputs.get(name)))
    fo = _ffi.FrameOutputs()
    outputs = outputs or {}
    for name in ("diffuse", "specular", "raw_diffuse", "raw_specular", "color", "taa"):
        setattr(fo, name, _ptr(outputs.get(name)))
    return fi, fo


class FrameBinding:
    """The input and output pointers of vlt_frame_run bound once, for buffers that are
    reused frame after frame (staging slots); View.run_bound fills in the frame."""

    def __init__(self, inputs, outputs=None):
        self.fi, self.fo = _frame_structs(_ffi.FrameParams(), 0, inputs, outputs)
        self._keep = (inputs, outputs)  # the buffers must outlive the binding


class FrameSequence:
    """The argument arrays of vlt_frames_run for n frames, built once: frame k runs
    frame_indices[k] with frame_params[k], inputs[k] and outputs[k] (outputs may be
    None: no outputs for any frame)."""

    def __init__(self, frame_params, frame_indices, inputs, outputs=None):
        n = len(inputs)
        if not (len(frame_params) == len(frame_indices) == n) or (outputs is not None and len(outputs) != n):
            raise ValueError("FrameSequence: one frame_params, frame index, inputs (and outputs) per frame")
        self.n = n
        self.fis = (_ffi.FrameInputs * n)()
        self.fos = (_ffi.FrameOutputs * n)() if outputs is not None else None
        for k in range(n):
            fi, fo = _frame_structs(frame_params[k], frame_indices[k], inputs[k], outputs[k] if outputs else None)
            self.fis[k] = fi
            if self.fos is not None:
                self.fos[k] = fo
        self._keep = (list(frame_params), inputs, outputs)  # everything must outlive the arrays


class View:
    """Resident per-view state and the per-frame pass sequence (vlt_frame_run)."""

    def __init__(self, ctx, width, height, form="ref", params=None):
        self._lib = _ffi.load()
        self.ctx = ctx
        self.width, self.height = int(width), int(height)
        self.form = form
        self.params = params if params is not None else params_reference()
        h = C.c_void_p()
        _ffi.check(
            self._lib.vlt_view_create(ctx.handle, self.width, self.height, _ffi.FORMS[form], C.byref(self.params),
                                      C.byref(h)),
            "vlt_view_create",
        )
        self.handle = h

    @staticmethod
    def device_bytes(width, height, form="ref", params=None):
        lib = _ffi.load()
        p = params if params is not None else params_reference()
        return int(lib.vlt_view_device_bytes(int(width), int(height), _ffi.FORMS[form], C.byref(p)))

    def run(self, frame_params, frame_index, inputs, outputs=None, stream=0):
        fi, fo = _frame_structs(frame_params, frame_index, inputs, outputs)
        _ffi.check(self._lib.vlt_frame_run(self.handle, C.byref(fi), C.byref(fo), C.c_void_p(stream)),
                   "vlt_frame_run")

    def run_bound(self, binding, frame_params, frame_index, stream=0):
        """vlt_frame_run with the pointers of a FrameBinding."""
        binding.fi.params = C.pointer(frame_params)
        binding.fi.frame_index = int(frame_index) & 0xFFFFFFFF
        _ffi.check(self._lib.vlt_frame_run(self.handle, C.byref(binding.fi), C.byref(binding.fo),
                                           C.c_void_p(stream)), "vlt_frame_run")

    def run_sequence(self, seq, stream=0):
        """vlt_frames_run over a FrameSequence: its frames in order, each frame's
        denoiser beside the next frame's resampling passes; results equal
        run() frame by frame."""
        _ffi.check(self._lib.vlt_frames_run(self.handle, seq.n, seq.fis, seq.fos, C.c_void_p(stream)),
                   "vlt_frames_run")

    def trace(self, frame_params, frame_index, inputs, rays, stream=0):
        """Phase one of a traced frame (params.trace = 1): fills the device ray arrays
        rays["cache"], rays["diffuse"], rays["spec_validate"] (vlt_ray records) and
        returns {"cache", "diffuse", "spec_validate": rays to trace, "diffuse_kind"}."""
        fi, _ = _frame_structs(frame_params, frame_index, inputs, None)
        fr = _ffi.FrameRays()
        for k in ("cache", "diffuse", "spec_validate"):
            setattr(fr, k, _ptr(rays.get(k)))
        _ffi.check(self._lib.vlt_frame_trace(self.handle, C.byref(fi), C.byref(fr), C.c_void_p(stream)),
                   "vlt_frame_trace")
        return {"cache": fr.n_cache, "diffuse": fr.n_diffuse, "spec_validate": fr.n_spec_validate,
                "diffuse_kind": fr.diffuse_kind}

    @property
    def state_bytes(self):
        return int(self._lib.vlt_view_state_bytes(self.handle))

    def export_state(self, dst=None, stream=0):
        """The view's temporal state into `dst` (host numpy array or device tensor of
        state_bytes bytes; a new uint8 numpy array when None). Returns dst."""
        if dst is None:
            dst = np.empty(self.state_bytes, np.uint8)
        nb = dst.nbytes if isinstance(dst, np.ndarray) else dst.numel() * dst.element_size()
        _ffi.check(self._lib.vlt_view_export_state(self.handle, _ptr(dst), nb, C.c_void_p(stream)),
                   "vlt_view_export_state")
        return dst

    def import_state(self, src, stream=0):
        nb = src.nbytes if isinstance(src, np.ndarray) else src.numel() * src.element_size()
        _ffi.check(self._lib.vlt_view_import_state(self.handle, _ptr(src), nb, C.c_void_p(stream)),
                   "vlt_view_import_state")

    @property
    def cache_ray_capacity(self):
        return int(self._lib.vlt_view_cache_ray_capacity(self.handle))

    def buffer(self, name):
        n = C.c_size_t(0)
        p = self._lib.vlt_view_buffer(self.handle, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        return int(p), int(n.value)

    def reset(self, stream=0):
        _ffi.check(self._lib.vlt_view_reset(self.handle, C.c_void_p(stream)), "vlt_view_reset")

    def set_timing(self, enable=True):
        _ffi.check(self._lib.vlt_view_set_timing(self.handle, 1 if enable else 0), "vlt_view_set_timing")

    def read_timing(self):
        """{pass name: (launches, total ms)} accumulated since the last read."""
        n = self._lib.vlt_view_read_timing(self.handle, None, 0)
        arr = (_ffi.PassTime * max(n, 1))()
        n = self._lib.vlt_view_read_timing(self.handle, arr, n)
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n)}

    @property
    def launches(self):
        return int(self._lib.vlt_view_last_launch_count(self.handle))

    def close(self):
        if self.handle:
            self._lib.vlt_view_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """Seeded synthetic frames (G-buffer, camera, candidate samples)."""

    def __init__(self, seed, width, height, disocclusion_frac=0.0, camera_speed=0.01, jitter_cycle=8):
        self._lib = _ffi.load()
        self.desc = _ffi.SceneDesc()
        self._lib.vlt_scene_desc_default(C.byref(self.desc), int(seed), int(width), int(height))
        self.desc.disocclusion_frac = float(disocclusion_frac)
        self.desc.camera_speed = float(camera_speed)
        self.desc.jitter_cycle = int(jitter_cycle)
        self.width, self.height = int(width), int(height)

    def frame_params(self, frame):
        fp = _ffi.FrameParams()
        _ffi.check(self._lib.vlt_scene_frame_params(C.byref(self.desc), int(frame), C.byref(fp)),
                   "vlt_scene_frame_params")
        return fp

    def alloc_host(self):
        n = self.width * self.height
        return {k: np.zeros(n * c, dtype=dt) for k, (dt, c) in FRAME_BUFFERS.items()}

    def _frame_struct(self, bufs):
        f = _ffi.SceneFrame()
        for k in FRAME_BUFFERS:
            setattr(f, k, _ptr(bufs.get(k)))
        return f

    def trace_host(self, frame_params, rays, n=None):
        """Traces host vlt_ray records (a uint8/float32 numpy array) against the scene;
        returns the vlt_ray_hit records as a float32 array (16 per ray)."""
        rays = np.ascontiguousarray(rays)
        n = rays.nbytes // _ffi.RAY_BYTES if n is None else int(n)
        hits = np.zeros(16 * n, np.float32)
        _ffi.check(self._lib.vlt_scene_trace_host(C.byref(self.desc), C.byref(frame_params), _ptr(rays), n,
                                                  _ptr(hits)), "vlt_scene_trace_host")
        return hits

    def trace_device(self, frame_params, rays, n, hits, stream=0):
        """Traces n device vlt_ray records into device vlt_ray_hit records."""
        _ffi.check(self._lib.vlt_scene_trace_device(C.byref(self.desc), C.byref(frame_params), _ptr(rays), int(n),
                                                    _ptr(hits), C.c_void_p(stream)), "vlt_scene_trace_device")

    def generate_host(self, frame, bufs=None):
        bufs = bufs if bufs is not None else self.alloc_host()
        f = self._frame_struct(bufs)
        _ffi.check(self._lib.vlt_scene_generate_host(C.byref(self.desc), int(frame), C.byref(f)),
                   "vlt_scene_generate_host")
        return bufs

    def generate_device(self, frame, bufs, stream=0):
        f = self._frame_struct(bufs)
        _ffi.check(self._lib.vlt_scene_generate_device(C.byref(self.desc), int(frame), C.byref(f),
                                                       C.c_void_p(stream)), "vlt_scene_generate_device")
        return bufs


class Batch:
    """One frame of many views per call, as batched launches (vlt_batch_run)."""

    def __init__(self, ctx):
        self._lib = _ffi.load()
        self.ctx = ctx
        h = C.c_void_p()
        _ffi.check(self._lib.vlt_batch_create(ctx.handle, C.byref(h)), "vlt_batch_create")
        self.handle = h

    def run(self, views, frame_params, frame_indices, inputs, outputs=None, stream=0):
        """views[k] runs frame frame_indices[k] with frame_params[k], inputs[k] and
        outputs[k] (dicts of device buffers, as View.run takes)."""
        n = len(views)
        fis = (_ffi.FrameInputs * n)()
        fos = (_ffi.FrameOutputs * n)()
        keep = []
        for k in range(n):
            fi, fo = _frame_structs(frame_params[k], frame_indices[k], inputs[k], outputs[k] if outputs else None)
            fis[k] = fi
            fos[k] = fo
            keep.append(frame_params[k])
        vh = (C.c_void_p * n)(*[v.handle.value for v in views])
        _ffi.check(self._lib.vlt_batch_run(self.handle, vh, fis, fos if outputs else None, n, C.c_void_p(stream)),
                   "vlt_batch_run")

    def set_graphs(self, enable=True):
        _ffi.check(self._lib.vlt_batch_set_graphs(self.handle, 1 if enable else 0), "vlt_batch_set_graphs")

    def set_chunk_pixels(self, pixels):
        _ffi.check(self._lib.vlt_batch_set_chunk_pixels(self.handle, int(pixels)), "vlt_batch_set_chunk_pixels")

    def set_persistent(self, enable=True):
        _ffi.check(self._lib.vlt_batch_set_persistent(self.handle, 1 if enable else 0), "vlt_batch_set_persistent")

    def autotune(self):
        _ffi.check(self._lib.vlt_batch_autotune(self.handle), "vlt_batch_autotune")

    def tile_table(self):
        n = self._lib.vlt_batch_tile_table(self.handle, None, 0)
        arr = (_ffi.TileChoice * max(n, 1))()
        n = self._lib.vlt_batch_tile_table(self.handle, arr, n)
        return {arr[i].pass_.decode(): {"tile": (arr[i].bx, arr[i].by), "persistent": bool(arr[i].persistent),
                                        "ns_per_kpix": list(arr[i].ns_per_kpix)} for i in range(n)}

    def stats(self):
        st = _ffi.BatchStats()
        _ffi.check(self._lib.vlt_batch_get_stats(self.handle, C.byref(st)), "vlt_batch_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if self.handle:
            self._lib.vlt_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """View-sessions admitted by HBM and per-step pixel budgets; each step batches
    the next queued frame of every admitted session (vlt_server_*)."""

    def __init__(self, ctx, hbm_budget_bytes, step_pixel_budget=0, max_sessions=0):
        self._lib = _ffi.load()
        self.ctx = ctx
        cfg = _ffi.ServerConfig(int(hbm_budget_bytes), int(step_pixel_budget), int(max_sessions))
        h = C.c_void_p()
        _ffi.check(self._lib.vlt_server_create(ctx.handle, C.byref(cfg), C.byref(h)), "vlt_server_create")
        self.handle = h
        self._keep = {}  # frame params / structs referenced by queued frames

    def open(self, width, height, form="ref", params=None):
        p = params if params is not None else params_reference()
        sid = C.c_uint64()
        _ffi.check(self._lib.vlt_server_open(self.handle, int(width), int(height), _ffi.FORMS[form], C.byref(p),
                                             C.byref(sid)), "vlt_server_open")
        return sid.value

    def submit(self, session, frame_params, frame_index, inputs, outputs=None, tag=0):
        fi, fo = _frame_structs(frame_params, frame_index, inputs, outputs)
        _ffi.check(self._lib.vlt_server_submit(self.handle, C.c_uint64(session), C.byref(fi),
                                               C.byref(fo) if outputs else None, C.c_uint64(tag)),
                   "vlt_server_submit")

    def close_session(self, session):
        _ffi.check(self._lib.vlt_server_close(self.handle, C.c_uint64(session)), "vlt_server_close")

    def step(self, stream=0):
        n = C.c_uint32()
        _ffi.check(self._lib.vlt_server_step(self.handle, C.c_void_p(stream), C.byref(n)), "vlt_server_step")
        return n.value

    def poll(self, wait=False, max_items=4096):
        arr = (_ffi.ServerCompletion * max_items)()
        n = self._lib.vlt_server_poll(self.handle, arr, max_items, 1 if wait else 0)
        return [(arr[i].session, arr[i].tag, arr[i].latency_ms, arr[i].step_ms) for i in range(n)]

    def batch_handle(self):
        return self._lib.vlt_server_batch(self.handle)

    def autotune(self):
        _ffi.check(self._lib.vlt_batch_autotune(C.c_void_p(self.batch_handle())), "vlt_batch_autotune")

    def stats(self):
        st = _ffi.ServerStats()
        _ffi.check(self._lib.vlt_server_get_stats(self.handle, C.byref(st)), "vlt_server_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if self.handle:
            self._lib.vlt_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
