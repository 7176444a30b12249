"""ctypes declarations of the C ABI in include/vlt.h and include/vlt_scene.h."""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvlt.so")

VLT_OK = 0
STATUS_NAMES = {
    0: "VLT_OK",
    1: "VLT_ERR_INVALID_ARG",
    2: "VLT_ERR_OUT_OF_MEMORY",
    3: "VLT_ERR_BUDGET_EXCEEDED",
    4: "VLT_ERR_CUDA",
    5: "VLT_ERR_DEVICE_TIMEOUT",
    6: "VLT_ERR_BAD_STATE",
    7: "VLT_ERR_NO_DEVICE",
}
FORMS = {"ref": 0, "f32": 1, "f16": 2}


class FrameParams(C.Structure):
    _fields_ = [
        ("view_proj", C.c_float * 16),
        ("inv_view_proj", C.c_float * 16),
        ("view_pos", C.c_float * 4),
        ("view_ray_top_left", C.c_float * 4),
        ("view_ray_right_shift", C.c_float * 4),
        ("view_ray_down_shift", C.c_float * 4),
        ("prev_view_proj", C.c_float * 16),
        ("prev_inv_view_proj", C.c_float * 16),
        ("prev_view_pos", C.c_float * 4),
        ("jitter", C.c_float * 4),
        ("sun_dir", C.c_float * 4),
        ("sun_inten", C.c_float * 4),
    ]


class Params(C.Structure):
    _fields_ = [
        ("diff_m_cap", C.c_uint32),
        ("spec_m_cap", C.c_uint32),
        ("use_input_pdf", C.c_uint32),
        ("diff_spatial_passes", C.c_uint32),
        ("diff_spatial_taps", C.c_uint32),
        ("diff_spatial_radius_px", C.c_float),
        ("spec_spatial_passes", C.c_uint32),
        ("spec_spatial_taps", C.c_uint32),
        ("spec_spatial_radius_px", C.c_float),
        ("ao_radius", C.c_float),
        ("denoise", C.c_uint32),
        ("disocclusion_fix", C.c_uint32),
        ("fast_history_clamp", C.c_uint32),
        ("atrous_iterations", C.c_uint32),
        ("history_max_frames", C.c_float),
        ("hg_enable", C.c_uint32),
        ("hg_decay", C.c_uint32),
        ("hg_log2_buckets", C.c_uint32),
        ("hg_key_mode", C.c_uint32),
        ("hg_max_queries", C.c_uint32),
        ("post", C.c_uint32),
        ("trace", C.c_uint32),
        ("diff_validate", C.c_uint32),
        ("spec_validate", C.c_uint32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class FrameInputs(C.Structure):
    _fields_ = [
        ("params", C.POINTER(FrameParams)),
        ("frame_index", C.c_uint32),
        ("depth", C.c_void_p),
        ("gbuffer", C.c_void_p),
        ("prev_depth", C.c_void_p),
        ("prev_gbuffer", C.c_void_p),
        ("diff_hit_pos_normal", C.c_void_p),
        ("diff_hit_radiance", C.c_void_p),
        ("diff_source_pdf", C.c_void_p),
        ("spec_hit_pos", C.c_void_p),
        ("spec_hit_radiance", C.c_void_p),
        ("shadow_mask", C.c_void_p),
        ("cache_hits", C.c_void_p),
        ("diffuse_hits", C.c_void_p),
        ("spec_validate_hits", C.c_void_p),
    ]


class FrameRays(C.Structure):
    _fields_ = [
        ("cache", C.c_void_p),
        ("diffuse", C.c_void_p),
        ("spec_validate", C.c_void_p),
        ("n_cache", C.c_uint32),
        ("n_diffuse", C.c_uint32),
        ("n_spec_validate", C.c_uint32),
        ("diffuse_kind", C.c_uint32),
    ]


RAY_BYTES = 32  # vlt_ray
HIT_BYTES = 64  # vlt_ray_hit


class FrameOutputs(C.Structure):
    _fields_ = [
        ("diffuse", C.c_void_p),
        ("specular", C.c_void_p),
        ("raw_diffuse", C.c_void_p),
        ("raw_specular", C.c_void_p),
        ("color", C.c_void_p),
        ("taa", C.c_void_p),
    ]


class PassTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("total_ms", C.c_double)]


TILE_CANDIDATES = 10  # VLT_TILE_CANDIDATES


class TileChoice(C.Structure):
    _fields_ = [("pass_", C.c_char * 32), ("bx", C.c_uint16), ("by", C.c_uint16), ("persistent", C.c_uint16),
                ("ns_per_kpix", C.c_float * TILE_CANDIDATES)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("step_pixel_budget", C.c_uint64), ("max_sessions", C.c_uint32)]


class ServerCompletion(C.Structure):
    _fields_ = [("session", C.c_uint64), ("tag", C.c_uint64), ("latency_ms", C.c_double), ("step_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("sessions_opened", C.c_uint64), ("sessions_admitted", C.c_uint64), ("sessions_closed", C.c_uint64),
                ("steps", C.c_uint64), ("frames_issued", C.c_uint64), ("frames_done", C.c_uint64),
                ("pixels_issued", C.c_uint64), ("admit_wait_ms_total", C.c_double), ("sessions_live", C.c_uint32),
                ("sessions_waiting", C.c_uint32), ("steps_in_flight", C.c_uint32), ("bytes_in_use", C.c_uint64),
                ("pixels_in_use", C.c_uint64), ("admit_failures", C.c_uint64), ("last_admit_status", C.c_uint32),
                ("pad0", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("launches", C.c_uint64), ("graph_replays", C.c_uint64),
                ("graph_captures", C.c_uint64), ("arena_bytes", C.c_uint64), ("last_launches", C.c_uint32),
                ("last_jobs", C.c_uint32), ("last_chunks", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("disocclusion_frac", C.c_float),
        ("camera_speed", C.c_float),
        ("jitter_cycle", C.c_uint32),
    ]


class SceneFrame(C.Structure):
    _fields_ = [
        ("depth", C.c_void_p),
        ("gbuffer", C.c_void_p),
        ("diff_hit_pos_normal", C.c_void_p),
        ("diff_hit_radiance", C.c_void_p),
        ("diff_source_pdf", C.c_void_p),
        ("spec_hit_pos", C.c_void_p),
        ("spec_hit_radiance", C.c_void_p),
        ("shadow_mask", C.c_void_p),
    ]


P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int32
F32 = C.c_float
FP = C.POINTER(FrameParams)
PP = C.POINTER(Params)

# name -> (restype, argtypes). Every function declared in include/vlt.h and
# include/vlt_scene.h.
SIGNATURES = {
    "vlt_params_reference": (None, [PP]),
    "vlt_params_plain": (None, [PP, C.c_int]),
    "vlt_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "vlt_ctx_destroy": (C.c_int, [P]),
    "vlt_status_string": (C.c_char_p, [C.c_int]),
    "vlt_last_error": (C.c_char_p, []),
    "vlt_view_create": (C.c_int, [P, U32, U32, C.c_int, PP, C.POINTER(P)]),
    "vlt_view_destroy": (C.c_int, [P]),
    "vlt_view_device_bytes": (C.c_size_t, [U32, U32, C.c_int, PP]),
    "vlt_view_reset": (C.c_int, [P, P]),
    "vlt_frame_run": (C.c_int, [P, C.POINTER(FrameInputs), C.POINTER(FrameOutputs), P]),
    "vlt_frames_run": (C.c_int, [P, C.c_uint32, C.POINTER(FrameInputs), C.POINTER(FrameOutputs), P]),
    "vlt_frame_trace": (C.c_int, [P, C.POINTER(FrameInputs), C.POINTER(FrameRays), P]),
    "vlt_view_state_bytes": (C.c_size_t, [P]),
    "vlt_view_export_state": (C.c_int, [P, P, C.c_size_t, P]),
    "vlt_view_import_state": (C.c_int, [P, P, C.c_size_t, P]),
    "vlt_view_cache_ray_capacity": (U32, [P]),
    "vlt_view_last_launch_count": (U32, [P]),
    "vlt_batch_create": (C.c_int, [P, C.POINTER(P)]),
    "vlt_batch_destroy": (C.c_int, [P]),
    "vlt_batch_run": (C.c_int, [P, C.POINTER(P), C.POINTER(FrameInputs), C.POINTER(FrameOutputs), U32, P]),
    "vlt_batch_set_graphs": (C.c_int, [P, C.c_int]),
    "vlt_batch_set_chunk_pixels": (C.c_int, [P, C.c_uint64]),
    "vlt_batch_set_persistent": (C.c_int, [P, C.c_int]),
    "vlt_batch_autotune": (C.c_int, [P]),
    "vlt_batch_tile_table": (U32, [P, C.POINTER(TileChoice), U32]),
    "vlt_batch_get_stats": (C.c_int, [P, C.POINTER(BatchStats)]),
    "vlt_server_create": (C.c_int, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
    "vlt_server_destroy": (C.c_int, [P]),
    "vlt_server_batch": (P, [P]),
    "vlt_server_open": (C.c_int, [P, U32, U32, C.c_int, C.POINTER(Params), C.POINTER(C.c_uint64)]),
    "vlt_server_submit": (C.c_int, [P, C.c_uint64, C.POINTER(FrameInputs), C.POINTER(FrameOutputs), C.c_uint64]),
    "vlt_server_close": (C.c_int, [P, C.c_uint64]),
    "vlt_server_step": (C.c_int, [P, P, C.POINTER(U32)]),
    "vlt_server_poll": (U32, [P, C.POINTER(ServerCompletion), U32, C.c_int]),
    "vlt_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "vlt_view_buffer": (P, [P, C.c_char_p, C.POINTER(C.c_size_t)]),
    "vlt_view_set_timing": (C.c_int, [P, C.c_int]),
    "vlt_view_read_timing": (U32, [P, C.POINTER(PassTime), U32]),
    "vlt_ind_diff_temporal_resample": (C.c_int, [FP, U32, U32, PP, P, P, P, P, P, P, P, U32, U32, U32, P]),
    "vlt_ao_gen": (C.c_int, [FP, U32, U32, P, P, P, P, U32, U32, F32, P]),
    "vlt_ao_filter": (C.c_int, [U32, U32, P, P, P, P]),
    "vlt_ind_diff_spatial_resample": (C.c_int, [FP, U32, U32, PP, P, P, P, P, P, P, U32, P]),
    "vlt_ind_spec_temporal_resample": (C.c_int, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, P, P, U32, U32, P]),
    "vlt_ind_spec_spatial_resample": (C.c_int, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, U32, P]),
    "vlt_denoise_temporal": (C.c_int, [FP, U32, U32, PP, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, U32, U32, P]),
    "vlt_denoise_disocclusion_fix": (C.c_int, [U32, U32, P, P, P, P, P, P, P, P]),
    "vlt_denoise_fast_history_clamp": (C.c_int, [U32, U32, P, P, P]),
    "vlt_denoise_spatial_fallback": (C.c_int, [U32, U32, P, P, P, P, P, P, P, P]),
    "vlt_denoise_atrous": (C.c_int, [U32, U32, P, P, P, P, P, P, I32, P]),
    "vlt_final_lighting": (C.c_int, [FP, U32, U32, P, P, P, P, P, P]),
    "vlt_hg_visualize": (C.c_int, [FP, U32, U32, U32, U32, P, P, P, U32, P, P]),
    "vlt_temporal_aa": (C.c_int, [FP, U32, U32, P, P, P, U32, P, P]),
    "vlt_hg_decay": (C.c_int, [U32, P, P, P]),
    "vlt_hg_select_scratch_bytes": (C.c_size_t, [U32, U32]),
    "vlt_hg_query_select": (C.c_int, [U32, U32, P, P, P, P, U32, P, P]),
    "vlt_hg_query_select_noalloc": (C.c_int, [U32, U32, P, P, P, P, U32, P]),
    "vlt_hg_query_compact": (C.c_int, [U32, U32, P, P, P, P, P]),
    "vlt_hg_update": (C.c_int, [U32, P, P, P, P, P, P, P]),
    "vlt_hg_emit_queries": (C.c_int, [FP, U32, U32, U32, U32, U32, P, P, P, P, P, P]),
    "vlt_hg_find": (C.c_int, [FP, U32, U32, P, U32, P, P, P, P, P]),
    "vlt_image_stats": (C.c_int, [P, C.c_int, P, C.c_int, U32, P, P]),
    "vlt_diag_math": (C.c_int, [C.c_int, P, P, U32, P]),
    "vlt_scene_desc_default": (None, [C.POINTER(SceneDesc), C.c_uint64, U32, U32]),
    "vlt_scene_frame_params": (C.c_int, [C.POINTER(SceneDesc), U32, FP]),
    "vlt_scene_generate_host": (C.c_int, [C.POINTER(SceneDesc), U32, C.POINTER(SceneFrame)]),
    "vlt_scene_generate_device": (C.c_int, [C.POINTER(SceneDesc), U32, C.POINTER(SceneFrame), P]),
    "vlt_scene_trace_host": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(FrameParams), P, U32, P]),
    "vlt_scene_trace_device": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(FrameParams), P, U32, P, P]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libvlt.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "violet_gb300: %s is missing; build it with `python -c \"import __graft_entry__ as g; g.build()\"`" % path
        )
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class VltError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.vlt_last_error().decode(errors="replace")
        super().__init__("%s: %s (%s)" % (where, STATUS_NAMES.get(status, status), msg))
        self.status = status


def check(status, where):
    if status != VLT_OK:
        raise VltError(status, where)
