"""CPU: the C-ABI library loads and exports every function include/*.h declares."""
import ctypes as C
import os
import re

import violet_gb300 as vg
from violet_gb300 import _ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("vlt.h", "vlt_scene.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(vlt_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = vg.lib()
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, "not exported: %s" % missing
    # and the ctypes table covers exactly the declared functions
    assert set(_ffi.SIGNATURES) == names


def test_presets_and_sizes_without_gpu():
    p = vg.params_reference()
    assert (p.diff_m_cap, p.diff_spatial_taps, p.spec_spatial_taps, p.atrous_iterations) == (16, 9, 4, 3)
    assert p.hg_log2_buckets == 16 and p.hg_max_queries == 131072
    q = vg.params_plain(1)
    assert (q.diff_spatial_passes, q.diff_spatial_taps, q.hg_log2_buckets, q.hg_key_mode) == (2, 8, 18, 1)
    n = vg.View.device_bytes(1920, 1080, "ref", q)
    assert 300e6 < n < 2e9
    lib = vg.lib()
    assert lib.vlt_status_string(1) == b"invalid argument"
    assert lib.vlt_hg_select_scratch_bytes(18, 2073600) > 2073600 * 4


def test_invalid_arguments_are_reported_not_raised():
    lib = vg.lib()
    h = C.c_void_p()
    # no context / null outputs -> VLT_ERR_INVALID_ARG without touching a GPU
    assert lib.vlt_view_create(None, 16, 16, 0, C.byref(vg.params_reference()), C.byref(h)) == 1
    assert lib.vlt_ctx_create(0, None) == 1
    assert lib.vlt_frame_run(None, None, None, None) == 1
    assert lib.vlt_frames_run(None, 0, None, None, None) == 1
    assert b"vlt_frames_run" in lib.vlt_last_error()
    assert lib.vlt_hg_decay(2, None, None, None) == 1
    assert lib.vlt_denoise_atrous(0, 0, None, None, None, None, None, None, 1, None) == 1


def test_noalloc_select_rejects_sizes_beyond_its_scratch():
    # The allocation-free query selection keeps its scratch in a fixed 12 MiB array;
    # larger sizes are refused before anything touches a GPU.
    lib = vg.lib()
    limit = 12 * 1024 * 1024
    assert lib.vlt_hg_select_scratch_bytes(16, 131072) <= limit
    assert lib.vlt_hg_select_scratch_bytes(18, 1920 * 1080) <= limit
    assert lib.vlt_hg_select_scratch_bytes(24, 1 << 24) > limit
    dummy = C.c_void_p(16)
    rc = lib.vlt_hg_query_select_noalloc(24, 1 << 24, dummy, dummy, dummy, dummy, 0, None)
    assert rc == 1
    assert b"scratch" in lib.vlt_last_error()
