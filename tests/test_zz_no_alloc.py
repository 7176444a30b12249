"""GPU: the query selection that allocates nothing.

vlt_hg_query_select_noalloc serves callers that may not allocate device memory (a
host with its own fixed device-memory budget or pool allocator, or a real-time
frame loop that cannot afford cudaMalloc's implicit synchronization). It keeps its
scratch in a fixed array inside the library instead of taking caller scratch. This
test drives it through the C ABI and checks that, on two calls in a row (the second
one starting from whatever the first left in the shared array), it produces
exactly the cell storage and selection words of vlt_hg_query_select with caller
scratch. Selection is integer work, so the comparison is exact.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import upload

pytestmark = pytest.mark.gpu

LOG2_BUCKETS = 16
MAX_QUERIES = 131072


def _emit(scene, frame, queries, count, W, H):
    lib = vg.lib()
    host = scene.generate_host(frame)
    dev = upload(host)
    fp = scene.frame_params(frame)
    rc = lib.vlt_hg_emit_queries(C.byref(fp), W, H, LOG2_BUCKETS, 0, MAX_QUERIES, C.c_void_p(dev["depth"].data_ptr()),
                                 C.c_void_p(dev["diff_hit_pos_normal"].data_ptr()),
                                 C.c_void_p(dev["diff_hit_radiance"].data_ptr()), C.c_void_p(queries.data_ptr()),
                                 C.c_void_p(count.data_ptr()), None)
    assert rc == 0
    return dev


def test_noalloc_select_matches_caller_scratch_two_calls():
    import torch

    lib = vg.lib()
    W, H = 320, 180
    scene = vg.Scene(21, W, H)
    ncells = 16 << LOG2_BUCKETS
    queries = torch.zeros(MAX_QUERIES * 32, dtype=torch.uint8, device="cuda")
    count = torch.zeros(4, dtype=torch.uint8, device="cuda")
    storage_a = torch.zeros(ncells * 16, dtype=torch.uint8, device="cuda")
    storage_b = torch.zeros_like(storage_a)
    scratch = torch.zeros(lib.vlt_hg_select_scratch_bytes(LOG2_BUCKETS, MAX_QUERIES), dtype=torch.uint8,
                          device="cuda")
    for call, (frame, seed) in enumerate([(0, 0x1234567), (1, 0x89ABCDE)]):
        _emit(scene, frame, queries, count, W, H)
        sel_a = torch.zeros(ncells * 4, dtype=torch.uint8, device="cuda")
        sel_b = torch.zeros_like(sel_a)
        rc = lib.vlt_hg_query_select(LOG2_BUCKETS, MAX_QUERIES, C.c_void_p(queries.data_ptr()),
                                     C.c_void_p(count.data_ptr()), C.c_void_p(storage_a.data_ptr()),
                                     C.c_void_p(sel_a.data_ptr()), seed, C.c_void_p(scratch.data_ptr()), None)
        assert rc == 0
        rc = lib.vlt_hg_query_select_noalloc(LOG2_BUCKETS, MAX_QUERIES, C.c_void_p(queries.data_ptr()),
                                             C.c_void_p(count.data_ptr()), C.c_void_p(storage_b.data_ptr()),
                                             C.c_void_p(sel_b.data_ptr()), seed, None)
        assert rc == 0, lib.vlt_last_error()
        torch.cuda.synchronize()
        a_st, b_st = storage_a.cpu().numpy().view(np.uint32), storage_b.cpu().numpy().view(np.uint32)
        a_sel, b_sel = sel_a.cpu().numpy().view(np.uint32), sel_b.cpu().numpy().view(np.uint32)
        assert np.count_nonzero(a_sel) > 1000, "call %d selected too few cells to be a meaningful check" % call
        assert np.array_equal(a_st, b_st), "call %d: cell storage differs" % call
        assert np.array_equal(a_sel, b_sel), "call %d: selection words differ" % call

