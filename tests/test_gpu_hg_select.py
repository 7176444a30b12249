"""GPU parity of the hash-grid query selection (hash_grid_query_select.hlsl:22-56 with
hash_grid_find_or_insert, hash_grid.inc.hlsl:149-184) on synthetic query sets that
stress the bucket-level insertion: buckets already full, buckets that fill up during
the frame (the later queries of new checksums fail), many misses per bucket (more
than one warp's worth) and few, query counts above max_queries, and empty queries.

The oracle runs the sequential loop over query indices; the GPU must give the same
cell storage and selection words bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

V = C.c_void_p


def _synth(seed, log2_buckets, n_queries, fill, pool, empty_frac=0.02):
    """Storage with `fill(rng, nb)` cells already in each bucket (slots in order) and
    queries whose checksums come from a per-bucket pool of `pool` values (the first
    ones are the bucket's existing cells, so part of the queries hit)."""
    rng = np.random.default_rng(seed)
    nb = 1 << log2_buckets
    storage = np.zeros((nb * 16, 4), np.uint32)
    pools = rng.integers(1, 1 << 31, size=(nb, pool), dtype=np.uint64).astype(np.uint32) | 1
    filled = fill(rng, nb)
    for b in range(nb):
        k = int(filled[b])
        storage[b * 16: b * 16 + k, 0] = pools[b, :k]
        storage[b * 16: b * 16 + k, 1:] = rng.integers(0, 1 << 30, size=(k, 3), dtype=np.uint64).astype(np.uint32)
    q = np.zeros((n_queries, 8), np.uint32)
    bucket = rng.integers(0, nb, size=n_queries).astype(np.uint32)
    pick = rng.integers(0, pool, size=n_queries)
    q[:, 4] = bucket
    q[:, 5] = pools[bucket, pick]
    q[:, 0:3] = rng.integers(0, 1 << 30, size=(n_queries, 3), dtype=np.uint64).astype(np.uint32)
    q[rng.random(n_queries) < empty_frac, 5] = 0  # no key: skipped
    return storage, q


def _run(log2_buckets, storage, queries, count, max_q, frame_hash):
    import torch

    lib = vg.lib()
    nc = 16 << log2_buckets
    q_pad = np.zeros((max(max_q, queries.shape[0]), 8), np.uint32)
    q_pad[: queries.shape[0]] = queries
    cnt = np.array([count], np.uint32)
    st_o = storage.copy()
    sel_o = np.zeros(nc, np.uint32)
    po.lib().vlto_hg_query_select(log2_buckets, max_q, po.ptr(q_pad), po.ptr(cnt), po.ptr(st_o), po.ptr(sel_o),
                                  frame_hash)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()

    q_g, c_g, st_g = dev(q_pad), dev(cnt), dev(storage)
    sel_g = torch.zeros(nc * 4, dtype=torch.uint8, device="cuda")
    scratch = torch.zeros(lib.vlt_hg_select_scratch_bytes(log2_buckets, max_q), dtype=torch.uint8, device="cuda")
    assert lib.vlt_hg_query_select(log2_buckets, max_q, V(q_g.data_ptr()), V(c_g.data_ptr()), V(st_g.data_ptr()),
                                   V(sel_g.data_ptr()), frame_hash, V(scratch.data_ptr()), None) == 0
    torch.cuda.synchronize()
    st = st_g.cpu().numpy().view(np.uint32).reshape(-1, 4)
    sel = sel_g.cpu().numpy().view(np.uint32)
    return st, sel, st_o, sel_o


def _check(st, sel, st_o, sel_o, what):
    bad = np.nonzero((st != st_o).any(axis=1))[0]
    assert bad.size == 0, "%s: %d cells differ, first %d: gpu %s oracle %s" % (what, bad.size, bad[0], st[bad[0]],
                                                                             st_o[bad[0]])
    bad = np.nonzero(sel != sel_o)[0]
    assert bad.size == 0, "%s: %d selection words differ, first cell %d: 0x%08x vs 0x%08x" % (
        what, bad.size, bad[0], sel[bad[0]], sel_o[bad[0]])


SEEDS = {"crowded": 11, "sparse": 12, "mixed": 13}
CASES = {
    # few buckets, hundreds of misses each: rounds over the segment in memory; every
    # bucket fills up and later checksums fail
    "crowded": (4, 6000, lambda rng, nb: rng.integers(0, 6, size=nb), 40),
    # many buckets, a few misses each: the register path
    "sparse": (12, 20000, lambda rng, nb: rng.integers(0, 16, size=nb), 20),
    # a mix: some buckets full from the start, some empty
    "mixed": (8, 12000, lambda rng, nb: np.where(rng.random(nb) < 0.3, 16, rng.integers(0, 4, size=nb)), 28),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_select_matches_sequential_loop(case):
    lb, nq, fill, pool = CASES[case]
    storage, queries = _synth(SEEDS[case], lb, nq, fill, pool)
    st, sel, st_o, sel_o = _run(lb, storage, queries, nq, nq, 0x5EED5)
    assert np.count_nonzero(sel_o) > 0 and np.count_nonzero(st_o[:, 0]) > np.count_nonzero(storage[:, 0])
    _check(st, sel, st_o, sel_o, case)


def test_select_count_above_max_queries_and_empty():
    lb = 6
    storage, queries = _synth(7, lb, 5000, lambda rng, nb: rng.integers(0, 8, size=nb), 24)
    # the counter kept counting past the cap: only the first max_queries are read
    st, sel, st_o, sel_o = _run(lb, storage, queries, 5000, 3000, 0xABCDEF)
    _check(st, sel, st_o, sel_o, "capped")
    # no queries at all
    st, sel, st_o, sel_o = _run(lb, storage, queries, 0, 3000, 0xABCDEF)
    _check(st, sel, st_o, sel_o, "empty")
    assert not sel.any() and np.array_equal(st, storage)
