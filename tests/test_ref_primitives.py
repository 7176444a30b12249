"""The oracle's shared primitives against the reference's own shader text.

oracle/_ref/libvlt_ref.so is the reference's rand.hlsl, enc.inc.hlsl, gbuffer.hlsl,
restir/reservoir.hlsl and restir/hash_grid.inc.hlsl compiled as C++
(oracle/ref_build.py). Every primitive of the oracle restatement (and through the
GPU parity tests, of the kernels) must give the same bits on the same inputs:
jenkins_hash, the LCG seed and draws, XXHash32, the octahedral codecs, the
ReservoirSimple packing (with its quirk), HitPosNormal, the hash-grid vertex key and
the G-buffer decode. Needs the reference tree (skipped without it; the fixtures in
tests/golden/ref_primitives.npz, made from the same library, are checked by
test_oracle_golden.py everywhere).
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import pyref

REF = pyref.lib()
pytestmark = pytest.mark.skipif(REF is None, reason="reference tree not available")

rng = np.random.default_rng(20261204)


def bits_equal(a, b):
    a = np.ascontiguousarray(a).view(np.uint32)
    b = np.ascontiguousarray(b).view(np.uint32)
    na = (a & 0x7FFFFFFF) > 0x7F800000
    nb = (b & 0x7FFFFFFF) > 0x7F800000
    bad = (a != b) & ~(na & nb)
    return int(np.count_nonzero(bad))


def test_jenkins_hash():
    x = rng.integers(0, 2 ** 32, 100000, dtype=np.uint64).astype(np.uint32)
    got = np.zeros_like(x)
    REF.vltr_jenkins_hash(pyref.ptr(x), pyref.ptr(got), x.size)
    assert np.array_equal(got, po.codec("jenkins", x))


def test_lcg_seed_and_draws():
    for _ in range(200):
        px, py = (int(v) for v in rng.integers(0, 2 ** 16, 2))
        seed = int(rng.integers(0, 2 ** 32))
        a = (np.zeros(16, np.float32), np.zeros(16, np.uint32))
        b = (np.zeros(16, np.float32), np.zeros(16, np.uint32))
        REF.vltr_lcg_sequence(px, py, seed, 16, pyref.ptr(a[0]), pyref.ptr(a[1]))
        po.lib().vlto_lcg_sequence(px, py, seed, 16, po.ptr(b[0]), po.ptr(b[1]))
        assert np.array_equal(a[1], b[1]) and bits_equal(a[0], b[0]) == 0


def test_xxhash32_chains():
    for n in range(1, 7):
        for _ in range(300):
            w = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
            assert REF.vltr_xxhash32(pyref.ptr(w), n) == po.lib().vlto_xxhash32(po.ptr(w), n)


def _normals(n):
    v = rng.standard_normal((n, 3)).astype(np.float32)
    v[: 6 * 4] = 0.0
    for k in range(6):  # axis directions, both signs, and tiny components
        v[4 * k, k // 2] = 1.0 if k % 2 == 0 else -1.0
        v[4 * k + 1, k // 2] = 1e-30 if k % 2 == 0 else -1e-30
        v[4 * k + 2] = [0.5, -0.5, 0.70710677 * (1 if k % 2 else -1)]
        v[4 * k + 3] = [-3.0, 2.0, 1e-7]
    return np.ascontiguousarray(v.reshape(-1))


def test_octahedral_encode():
    n3 = _normals(50000)
    n = n3.size // 3
    a16, a32 = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    b16, b32, dec = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(3 * n, np.float32)
    REF.vltr_oct_encode(pyref.ptr(n3), pyref.ptr(a16), pyref.ptr(a32), n)
    po.lib().vlto_oct(po.ptr(n3), po.ptr(b16), po.ptr(b32), po.ptr(dec), n)
    assert np.array_equal(a16, b16)
    assert np.array_equal(a32, b32)


def test_octahedral_decode_every_u16_code():
    u16 = np.arange(65536, dtype=np.uint32)
    u32 = rng.integers(0, 2 ** 32, 65536, dtype=np.uint64).astype(np.uint32)
    u32[:4] = [0, 0xFFFFFFFF, 0x7FFF7FFF, 0x80008000]
    a = (np.zeros(3 * 65536, np.float32), np.zeros(3 * 65536, np.float32))
    b = (np.zeros(3 * 65536, np.float32), np.zeros(3 * 65536, np.float32))
    REF.vltr_oct_decode(pyref.ptr(u16), pyref.ptr(u32), pyref.ptr(a[0]), pyref.ptr(a[1]), 65536)
    po.lib().vlto_oct_decode(po.ptr(u16), po.ptr(u32), po.ptr(b[0]), po.ptr(b[1]), 65536)
    assert bits_equal(a[0], b[0]) == 0
    assert bits_equal(a[1], b[1]) == 0


def test_reservoir_simple_packing_quirk():
    n = 20000
    M = rng.integers(0, 400, n).astype(np.uint32)
    W = (rng.lognormal(0, 6, n) * rng.choice([1, -1], n)).astype(np.float32)
    W[:6] = [0.0, -0.0, np.inf, 3.4e38, 1e-40, np.nan]
    enc, dm, dw = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(n, np.float32)
    REF.vltr_reservoir_simple(pyref.ptr(M), pyref.ptr(W), pyref.ptr(enc), pyref.ptr(dm), pyref.ptr(dw), n)
    for i in range(0, n, 7):
        assert enc[i] == po.lib().vlto_reservoir_encode(int(M[i]), float(W[i])), i
        m2, w2 = po.C.c_uint32(), po.C.c_float()
        po.lib().vlto_reservoir_decode(int(enc[i]), po.C.byref(m2), po.C.byref(w2))
        assert m2.value == dm[i]
        assert np.float32(w2.value).view(np.uint32) == dw[i].view(np.uint32)


def test_hit_pos_normal():
    n = 20000
    pos = (rng.standard_normal((n, 3)) * rng.choice([0.01, 1.0, 100.0, 70000.0], (n, 1))).astype(np.float32).ravel()
    nrm = _normals(n)[: 3 * n]
    a = (np.zeros(2 * n, np.uint32), np.zeros(3 * n, np.float32), np.zeros(3 * n, np.float32))
    b = (np.zeros(2 * n, np.uint32), np.zeros(3 * n, np.float32), np.zeros(3 * n, np.float32))
    REF.vltr_hit_pos_normal(pyref.ptr(pos), pyref.ptr(nrm), *(pyref.ptr(x) for x in a), n)
    po.lib().vlto_hit_pos_normal(po.ptr(pos), po.ptr(nrm), *(po.ptr(x) for x in b), n)
    assert np.array_equal(a[0], b[0])
    assert bits_equal(a[1], b[1]) == 0 and bits_equal(a[2], b[2]) == 0


def test_hash_grid_vertex_key():
    n = 50000
    cam = np.array([1.5, 2.0, -3.0], np.float32)
    dist = rng.choice([0.3, 2.0, 20.0, 300.0], (n, 1))
    pos = (cam + rng.standard_normal((n, 3)) * dist).astype(np.float32).ravel()
    pos[:3] = cam  # zero distance: LOD 0
    a = np.zeros(5 * n, np.uint32)
    b = np.zeros(2 * n, np.uint32)
    REF.vltr_vertex_key(pyref.ptr(pos), pyref.ptr(cam), pyref.ptr(a), n)
    po.lib().vlto_vertex_key(po.ptr(pos), po.ptr(cam), po.ptr(b), n)
    a = a.reshape(n, 5)
    b = b.reshape(n, 2)
    assert np.array_equal(a[:, 0], b[:, 0]), "bucket hash"
    assert np.array_equal(a[:, 1], b[:, 1]), "checksum"


def test_gbuffer_decode():
    n = 50000
    enc = rng.integers(0, 2 ** 32, 4 * n, dtype=np.uint64).astype(np.uint32)
    a, b = np.zeros(11 * n, np.float32), np.zeros(11 * n, np.float32)
    REF.vltr_gbuffer_decode(pyref.ptr(enc), pyref.ptr(a), n)
    po.lib().vlto_gbuffer_decode(po.ptr(enc), po.ptr(b), n)
    assert bits_equal(a, b) == 0
