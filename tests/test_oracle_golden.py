"""CPU: the oracle's bit-level primitives against the golden vectors of
tests/golden/primitives.json (an independent restatement of the shader text)."""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "primitives.json")))


def _pairs(name):
    a = np.array(GOLDEN[name], dtype=np.uint64)
    return a[:, 0].astype(np.uint32), a[:, 1].astype(np.uint32)


@pytest.mark.parametrize("name,fn", [("jenkins_hash", "jenkins"), ("lcg_xorshift", "xorshift"),
                                     ("xxh32_one", "xxh1"), ("xxh32_three", "xxh3"),
                                     ("f32tof16", "f32tof16"), ("ufloat11", "uf11"), ("ufloat10", "uf10")])
def test_codec_vectors(name, fn):
    x, y = _pairs(name)
    got = po.codec(fn, x)
    bad = np.nonzero(got != y)[0]
    assert bad.size == 0, "%s: input 0x%08x -> 0x%08x, golden 0x%08x" % (name, x[bad[0]], got[bad[0]], y[bad[0]])


def test_lcg_uint_to_float():
    x, y = _pairs("lcg_uint_to_float_bits")
    # lcg_uint_to_float = asfloat(0x3f800000 | x >> 9) - 1, exercised through f16/f32 free path:
    got = (np.bitwise_or(np.uint32(0x3F800000), x >> np.uint32(9)).view(np.float32) - np.float32(1)).view(np.uint32)
    assert np.array_equal(got, y)


def test_frame_rand_chain():
    for fi, chain in GOLDEN["frame_rand_chain"]:
        s = np.array([fi], np.uint32)
        for expected in chain:
            s = po.codec("jenkins", s)
            assert int(s[0]) == expected


def test_reservoir_32b_quirk():
    lib = po.lib()
    import ctypes as C

    for M, Wbits, u, dm, dwbits in GOLDEN["reservoir_32b"]:
        W = np.array([Wbits], np.uint32).view(np.float32)[0]
        assert lib.vlto_reservoir_encode(M, float(W)) == u
        m, w = C.c_uint32(), C.c_float()
        lib.vlto_reservoir_decode(u, C.byref(m), C.byref(w))
        assert m.value == dm
        assert np.array([w.value], np.float32).view(np.uint32)[0] == dwbits
    # The quirk: M bits 6..7 leak into the decoded W (reservoir.hlsl:59-72).
    W = np.float32(1.0)
    a = lib.vlto_reservoir_encode(0, float(W))
    b = lib.vlto_reservoir_encode(192, float(W))
    ma, wa, mb, wb = C.c_uint32(), C.c_float(), C.c_uint32(), C.c_float()
    lib.vlto_reservoir_decode(a, C.byref(ma), C.byref(wa))
    lib.vlto_reservoir_decode(b, C.byref(mb), C.byref(wb))
    assert wa.value != wb.value and mb.value == 192


def test_octahedral_vectors():
    lib = po.lib()
    rows = GOLDEN["oct"]
    n = np.array([r[0] for r in rows], np.uint32).view(np.float32).reshape(-1)
    u16 = np.zeros(len(rows), np.uint32)
    u32 = np.zeros(len(rows), np.uint32)
    d16 = np.zeros(3 * len(rows), np.float32)
    lib.vlto_oct(po.ptr(n), po.ptr(u16), po.ptr(u32), po.ptr(d16), len(rows))
    assert np.array_equal(u16, np.array([r[1] for r in rows], np.uint32))
    assert np.array_equal(u32, np.array([r[2] for r in rows], np.uint32))
    assert np.array_equal(d16.view(np.uint32), np.array([r[3] for r in rows], np.uint32).reshape(-1))


@pytest.mark.parametrize("fn,ref,lo,hi,ulps", [
    ("exp2", np.exp2, -20, 20, 4), ("exp", np.exp, -20, 20, 20), ("log2", np.log2, 1e-6, 1e6, 4),
    ("sin", np.sin, -40, 40, 4), ("cos", np.cos, -40, 40, 4)])
def test_own_math_accuracy(fn, ref, lo, hi, ulps):
    rng = np.random.default_rng(0)
    x = rng.uniform(lo, hi, 100000).astype(np.float32)
    y = po.math(fn, x).astype(np.float64)
    r = ref(x.astype(np.float64))
    # error in units of the binary32 spacing at the true value (absolute near zero crossings)
    spacing = np.spacing(np.abs(r).astype(np.float32)).astype(np.float64)
    if fn in ("sin", "cos"):
        spacing = np.maximum(spacing, 2.0 ** -24)
    err = np.abs(y - r) / spacing
    assert np.max(err) <= ulps, "%s max error %.2f ulp" % (fn, np.max(err))


def test_own_math_special_values():
    assert po.math("exp2", np.array([0.0], np.float32))[0] == 1.0
    assert po.math("exp2", np.array([128.0], np.float32))[0] == np.inf
    assert po.math("exp2", np.array([-200.0], np.float32))[0] == 0.0
    assert po.math("log2", np.array([0.0], np.float32))[0] == -np.inf
    assert np.isnan(po.math("log2", np.array([-1.0], np.float32))[0])
    assert po.math("log2", np.array([8.0], np.float32))[0] == 3.0
    assert np.isnan(po.math("sin", np.array([np.inf], np.float32))[0])


# ---- known answers of the reference's own shader text (tests/golden/ref_primitives.npz,
# made by tests/golden/make_ref_golden.py from the HLSL compiled as C++)

REFP = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_primitives.npz"))


def _bits(a):
    a = np.ascontiguousarray(a).view(np.uint32)
    return np.where((a & 0x7FFFFFFF) > 0x7F800000, np.uint32(0x7FC00000), a)


def test_reference_shader_hashes_and_lcg():
    assert np.array_equal(po.codec("jenkins", REFP["jenkins_in"]), REFP["jenkins_out"])
    for (px, py, sd), rands, states in zip(REFP["lcg_seeds"], REFP["lcg_rands"], REFP["lcg_states"]):
        r, st = np.zeros(8, np.float32), np.zeros(8, np.uint32)
        po.lib().vlto_lcg_sequence(int(px), int(py), int(sd), 8, po.ptr(r), po.ptr(st))
        assert np.array_equal(st, states) and np.array_equal(_bits(r), _bits(rands))
    for w, outs in zip(REFP["xxh_words"], REFP["xxh_out"]):
        for k in range(1, 5):
            assert po.lib().vlto_xxhash32(po.ptr(np.ascontiguousarray(w[:k])), k) == outs[k - 1]


def test_reference_shader_codecs():
    n3 = np.ascontiguousarray(REFP["oct_in"].reshape(-1))
    n = n3.size // 3
    u16, u32, dec = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(3 * n, np.float32)
    po.lib().vlto_oct(po.ptr(n3), po.ptr(u16), po.ptr(u32), po.ptr(dec), n)
    assert np.array_equal(u16, REFP["oct_u16"]) and np.array_equal(u32, REFP["oct_u32"])
    c16, c32 = REFP["octd_u16"], REFP["octd_u32"]
    a, b = np.zeros(3 * c16.size, np.float32), np.zeros(3 * c16.size, np.float32)
    po.lib().vlto_oct_decode(po.ptr(c16), po.ptr(c32), po.ptr(a), po.ptr(b), c16.size)
    assert np.array_equal(_bits(a), _bits(REFP["octd_n16"])) and np.array_equal(_bits(b), _bits(REFP["octd_n32"]))
    for M, W, e, dM, dW in zip(REFP["rs_M"][::5], REFP["rs_W"][::5], REFP["rs_enc"][::5], REFP["rs_dM"][::5],
                               REFP["rs_dW"][::5]):
        assert po.lib().vlto_reservoir_encode(int(M), float(W)) == e
    pos, nrm = np.ascontiguousarray(REFP["hpn_pos"].reshape(-1)), np.ascontiguousarray(REFP["hpn_nrm"].reshape(-1))
    n = pos.size // 3
    enc, dp, dn = np.zeros(2 * n, np.uint32), np.zeros(3 * n, np.float32), np.zeros(3 * n, np.float32)
    po.lib().vlto_hit_pos_normal(po.ptr(pos), po.ptr(nrm), po.ptr(enc), po.ptr(dp), po.ptr(dn), n)
    assert np.array_equal(enc, REFP["hpn_enc"])
    assert np.array_equal(_bits(dp), _bits(REFP["hpn_dpos"])) and np.array_equal(_bits(dn), _bits(REFP["hpn_dnrm"]))


def test_reference_shader_vertex_key_and_gbuffer():
    pos = np.ascontiguousarray(REFP["vk_pos"].reshape(-1))
    n = pos.size // 3
    out = np.zeros(2 * n, np.uint32)
    po.lib().vlto_vertex_key(po.ptr(pos), po.ptr(REFP["vk_cam"]), po.ptr(out), n)
    ref = REFP["vk_out"].reshape(n, 5)
    assert np.array_equal(out.reshape(n, 2), ref[:, :2])
    enc = REFP["gb_enc"]
    g = np.zeros(11 * (enc.size // 4), np.float32)
    po.lib().vlto_gbuffer_decode(po.ptr(enc), po.ptr(g), enc.size // 4)
    assert np.array_equal(_bits(g), _bits(REFP["gb_out"]))
