"""Writes tests/golden/ref_passes.npz and ref_primitives.npz: inputs and outputs of the reference's own
shaders (oracle/_ref/libvlt_ref.so, the HLSL compiled as C++ by oracle/ref_build.py)
for every per-pass entry point, on the state of a reference-preset view of the
synthetic scene (37x23 pixels, odd-sized groups at the edges, after 4 frames).

The fixtures let machines without the reference tree (the GPU machines) check the
product's per-pass kernels and the oracle against the reference's text directly:
tests/test_gpu_ref_golden.py and tests/test_oracle_golden.py.

Run from the repository root: python tests/golden/make_ref_golden.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from oracle import pyref  # noqa: E402
from tests import test_ref_passes as T  # noqa: E402

OUT = os.path.join(HERE, "ref_passes.npz")


class Case:
    def __init__(self, name):
        self.name = name
        self.args = []

    def fp(self, fp):
        self.args.append(("fp", np.frombuffer(bytes(fp), np.uint8).copy()))
        return self

    def params(self, p):
        self.args.append(("params", np.frombuffer(bytes(p), np.uint8).copy()))
        return self

    def inp(self, a):
        self.args.append(("in", np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()))
        return self

    def out(self, nbytes):
        self.args.append(("out", np.zeros(nbytes, np.uint8)))
        return self

    def inout(self, a):
        self.args.append(("inout", np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()))
        return self

    def u32(self, v):
        self.args.append(("u32", int(v)))
        return self

    def i32(self, v):
        self.args.append(("i32", int(v)))
        return self

    def f32(self, v):
        self.args.append(("f32", float(v)))
        return self

    def none(self):
        self.args.append(("none", None))
        return self

    def run(self):
        """Runs the reference shader; returns the output arrays (out and inout)."""
        f = getattr(pyref.lib(), "vltr_" + self.name)
        f.restype = None
        call, outs, keep = [], [], []
        for kind, v in self.args:
            if kind == "fp":
                s = po._ffi.FrameParams.from_buffer_copy(v.tobytes())
                keep.append(s)
                call.append(C.byref(s))
            elif kind == "params":
                s = po._ffi.Params.from_buffer_copy(v.tobytes())
                keep.append(s)
                call.append(C.byref(s))
            elif kind in ("in",):
                call.append(C.c_void_p(v.ctypes.data))
            elif kind in ("out", "inout"):
                a = v.copy()
                outs.append(a)
                call.append(C.c_void_p(a.ctypes.data))
            elif kind == "u32":
                call.append(C.c_uint32(v))
            elif kind == "i32":
                call.append(C.c_int32(v))
            elif kind == "f32":
                call.append(C.c_float(v))
            else:
                call.append(None)
        f(*call)
        return outs


def cases():
    s = T.State(W=37, H=23, warm=4, seed=5)
    W, H, n = s.W, s.H, s.n
    P = s.params
    out = []

    def add(c):
        out.append(c)
        return c

    for hp, hn in ((1, 1), (1, 0), (0, 1)):
        add(Case("ind_diff_temporal_resample").fp(s.fp).u32(W).u32(H).params(P).inp(s.buf("prev_depth"))
            .inp(s.inp["depth"]).inp(s.inp["diff_hit_pos_normal"]).inp(s.inp["diff_hit_radiance"]).none()
            .inp(s.buf("diff_reservoir")).out(16 * n).u32(1000 + hp * 2 + hn).u32(hp).u32(hn))
    add(Case("ind_diff_spatial_resample").fp(s.fp).u32(W).u32(H).params(P).inp(s.inp["gbuffer"])
        .inp(s.inp["depth"]).inp(s.buf("ao_filtered")).inp(T._diff_temporal_out(s)).out(16 * n).out(4 * n)
        .u32(4242))
    for hn, hp in ((1, 1), (0, 1), (1, 0)):
        add(Case("ao_gen").fp(s.fp).u32(W).u32(H).inp(s.inp["diff_hit_pos_normal"]).inp(s.inp["depth"])
            .inp(s.buf("ao_history")).out(4 * n).u32(hn).u32(hp).f32(P.ao_radius))
    add(Case("ao_filter").u32(W).u32(H).inp(s.inp["depth"]).inp(s.buf("ao_history")).out(2 * n))
    for hp in (1, 0):
        add(Case("ind_spec_temporal_resample").fp(s.fp).u32(W).u32(H).params(P).inp(s.buf("prev_depth"))
            .inp(s.buf("prev_gbuffer")).inp(s.inp["depth"]).inp(s.inp["gbuffer"]).inp(s.buf("spec_reservoir"))
            .inp(s.buf("spec_hit_pos")).inp(s.buf("spec_radiance")).inp(s.inp["spec_hit_pos"])
            .inp(s.inp["spec_hit_radiance"]).out(8 * n).out(16 * n).out(4 * n).u32(777 + hp).u32(hp))
    rsv, hp_, rad = T._spec_temporal_out(s)
    add(Case("ind_spec_spatial_resample").fp(s.fp).u32(W).u32(H).params(P).inp(s.inp["gbuffer"])
        .inp(s.inp["depth"]).inp(rsv).inp(hp_).inp(rad).out(4 * n).out(2 * n).none().none().none().u32(2024))
    dl, sl, rl = T._lighting(s)
    fast = np.ascontiguousarray(s.buf("hist_color")[::-1])
    for fast_on, hist in ((0, 1), (1, 1), (0, 0)):
        add(Case("denoise_temporal").fp(s.fp).u32(W).u32(H).params(P).inp(s.inp["depth"]).inp(s.inp["gbuffer"])
            .inp(dl).inp(sl).inp(rl).inp(s.buf("prev_depth")).inp(s.buf("prev_gbuffer")).inp(s.buf("hist_color"))
            .inp(s.buf("hist_moments")).inp(s.buf("hist_len")).inp(fast).out(8 * n).out(4 * n).out(n).out(8 * n)
            .u32(hist).u32(fast_on))
    color, mom, ln, _ = T._temporal_outputs(s)
    add(Case("denoise_disocclusion_fix").u32(W).u32(H).inp(s.inp["depth"]).inp(s.inp["gbuffer"]).inp(ln)
        .inp(color).inp(mom).out(8 * n).out(4 * n))
    add(Case("denoise_fast_history_clamp").u32(W).u32(H).inp(s.buf("hist_color")).inout(color))
    add(Case("denoise_spatial_fallback").u32(W).u32(H).inp(s.inp["depth"]).inp(s.inp["gbuffer"]).inp(ln)
        .inp(color).inp(mom).out(8 * n).out(4 * n))
    c2, var = np.zeros(8 * n, np.uint8), np.zeros(4 * n, np.uint8)
    po.lib().vlto_denoise_spatial_fallback(W, H, po.ptr(s.inp["depth"]), po.ptr(s.inp["gbuffer"]), po.ptr(ln),
                                           po.ptr(color), po.ptr(mom), po.ptr(c2), po.ptr(var))
    for step in (1, 2, 4):
        add(Case("denoise_atrous").u32(W).u32(H).inp(s.inp["depth"]).inp(s.inp["gbuffer"]).inp(c2).inp(var)
            .out(8 * n).out(4 * n).i32(step))
    add(Case("hg_decay").u32(16).inout(s.buf("hg_decay")).inout(s.buf("hg_storage")))
    decay, storage = s.buf("hg_decay").copy(), s.buf("hg_storage").copy()
    po.lib().vlto_hg_decay(16, po.ptr(decay), po.ptr(storage))
    max_q = P.hg_max_queries
    q = s.buf("hg_queries").view(np.uint32).reshape(-1, 8)[: int(s.buf("hg_query_count").view(np.uint32)[0])]
    q = q[q[:, 5] != 0]
    queries = np.zeros(32 * max_q, np.uint8)
    queries[: q.nbytes] = q.reshape(-1).view(np.uint8)
    add(Case("hg_query_select").u32(16).u32(max_q).inp(queries).inp(np.array([q.shape[0]], np.uint32))
        .inout(storage).out(4 * (16 << 16)).u32(0x9E3779B9))
    rng = np.random.default_rng(11)
    shadow = rng.integers(0, 256, n).astype(np.uint8)
    hc = s.buf("hist_color")
    add(Case("final_lighting").i32(0).fp(s.fp).u32(W).u32(H).inp(s.inp["gbuffer"]).inp(shadow)
        .inp(np.ascontiguousarray(hc.view(np.uint32)[0::2])).inp(np.ascontiguousarray(hc.view(np.uint32)[1::2]))
        .i32(1).out(4 * n))
    for hh in (1, 0):
        add(Case("temporal_aa").i32(0).fp(s.fp).u32(W).u32(H).inp(s.inp["depth"])
            .inp(np.ascontiguousarray(hc.view(np.uint32)[0::2])).inp(np.ascontiguousarray(hc.view(np.uint32)[1::2]))
            .u32(hh).out(4 * n))
    return s, out


PRIM_OUT = os.path.join(HERE, "ref_primitives.npz")


def primitives():
    """Known answers of the reference's shared shader functions (rand.hlsl,
    enc.inc.hlsl, gbuffer.hlsl, restir/reservoir.hlsl, restir/hash_grid.inc.hlsl)."""
    R = pyref.lib()
    rng = np.random.default_rng(7)
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    z = {}
    x = rng.integers(0, 2 ** 32, 4096, dtype=np.uint64).astype(np.uint32)
    z["jenkins_in"], z["jenkins_out"] = x, np.zeros_like(x)
    R.vltr_jenkins_hash(P(x), P(z["jenkins_out"]), x.size)
    seeds = rng.integers(0, 2 ** 16, (64, 3)).astype(np.uint32)
    seeds[:, 2] = rng.integers(0, 2 ** 32, 64, dtype=np.uint64).astype(np.uint32)
    z["lcg_seeds"], z["lcg_rands"], z["lcg_states"] = seeds, np.zeros((64, 8), np.float32), np.zeros((64, 8), np.uint32)
    for i, (px, py, sd) in enumerate(seeds):
        R.vltr_lcg_sequence(int(px), int(py), int(sd), 8, P(z["lcg_rands"][i]), P(z["lcg_states"][i]))
    words = rng.integers(0, 2 ** 32, (256, 4), dtype=np.uint64).astype(np.uint32)
    z["xxh_words"] = words
    z["xxh_out"] = np.array([[R.vltr_xxhash32(P(np.ascontiguousarray(w[:k])), k) for k in range(1, 5)]
                             for w in words], np.uint32)
    n3 = rng.standard_normal((4096, 3)).astype(np.float32)
    z["oct_in"], z["oct_u16"], z["oct_u32"] = n3, np.zeros(4096, np.uint32), np.zeros(4096, np.uint32)
    R.vltr_oct_encode(P(n3), P(z["oct_u16"]), P(z["oct_u32"]), 4096)
    u16 = np.ascontiguousarray(np.arange(0, 65536, 8, dtype=np.uint32))
    u32 = rng.integers(0, 2 ** 32, u16.size, dtype=np.uint64).astype(np.uint32)
    z["octd_u16"], z["octd_u32"] = u16, u32
    z["octd_n16"], z["octd_n32"] = np.zeros(3 * u16.size, np.float32), np.zeros(3 * u16.size, np.float32)
    R.vltr_oct_decode(P(u16), P(u32), P(z["octd_n16"]), P(z["octd_n32"]), u16.size)
    M = rng.integers(0, 400, 4096).astype(np.uint32)
    W = (rng.lognormal(0, 6, 4096) * rng.choice([1, -1], 4096)).astype(np.float32)
    z["rs_M"], z["rs_W"] = M, W
    z["rs_enc"], z["rs_dM"], z["rs_dW"] = np.zeros(4096, np.uint32), np.zeros(4096, np.uint32), np.zeros(4096, np.float32)
    R.vltr_reservoir_simple(P(M), P(W), P(z["rs_enc"]), P(z["rs_dM"]), P(z["rs_dW"]), 4096)
    pos = (rng.standard_normal((4096, 3)) * rng.choice([0.01, 1.0, 100.0, 70000.0], (4096, 1))).astype(np.float32)
    z["hpn_pos"], z["hpn_nrm"] = pos, n3
    z["hpn_enc"], z["hpn_dpos"], z["hpn_dnrm"] = (np.zeros(2 * 4096, np.uint32), np.zeros(3 * 4096, np.float32),
                                                 np.zeros(3 * 4096, np.float32))
    R.vltr_hit_pos_normal(P(pos), P(n3), P(z["hpn_enc"]), P(z["hpn_dpos"]), P(z["hpn_dnrm"]), 4096)
    cam = np.array([1.5, 2.0, -3.0], np.float32)
    vpos = (cam + rng.standard_normal((4096, 3)) * rng.choice([0.3, 2.0, 20.0, 300.0], (4096, 1))).astype(np.float32)
    z["vk_cam"], z["vk_pos"], z["vk_out"] = cam, vpos, np.zeros(5 * 4096, np.uint32)
    R.vltr_vertex_key(P(vpos), P(cam), P(z["vk_out"]), 4096)
    enc = rng.integers(0, 2 ** 32, 4 * 4096, dtype=np.uint64).astype(np.uint32)
    z["gb_enc"], z["gb_out"] = enc, np.zeros(11 * 4096, np.float32)
    R.vltr_gbuffer_decode(P(enc), P(z["gb_out"]), 4096)
    np.savez_compressed(PRIM_OUT, **z)
    print("%s: %.0f KB" % (PRIM_OUT, os.path.getsize(PRIM_OUT) / 1024))


def main():
    assert pyref.lib() is not None, "the reference tree is needed to make these fixtures"
    primitives()
    s, cs = cases()
    arrays, manifest = {}, {"width": s.W, "height": s.H, "cases": []}
    for i, c in enumerate(cs):
        outs = c.run()
        entry = {"pass": c.name, "args": [], "expect": []}
        for j, (kind, v) in enumerate(c.args):
            if isinstance(v, np.ndarray):
                key = "c%d_a%d" % (i, j)
                arrays[key] = v
                entry["args"].append([kind, key])
            else:
                entry["args"].append([kind, v])
        for k, o in enumerate(outs):
            key = "c%d_o%d" % (i, k)
            arrays[key] = o
            entry["expect"].append(key)
        manifest["cases"].append(entry)
    arrays["manifest"] = np.frombuffer(json.dumps(manifest).encode(), np.uint8)
    np.savez_compressed(OUT, **arrays)
    print("%s: %d cases, %.0f KB" % (OUT, len(cs), os.path.getsize(OUT) / 1024))


if __name__ == "__main__":
    main()
