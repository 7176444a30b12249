"""The oracle's passes against the reference's own shader text, pass by pass.

oracle/_ref/libvlt_ref.so runs each of the reference's compute shaders compiled as
C++ (oracle/ref_build.py) behind the same signature as the oracle's per-pass entry
point (vltr_X beside vlto_X). Both are given the same inputs, taken from a reference
-preset view of the synthetic scene after a few frames (so reservoirs, AO, history
and the hash grid hold realistic state), and their outputs must be identical bit for
bit. The GPU parity tests then tie the kernels to the oracle. Needs the reference
tree (skipped without it).
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from oracle import pyref
from tests.helpers import first_float_mismatch, first_mismatch

REF = pyref.lib()
pytestmark = pytest.mark.skipif(REF is None, reason="reference tree not available")

SIGS = {k.replace("vlto_", "vltr_"): v for k, v in po.SIGS.items()}


def ref(name):
    f = getattr(REF, name)
    r, a = SIGS[name]
    f.restype, f.argtypes = r, a
    return f


def orc(name):
    return getattr(po.lib(), name)


def p_(a):
    return None if a is None else a.ctypes.data


def same(a, b, W, words=None, what=""):
    if words is None:
        msg = first_mismatch(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8), W)
    else:
        msg = first_float_mismatch(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32),
                                   W, words)
    assert msg is None, "%s: %s" % (what, msg)


def same_written(a, b, fill, W, words, depth, what):
    """With outputs pre-filled with a sentinel: every word the reference shader wrote
    equals the oracle's; the words it left unwritten (still the sentinel) belong to
    pixels without geometry, where the oracle defines them (as 0)."""
    if fill == 0:
        return same(a, b, W, words, what)
    a = np.ascontiguousarray(a).view(np.uint32)
    b = np.ascontiguousarray(b).view(np.uint32)
    sentinel = np.uint32(fill * 0x01010101)
    written = b != sentinel
    same(np.where(written, a, 0), np.where(written, b, 0), W, words, what)
    px = np.nonzero(~written)[0] // words
    assert np.all(depth[px] == 0.0), "%s: the reference left words of pixels with geometry unwritten" % what


class State:
    """A reference-preset oracle view after `warm` frames plus the next frame's
    inputs: the inputs of every pass of that next frame."""

    def __init__(self, W=160, H=96, warm=4, seed=17):
        self.W, self.H, self.n = W, H, W * H
        self.params = vg.params_reference()
        self.scene = vg.Scene(seed, W, H, disocclusion_frac=0.02)
        self.view = po.OracleView(W, H, self.params)
        for f in range(warm):
            self.view.run(self.scene.frame_params(f), f, self.scene.generate_host(f))
        self.frame = warm
        self.fp = self.scene.frame_params(warm)
        self.inp = self.scene.generate_host(warm)
        self.rng = np.random.default_rng(seed)

    def buf(self, name, dtype=np.uint8):
        return np.ascontiguousarray(self.view.buffer(name, dtype))

    def rand(self):
        return int(self.rng.integers(0, 2 ** 32))


@pytest.fixture(scope="module")
def st():
    return State()


@pytest.fixture(scope="module")
def st_odd():
    return State(W=37, H=23, warm=3, seed=5)


def both(name, *args):
    """Calls vlto_name and vltr_name; `args` lists inputs, and outputs as
    ('out', nbytes, fill) tuples (the same fill in both). Returns the two output lists."""
    outs = []
    for _ in range(2):
        call, o = [], []
        for a in args:
            if isinstance(a, tuple) and a and a[0] == "out":
                arr = np.full(a[1], a[2], np.uint8)
                o.append(arr)
                call.append(p_(arr))
            elif isinstance(a, tuple) and a and a[0] == "inout":
                arr = np.array(a[1], copy=True)
                o.append(arr)
                call.append(p_(arr))
            elif isinstance(a, np.ndarray):
                call.append(p_(a))
            else:
                call.append(a)
        outs.append((call, o))
    orc(name)(*outs[0][0])
    ref(name.replace("vlto_", "vltr_"))(*outs[1][0])
    return outs[0][1], outs[1][1]


def fp_ptr(fp):
    return C.byref(fp)


@pytest.mark.parametrize("fill", [0, 0xCD])
@pytest.mark.parametrize("has_prev,has_new", [(1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ind_diff_temporal_resample(which, has_prev, has_new, fill, request):
    s = request.getfixturevalue(which)
    a, b = both("vlto_ind_diff_temporal_resample", fp_ptr(s.fp), s.W, s.H, C.byref(s.params),
                s.buf("prev_depth"), s.inp["depth"], s.inp["diff_hit_pos_normal"], s.inp["diff_hit_radiance"], None,
                s.buf("diff_reservoir"), ("out", 16 * s.n, fill), s.rand(), has_prev, has_new)
    same_written(a[0], b[0], fill, s.W, 4, s.inp["depth"], "diffuse reservoir")


def _diff_temporal_out(s):
    out = np.zeros(16 * s.n, np.uint8)
    orc("vlto_ind_diff_temporal_resample")(fp_ptr(s.fp), s.W, s.H, C.byref(s.params), p_(s.buf("prev_depth")),
                                           p_(s.inp["depth"]), p_(s.inp["diff_hit_pos_normal"]),
                                           p_(s.inp["diff_hit_radiance"]), None, p_(s.buf("diff_reservoir")),
                                           p_(out), 12345, 1, 1)
    return out


@pytest.mark.parametrize("fill", [0, 0xCD])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ind_diff_spatial_resample(which, fill, request):
    s = request.getfixturevalue(which)
    rsv = _diff_temporal_out(s)
    a, b = both("vlto_ind_diff_spatial_resample", fp_ptr(s.fp), s.W, s.H, C.byref(s.params), s.inp["gbuffer"],
                s.inp["depth"], s.buf("ao_filtered"), rsv, ("out", 16 * s.n, fill), ("out", 4 * s.n, fill),
                s.rand())
    same_written(a[0], b[0], fill, s.W, 4, s.inp["depth"], "diffuse reservoir")
    same_written(a[1], b[1], fill, s.W, 1, s.inp["depth"], "lighting")


@pytest.mark.parametrize("has_prev,has_new", [(1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ao_gen(which, has_prev, has_new, request):
    s = request.getfixturevalue(which)
    a, b = both("vlto_ao_gen", fp_ptr(s.fp), s.W, s.H, s.inp["diff_hit_pos_normal"], s.inp["depth"],
                s.buf("ao_history"), ("out", 4 * s.n, 0), has_new, has_prev, C.c_float(s.params.ao_radius))
    same(a[0], b[0], s.W, None, "ao history")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ao_filter(which, request):
    s = request.getfixturevalue(which)
    a, b = both("vlto_ao_filter", s.W, s.H, s.inp["depth"], s.buf("ao_history"), ("out", 2 * s.n, 0))
    same(a[0], b[0], s.W, None, "filtered ao")


def _spec_temporal_out(s, frame_rand=777):
    n = s.n
    o = (np.zeros(8 * n, np.uint8), np.zeros(16 * n, np.uint8), np.zeros(4 * n, np.uint8))
    orc("vlto_ind_spec_temporal_resample")(fp_ptr(s.fp), s.W, s.H, C.byref(s.params), p_(s.buf("prev_depth")),
                                           p_(s.buf("prev_gbuffer")), p_(s.inp["depth"]), p_(s.inp["gbuffer"]),
                                           p_(s.buf("spec_reservoir")), p_(s.buf("spec_hit_pos")),
                                           p_(s.buf("spec_radiance")), p_(s.inp["spec_hit_pos"]),
                                           p_(s.inp["spec_hit_radiance"]), *(p_(x) for x in o), frame_rand, 1)
    return o


@pytest.mark.parametrize("has_prev", [1, 0])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ind_spec_temporal_resample(which, has_prev, request):
    s = request.getfixturevalue(which)
    n = s.n
    a, b = both("vlto_ind_spec_temporal_resample", fp_ptr(s.fp), s.W, s.H, C.byref(s.params), s.buf("prev_depth"),
                s.buf("prev_gbuffer"), s.inp["depth"], s.inp["gbuffer"], s.buf("spec_reservoir"),
                s.buf("spec_hit_pos"), s.buf("spec_radiance"), s.inp["spec_hit_pos"], s.inp["spec_hit_radiance"],
                ("out", 8 * n, 0), ("out", 16 * n, 0), ("out", 4 * n, 0), s.rand(), has_prev)
    same(a[0], b[0], s.W, 2, "specular reservoir {M, W}")
    same(a[1], b[1], s.W, 4, "specular hit position / target function")
    same(a[2], b[2], s.W, 1, "specular radiance")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_ind_spec_spatial_resample(which, request):
    s = request.getfixturevalue(which)
    rsv, hp, rad = _spec_temporal_out(s)
    a, b = both("vlto_ind_spec_spatial_resample", fp_ptr(s.fp), s.W, s.H, C.byref(s.params), s.inp["gbuffer"],
                s.inp["depth"], rsv, hp, rad, ("out", 4 * s.n, 0), ("out", 2 * s.n, 0), None, None, None, s.rand())
    same(a[0], b[0], s.W, 1, "specular lighting")
    same(a[1], b[1], s.W, None, "specular ray length")


def _lighting(s):
    """Raw diffuse / specular lighting and ray length of the next frame (oracle)."""
    n = s.n
    rsv = _diff_temporal_out(s)
    drsv, dl = np.zeros(16 * n, np.uint8), np.zeros(4 * n, np.uint8)
    orc("vlto_ind_diff_spatial_resample")(fp_ptr(s.fp), s.W, s.H, C.byref(s.params), p_(s.inp["gbuffer"]),
                                          p_(s.inp["depth"]), p_(s.buf("ao_filtered")), p_(rsv), p_(drsv), p_(dl), 99)
    srsv, shp, srad = _spec_temporal_out(s)
    sl, rl = np.zeros(4 * n, np.uint8), np.zeros(2 * n, np.uint8)
    orc("vlto_ind_spec_spatial_resample")(fp_ptr(s.fp), s.W, s.H, C.byref(s.params), p_(s.inp["gbuffer"]),
                                          p_(s.inp["depth"]), p_(srsv), p_(shp), p_(srad), p_(sl), p_(rl), None,
                                          None, None, 98)
    return dl, sl, rl


def _dn_temporal(s, fast_on=0, has_history=1, fast_hist=None):
    n = s.n
    dl, sl, rl = _lighting(s)
    fast_hist = fast_hist if fast_hist is not None else np.zeros(8 * n, np.uint8)
    args = (fp_ptr(s.fp), s.W, s.H, C.byref(s.params), s.inp["depth"], s.inp["gbuffer"], dl, sl, rl,
            s.buf("prev_depth"), s.buf("prev_gbuffer"), s.buf("hist_color"), s.buf("hist_moments"), s.buf("hist_len"),
            fast_hist, ("out", 8 * n, 0), ("out", 4 * n, 0), ("out", n, 0), ("out", 8 * n, 0), has_history, fast_on)
    return args


@pytest.mark.parametrize("fast_on,has_history", [(0, 1), (1, 1), (0, 0)])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_denoise_temporal(which, fast_on, has_history, request):
    s = request.getfixturevalue(which)
    fast = np.ascontiguousarray(s.buf("hist_color")[::-1])  # any plausible colour records
    a, b = both("vlto_denoise_temporal", *_dn_temporal(s, fast_on, has_history, fast))
    for k, (nm, words) in enumerate([("colour", 2), ("moments", 1), ("history length", None), ("fast history", 2)]):
        if k == 3 and not fast_on:
            continue
        same(a[k], b[k], s.W, words, "denoiser temporal " + nm)


def _temporal_outputs(s):
    args = list(_dn_temporal(s))
    outs = []
    for i, x in enumerate(args):
        if isinstance(x, tuple) and x[0] == "out":
            arr = np.zeros(x[1], np.uint8)
            outs.append(arr)
            args[i] = arr
    orc("vlto_denoise_temporal")(*(p_(x) if isinstance(x, np.ndarray) else x for x in args))
    return outs  # colour, moments, length, fast


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_denoise_disocclusion_fix(which, request):
    s = request.getfixturevalue(which)
    color, mom, ln, _ = _temporal_outputs(s)
    a, b = both("vlto_denoise_disocclusion_fix", s.W, s.H, s.inp["depth"], s.inp["gbuffer"], ln, color, mom,
                ("out", 8 * s.n, 0), ("out", 4 * s.n, 0))
    same(a[0], b[0], s.W, 2, "fix colour")
    same(a[1], b[1], s.W, 1, "fix moments")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_denoise_fast_history_clamp(which, request):
    s = request.getfixturevalue(which)
    color, _, _, _ = _temporal_outputs(s)
    fast = np.ascontiguousarray(s.buf("hist_color"))
    a, b = both("vlto_denoise_fast_history_clamp", s.W, s.H, fast, ("inout", color))
    same(a[0], b[0], s.W, 2, "clamped colour")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_denoise_spatial_fallback(which, request):
    s = request.getfixturevalue(which)
    color, mom, ln, _ = _temporal_outputs(s)
    a, b = both("vlto_denoise_spatial_fallback", s.W, s.H, s.inp["depth"], s.inp["gbuffer"], ln, color, mom,
                ("out", 8 * s.n, 0), ("out", 4 * s.n, 0))
    same(a[0], b[0], s.W, 2, "fallback colour")
    same(a[1], b[1], s.W, 1, "fallback variance")


@pytest.mark.parametrize("step", [1, 2, 4, 16])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_denoise_atrous(which, step, request):
    s = request.getfixturevalue(which)
    color, mom, ln, _ = _temporal_outputs(s)
    c2, var = np.zeros(8 * s.n, np.uint8), np.zeros(4 * s.n, np.uint8)
    orc("vlto_denoise_spatial_fallback")(s.W, s.H, p_(s.inp["depth"]), p_(s.inp["gbuffer"]), p_(ln), p_(color),
                                         p_(mom), p_(c2), p_(var))
    a, b = both("vlto_denoise_atrous", s.W, s.H, s.inp["depth"], s.inp["gbuffer"], c2, var, ("out", 8 * s.n, 0),
                ("out", 4 * s.n, 0), step)
    same(a[0], b[0], s.W, 2, "a-trous colour")
    same(a[1], b[1], s.W, 1, "a-trous variance")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_hg_decay(which, request):
    s = request.getfixturevalue(which)
    a, b = both("vlto_hg_decay", 16, ("inout", s.buf("hg_decay")), ("inout", s.buf("hg_storage")))
    same(a[0], b[0], None, None, "decay bytes")
    same(a[1], b[1], None, 4, "cells")


@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_hg_query_select(which, request):
    s = request.getfixturevalue(which)
    decay, storage = s.buf("hg_decay").copy(), s.buf("hg_storage").copy()
    orc("vlto_hg_decay")(16, p_(decay), p_(storage))
    # The view emits one record per pixel, empty (checksum 0) for pixels without
    # geometry; the reference appends queries for hits only, so the shader sees the
    # non-empty records, densely.
    max_q = s.params.hg_max_queries
    q = s.buf("hg_queries").view(np.uint32).reshape(-1, 8)[: int(s.buf("hg_query_count").view(np.uint32)[0])]
    q = q[q[:, 5] != 0]
    count = np.array([q.shape[0]], np.uint32)
    queries = np.zeros(32 * max_q, np.uint8)
    queries[: q.nbytes] = q.reshape(-1).view(np.uint8)
    a, b = both("vlto_hg_query_select", 16, max_q, queries, count, ("inout", storage),
                ("out", 4 * (16 << 16), 0), s.rand())
    same(a[0], b[0], None, 4, "cells after insertion")
    same(a[1], b[1], None, 1, "selection words")
    assert np.count_nonzero(a[1].view(np.uint32)) > 0


@pytest.mark.parametrize("stride", [1, 2])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_final_lighting(which, stride, request):
    s = request.getfixturevalue(which)
    shadow = np.ascontiguousarray(s.rng.integers(0, 256, s.n).astype(np.uint8))
    hc = s.buf("hist_color")
    diff = hc if stride == 2 else np.ascontiguousarray(hc.view(np.uint32)[0::2])
    spec = np.ascontiguousarray(hc[4:]) if stride == 2 else np.ascontiguousarray(hc.view(np.uint32)[1::2])
    a, b = both("vlto_final_lighting", 0, fp_ptr(s.fp), s.W, s.H, s.inp["gbuffer"], shadow, diff, spec, stride,
                ("out", 4 * s.n, 0))
    same(a[0], b[0], s.W, 1, "final lighting")


@pytest.mark.parametrize("has_history", [1, 0])
@pytest.mark.parametrize("which", ["st", "st_odd"])
def test_temporal_aa(which, has_history, request):
    s = request.getfixturevalue(which)
    hc = s.buf("hist_color").view(np.uint32)
    source = np.ascontiguousarray(hc[0::2])
    history = np.ascontiguousarray(hc[1::2])
    a, b = both("vlto_temporal_aa", 0, fp_ptr(s.fp), s.W, s.H, s.inp["depth"], source, history, has_history,
                ("out", 4 * s.n, 0))
    same(a[0], b[0], s.W, 1, "temporal AA")
