"""GPU parity of the passes after the denoiser: the final lighting combine
(restir/final_lighting.hlsl, restir_renderer.rs:897-915) and temporal AA
(temporal_aa.hlsl, restir_renderer.rs:920-948), inside the frame driver
(params.post) in every storage form and through their per-pass entry points.

Both sides evaluate the same binary32 expressions (no contraction, IEEE division and
square root) and store colours with the same rounding (R11G11B10 round-to-nearest-
even with clamping, binary32, or binary16 with saturation), so every comparison is
byte for byte. Colour buffers start filled with a known colour: pixels without
geometry must keep it (the reference's sky pass writes them).
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, first_mismatch, upload

pytestmark = pytest.mark.gpu

PX = {"ref": 4, "f32": 16, "f16": 8}
SKY = (0.25, 0.5, 1.0)


def pack_r11g11b10(rgb):
    rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    r = po.codec("uf11", rgb[:, 0].copy().view(np.uint32))
    g = po.codec("uf11", rgb[:, 1].copy().view(np.uint32))
    b = po.codec("uf10", rgb[:, 2].copy().view(np.uint32))
    return (r | (g << 11) | (b << 22)).astype(np.uint32)


def filled(form, n, rgb=SKY):
    """n pixels of one colour in the form's colour element, as bytes."""
    if form == "ref":
        return np.repeat(pack_r11g11b10(np.array(rgb, np.float32)), n).view(np.uint8)
    dt = np.float32 if form == "f32" else np.float16
    return np.tile(np.array(list(rgb) + [0.0], dt), n).view(np.uint8)


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def compare(got, exp, W, form, what):
    words = got.view(np.uint32) if form != "f16" else got.view(np.uint16)
    ewords = exp.view(np.uint32) if form != "f16" else exp.view(np.uint16)
    rec = {"ref": 1, "f32": 4, "f16": 4}[form]
    msg = first_mismatch(words, ewords, W, rec)
    assert msg is None, "%s: %s" % (what, msg)


def run_post(ctx, form, W, H, params, frames, seed=5, give_color=lambda f: f % 2 == 0, shadow=True):
    import torch

    scene = vg.Scene(seed, W, H, disocclusion_frac=0.02)
    view = vg.View(ctx, W, H, form, params)
    oview = po.OracleView(W, H, params, form)
    n = W * H
    pb = PX[form]
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            if not shadow:
                host.pop("shadow_mask")
            dev = upload(host)
            fp = scene.frame_params(f)
            names = ["diffuse"]
            if params.post >= 1 and give_color(f):
                names.append("color")
            if params.post >= 2:
                names.append("taa")
            init = filled(form, n)
            out_dev = {k: torch.from_numpy(init.copy()).cuda() for k in names}
            out_host = {k: init.copy() for k in names}
            view.run(fp, f, dev, out_dev)
            oview.run(fp, f, host, out_host)
            torch.cuda.synchronize()
            for k in names:
                compare(out_dev[k].cpu().numpy(), out_host[k], W, form, "frame %d output %s" % (f, k))
            for name in ("color", "taa_history"):
                try:
                    exp = oview.buffer(name)
                except KeyError:
                    with pytest.raises(KeyError):
                        view.buffer(name)
                    continue
                ptr, nb = view.buffer(name)
                compare(d2h(ptr, nb), exp, W, form, "frame %d buffer %s" % (f, name))
            if params.post >= 1 and give_color(f):
                # pixels without geometry keep the caller's colour
                sky = host["gbuffer"][3 * n:4 * n] == 0
                got = out_dev["color"].cpu().numpy().reshape(n, pb)
                assert np.array_equal(got[sky], init.reshape(n, pb)[sky]), "frame %d: sky pixels written" % f
    finally:
        view.close()
        oview.close()


FORMS = ["ref", "f32", "f16"]


def post_params(base, post):
    p = base
    p.post = post
    return p


@pytest.mark.parametrize("form", FORMS)
def test_post_reference_preset(ctx, form):
    run_post(ctx, form, 160, 90, post_params(vg.params_reference(), 2), 6)


@pytest.mark.parametrize("form", FORMS)
def test_post_plain_config1(ctx, form):
    p = post_params(vg.params_plain(1), 2)
    p.hg_log2_buckets = 12
    run_post(ctx, form, 128, 72, p, 4, seed=9, give_color=lambda f: True)


@pytest.mark.parametrize("form", FORMS)
def test_post_variants(ctx, form):
    p = post_params(vg.params_reference(), 2)
    p.denoise = 0  # final lighting reads the raw lighting planes
    run_post(ctx, form, 64, 48, p, 3, seed=2)
    p = post_params(vg.params_reference(), 2)
    p.atrous_iterations = 0  # reads the fallback records
    run_post(ctx, form, 64, 48, p, 3, seed=3, shadow=False)
    p = post_params(vg.params_plain(0), 1)  # final lighting only
    run_post(ctx, form, 80, 45, p, 3, seed=4, give_color=lambda f: f != 1)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("W,H", [(17, 9), (1, 1), (2, 33)])
def test_post_odd_sizes(ctx, form, W, H):
    run_post(ctx, form, W, H, post_params(vg.params_reference(), 2), 3, seed=W + H)


def test_post_outputs_need_the_knob(ctx):
    import torch

    sc = vg.Scene(1, 16, 8)
    dev = upload(sc.generate_host(0))
    fp = sc.frame_params(0)
    buf = torch.zeros(4 * 16 * 8, dtype=torch.uint8, device="cuda")
    v0 = vg.View(ctx, 16, 8, "ref", vg.params_reference())
    v1 = vg.View(ctx, 16, 8, "ref", post_params(vg.params_reference(), 1))
    try:
        with pytest.raises(vg.VltError):
            v0.run(fp, 0, dev, {"color": buf})
        with pytest.raises(vg.VltError):
            v1.run(fp, 0, dev, {"taa": buf})
        v1.run(fp, 0, dev, {"color": buf})
        with pytest.raises(KeyError):
            v0.buffer("color")
        with pytest.raises(KeyError):
            v1.buffer("taa_history")
        torch.cuda.synchronize()
    finally:
        v0.close()
        v1.close()


def test_post_reset_drops_taa_history(ctx):
    import torch

    W, H = 48, 32
    n = W * H
    p = post_params(vg.params_reference(), 2)
    sc = vg.Scene(7, W, H)
    view = vg.View(ctx, W, H, "f32", p)
    oview = po.OracleView(W, H, p, "f32")
    try:
        for f in range(2):
            view.run(sc.frame_params(f), f, upload(sc.generate_host(f)))
        view.buffer("taa_history")
        view.reset()
        torch.cuda.synchronize()
        with pytest.raises(KeyError):
            view.buffer("taa_history")
        # after the reset the view runs like a fresh one
        for f in range(2):
            host = sc.generate_host(f)
            out_dev = {"taa": torch.zeros(16 * n, dtype=torch.uint8, device="cuda")}
            out_host = {"taa": np.zeros(16 * n, np.uint8)}
            view.run(sc.frame_params(f), f, upload(host), out_dev)
            oview.run(sc.frame_params(f), f, host, out_host)
            torch.cuda.synchronize()
            compare(out_dev["taa"].cpu().numpy(), out_host["taa"], W, "f32", "after reset, frame %d" % f)
    finally:
        view.close()
        oview.close()


def test_per_pass_final_lighting_and_taa():
    import torch

    lib = vg.lib()
    olib = po.lib()
    W, H = 96, 54
    n = W * H
    sc = vg.Scene(13, W, H)
    rng = np.random.default_rng(3)
    for f in range(3):
        host = sc.generate_host(f)
        fp = sc.frame_params(f)
        diff = pack_r11g11b10(rng.lognormal(-1.0, 1.5, (n, 3)).astype(np.float32))
        spec = pack_r11g11b10(rng.lognormal(-1.0, 1.5, (n, 3)).astype(np.float32))
        hist = pack_r11g11b10(rng.lognormal(-0.5, 1.0, (n, 3)).astype(np.float32))
        init = filled("ref", n).view(np.uint32)
        d = {k: torch.from_numpy(v.view(np.uint8)).cuda() for k, v in
             (("gbuffer", host["gbuffer"]), ("shadow", host["shadow_mask"]), ("diff", diff), ("spec", spec),
              ("depth", host["depth"]), ("hist", hist), ("color", init.copy()))}
        ptr = {k: C.c_void_p(t.data_ptr()) for k, t in d.items()}
        shadow = ptr["shadow"] if f != 1 else None
        assert lib.vlt_final_lighting(C.byref(fp), W, H, ptr["gbuffer"], shadow, ptr["diff"], ptr["spec"],
                                      ptr["color"], None) == 0
        color = init.copy()
        olib.vlto_final_lighting(0, C.byref(fp), W, H, po.ptr(host["gbuffer"]),
                                 po.ptr(host["shadow_mask"]) if f != 1 else None, po.ptr(diff), po.ptr(spec), 1,
                                 po.ptr(color))
        torch.cuda.synchronize()
        got = d["color"].cpu().numpy().view(np.uint32)
        assert first_mismatch(got, color, W) is None, "final lighting frame %d: %s" % (f, first_mismatch(got, color, W))
        for has_history in (0, 1):
            tgt = torch.zeros(4 * n, dtype=torch.uint8, device="cuda")
            assert lib.vlt_temporal_aa(C.byref(fp), W, H, ptr["depth"], ptr["color"], ptr["hist"], has_history,
                                       C.c_void_p(tgt.data_ptr()), None) == 0
            exp = np.zeros(n, np.uint32)
            olib.vlto_temporal_aa(0, C.byref(fp), W, H, po.ptr(host["depth"]), po.ptr(color), po.ptr(hist),
                                  has_history, po.ptr(exp))
            torch.cuda.synchronize()
            got = tgt.cpu().numpy().view(np.uint32)
            msg = first_mismatch(got, exp, W)
            assert msg is None, "taa frame %d has_history %d: %s" % (f, has_history, msg)
    # argument checks
    assert lib.vlt_temporal_aa(C.byref(fp), W, H, ptr["depth"], ptr["color"], None, 1, ptr["hist"], None) != 0
    assert lib.vlt_final_lighting(C.byref(fp), W, H, None, None, ptr["diff"], ptr["spec"], ptr["color"], None) != 0
