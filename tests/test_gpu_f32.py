"""GPU parity of the float storage forms (VLT_FORM_F32, VLT_FORM_F16) against the
oracle's same forms.

Every resident buffer and output is compared byte for byte (NaNs, if any, compare
equal to NaNs): reservoirs, AO, lighting, the specular reservoirs and the hash grid
keep the binary32 contract of the reference form, with the form's own storage
(f32 values, or f16 values stored with round-to-nearest-even and saturation); the
denoiser's records, history length, variance and outputs follow the float forms'
explicit-FMA contract (each FMA one IEEE fusedMultiplyAdd on both sides, own exp2 by
FMA Horner steps, no approximate hardware functions). For the f32 form the relative
L2 error of the denoised outputs, the accuracy figure this form is specified by
(<= 1e-5), is asserted as well.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, dev_zeros, first_float_mismatch, first_mismatch, rel_l2, to_np, upload

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5

# name -> 32-bit words per pixel (None: compare as bytes)
BUFFERS = {
    "f32": [("diff_reservoir", 12), ("spec_hit_pos", 4), ("spec_reservoir", 2), ("spec_radiance", 1),
            ("ao_history", 2), ("ao_filtered", 1), ("raw_diffuse", 4), ("raw_specular", 4)],
    "f16": [("diff_reservoir", None), ("spec_hit_pos", 4), ("spec_reservoir", 2), ("spec_radiance", 1),
            ("ao_history", 1), ("ao_filtered", None),
            ("raw_diffuse", 2), ("raw_specular", 2)],
}
DENOISE = {
    "f32": [("hist_len", None), ("hist_record", 8), ("fallback_record", 8)],
    "f16": [("hist_len", None), ("hist_record", 4), ("fallback_record", 4)],
}
OUT_PX = {"f32": 16, "f16": 8}


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def compare(got, exp, W, words, what):
    assert got.nbytes == exp.nbytes, what
    if words is None:
        a, b = got.view(np.uint8), exp.view(np.uint8)
        msg = first_mismatch(a, b, W)
    else:
        msg = first_float_mismatch(got.view(np.uint32), exp.view(np.uint32), W, words)
    assert msg is None, "%s: %s" % (what, msg)


def run_form(ctx, form, W, H, params, frames, seed=11, disocc=0.02):
    scene = vg.Scene(seed, W, H, disocclusion_frac=disocc)
    view = vg.View(ctx, W, H, form, params)
    oview = po.OracleView(W, H, params, form)
    n = W * H
    ob = OUT_PX[form]
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            dev = upload(host)
            fp = scene.frame_params(f)
            out_dev = {k: dev_zeros(ob * n) for k in ("diffuse", "specular")}
            view.run(fp, f, dev, out_dev)
            out_host = {k: np.zeros(ob * n, np.uint8) for k in ("diffuse", "specular")}
            oview.run(fp, f, host, out_host)
            import torch

            torch.cuda.synchronize()
            denoised = params.denoise and f > 0
            names = BUFFERS[form] + (DENOISE[form] if denoised else [])
            for name, words in names:
                ptr, nb = view.buffer(name)
                compare(d2h(ptr, nb, np.uint8), oview.buffer(name, np.uint8), W, words, "frame %d %s" % (f, name))
            for k in ("diffuse", "specular"):
                got = to_np(out_dev[k][: ob * n], np.uint8)
                compare(got, out_host[k], W, 4 if form == "f32" else 2, "frame %d output %s" % (f, k))
                if form == "f32" and denoised:
                    err, same = rel_l2(got.view(np.float32), out_host[k].view(np.float32))
                    assert same and err <= REL_TOL, "frame %d output %s: rel L2 %.3g" % (f, k, err)
            if params.hg_enable:
                for name, dt in (("hg_storage", np.uint32), ("hg_decay", np.uint8), ("hg_query_count", np.uint32)):
                    ptr, nb = view.buffer(name)
                    msg = first_mismatch(d2h(ptr, nb, dt), oview.buffer(name, dt))
                    assert msg is None, "frame %d %s: %s" % (f, name, msg)
    finally:
        view.close()
        oview.close()


FORMS = ["f32", "f16"]


@pytest.mark.parametrize("form", FORMS)
def test_float_form_reference_preset_8_frames(ctx, form):
    run_form(ctx, form, 320, 180, vg.params_reference(), 8)


@pytest.mark.parametrize("form", FORMS)
def test_float_form_plain_config1_small(ctx, form):
    run_form(ctx, form, 256, 144, vg.params_plain(1), 6, seed=3)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("W,H", [(17, 9), (1, 1), (33, 7), (2, 64)])
def test_float_form_odd_sizes(ctx, form, W, H):
    run_form(ctx, form, W, H, vg.params_reference(), 4, seed=W * 100 + H)


@pytest.mark.parametrize("form", FORMS)
def test_float_form_variants(ctx, form):
    p = vg.params_reference()
    p.denoise = 0
    run_form(ctx, form, 96, 64, p, 3, seed=2)
    p = vg.params_reference()
    p.fast_history_clamp = 1
    p.disocclusion_fix = 0
    p.atrous_iterations = 0
    run_form(ctx, form, 96, 64, p, 4, seed=4)
    p = vg.params_plain(0)
    p.fast_history_clamp = 1
    run_form(ctx, form, 128, 72, p, 5, seed=8)


@pytest.mark.parametrize("form", FORMS)
def test_float_form_reference_buffers_absent(ctx, form):
    view = vg.View(ctx, 32, 16, form, vg.params_reference())
    try:
        for name in ("hist_color", "hist_moments", "variance", "spec_ray_len"):
            with pytest.raises(KeyError):
                view.buffer(name)
    finally:
        view.close()
