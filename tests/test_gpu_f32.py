"""GPU parity of the f32 storage form (VLT_FORM_F32) against the oracle's F32 form.

Every buffer is compared bit for bit (NaNs, if any, compare equal to NaNs):
reservoirs, AO, lighting, the specular reservoirs and the hash grid keep the
binary32 contract of the reference form without quantizing between passes; the
denoiser's records, history length, variance and outputs follow the form's
explicit-FMA contract (each FMA one IEEE fusedMultiplyAdd on both sides, own exp2
by FMA Horner steps, no approximate hardware functions). The relative L2 error of
the denoised outputs, the accuracy figure this form is specified by (<= 1e-5), is
asserted as well, so a change that trades exactness for speed still has a bound.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, dev_zeros, first_float_mismatch, first_mismatch, rel_l2, to_np, upload

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5

EXACT = [
    ("diff_reservoir", 12),
    ("spec_hit_pos", 4),
    ("spec_reservoir", 2),
    ("spec_radiance", 1),
    ("ao_history", 2),
    ("ao_filtered", 1),
    ("raw_diffuse", 4),
    ("raw_specular", 4),
]
DENOISE_EXACT = [("hist_len", 1), ("hist_record", 8), ("fallback_record", 8)]


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def run_f32(ctx, W, H, params, frames, seed=11, disocc=0.02):
    scene = vg.Scene(seed, W, H, disocclusion_frac=disocc)
    view = vg.View(ctx, W, H, "f32", params)
    oview = po.OracleView(W, H, params, "f32")
    n = W * H
    worst = 0.0
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            dev = upload(host)
            fp = scene.frame_params(f)
            out_dev = {k: dev_zeros(16 * n) for k in ("diffuse", "specular")}
            view.run(fp, f, dev, out_dev)
            out_host = {k: np.zeros(4 * n, np.float32) for k in ("diffuse", "specular")}
            oview.run(fp, f, host, out_host)
            import torch

            torch.cuda.synchronize()
            denoised = params.denoise and f > 0
            names = EXACT + (DENOISE_EXACT if denoised else [])
            for name, rec in names:
                ptr, nb = view.buffer(name)
                got = d2h(ptr, nb, np.uint32)
                exp = oview.buffer(name, np.uint32)
                assert got.shape == exp.shape, name
                msg = first_float_mismatch(got, exp, W, rec)
                assert msg is None, "frame %d %s: %s" % (f, name, msg)
            for k in ("diffuse", "specular"):
                got = to_np(out_dev[k][: 16 * n], np.float32)
                err, same = rel_l2(got, out_host[k])
                assert same, "frame %d output %s: non-finite pattern differs" % (f, k)
                assert err <= REL_TOL, "frame %d output %s: rel L2 %.3g" % (f, k, err)
                worst = max(worst, err)
                msg = first_float_mismatch(got, out_host[k], W, 4)
                assert msg is None, "frame %d output %s: %s" % (f, k, msg)
            if params.hg_enable:
                for name, dt in (("hg_storage", np.uint32), ("hg_decay", np.uint8), ("hg_query_count", np.uint32)):
                    ptr, nb = view.buffer(name)
                    msg = first_mismatch(d2h(ptr, nb, dt), oview.buffer(name, dt))
                    assert msg is None, "frame %d %s: %s" % (f, name, msg)
        return worst
    finally:
        view.close()
        oview.close()


def test_f32_reference_preset_8_frames(ctx):
    run_f32(ctx, 320, 180, vg.params_reference(), 8)


def test_f32_plain_config1_small(ctx):
    run_f32(ctx, 256, 144, vg.params_plain(1), 6, seed=3)


@pytest.mark.parametrize("W,H", [(17, 9), (1, 1), (33, 7), (2, 64)])
def test_f32_odd_sizes(ctx, W, H):
    run_f32(ctx, W, H, vg.params_reference(), 4, seed=W * 100 + H)


def test_f32_variants(ctx):
    p = vg.params_reference()
    p.denoise = 0
    run_f32(ctx, 96, 64, p, 3, seed=2)
    p = vg.params_reference()
    p.fast_history_clamp = 1
    p.disocclusion_fix = 0
    p.atrous_iterations = 0
    run_f32(ctx, 96, 64, p, 4, seed=4)
    p = vg.params_plain(0)
    p.fast_history_clamp = 1
    run_f32(ctx, 128, 72, p, 5, seed=8)


def test_f32_reference_form_buffers_absent(ctx):
    view = vg.View(ctx, 32, 16, "f32", vg.params_reference())
    try:
        for name in ("hist_color", "hist_moments", "variance", "spec_ray_len"):
            with pytest.raises(KeyError):
                view.buffer(name)
    finally:
        view.close()
