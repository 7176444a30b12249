"""GPU parity at the benchmarked size: the plain 1920x1080 workload (two spatial
passes of 8 taps per channel, 5 a-trous iterations, 2^22-cell hash grid keyed by
position and normal octant, one query per pixel, so the selection word keeps 21
query-index bits) against the CPU oracle, every resident buffer and output compared
after every frame.

- FP32 storage form, 64 frames (the benchmarked form and length): bit for bit
  against the oracle's FP32 form, and the denoised outputs within 1e-5 relative L2
  of an oracle whose a-trous evaluates the edge-stopping weight with the reference's
  own formulas (svgf.inc.hlsl:60-82: exp of the summed log-weights, pow(n, 128), the
  depth term by division, every operation separately rounded). The float forms
  evaluate that weight in base 2 with a short polynomial and fused multiply-adds; the
  history is fed back before the a-trous (denoising.rs:206-213), so the difference
  stays inside each frame's filter and does not accumulate. The per-frame errors are
  printed.
- Reference storage form, 8 frames: bit for bit.
- FP16 storage form at the 3840x2160 precision workload with the same knobs, 8
  frames: bit for bit.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, first_float_mismatch, first_mismatch, rel_l2

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
N = W * H
REF_WEIGHTS_TOL = 1e-5

F32_BUFFERS = [("diff_reservoir", 12), ("spec_hit_pos", 4), ("spec_reservoir", 2), ("spec_radiance", 1),
               ("ao_history", 2), ("ao_filtered", 1), ("raw_diffuse", 4), ("raw_specular", 4)]
F32_DENOISE = [("hist_len", None), ("hist_record", 8), ("fallback_record", 8)]
REF_BUFFERS = [("diff_reservoir", 4), ("spec_hit_pos", 4), ("spec_reservoir", 2), ("spec_radiance", 1),
               ("ao_history", 1), ("ao_filtered", None), ("raw_diffuse", 1), ("raw_specular", 1),
               ("spec_ray_len", None)]
REF_DENOISE = [("hist_color", 2), ("hist_moments", 1), ("hist_len", None), ("variance", 1)]
F16_BUFFERS = [("diff_reservoir", None), ("spec_hit_pos", 4), ("spec_reservoir", 2), ("spec_radiance", 1),
               ("ao_history", 1), ("ao_filtered", None), ("raw_diffuse", 2), ("raw_specular", 2)]
F16_DENOISE = [("hist_len", None), ("hist_record", 4), ("fallback_record", 4)]
OUT_PX = {"ref": 4, "f32": 16, "f16": 8}
OUT_WORDS = {"ref": 1, "f32": 4, "f16": 2}
LISTS = {"ref": (REF_BUFFERS, REF_DENOISE), "f32": (F32_BUFFERS, F32_DENOISE), "f16": (F16_BUFFERS, F16_DENOISE)}


def _compare(got, exp, words, what, width=W):
    assert got.nbytes == exp.nbytes, what
    if words is None:
        msg = first_mismatch(got.view(np.uint8), exp.view(np.uint8), width)
    else:
        msg = first_float_mismatch(got.view(np.uint32), exp.view(np.uint32), width, words)
    assert msg is None, "%s: %s" % (what, msg)


def _run(form, frames, with_reference_weights, W=W, H=H):
    import torch

    N = W * H
    params = vg.params_plain(1)
    assert params.diff_spatial_passes == 2 and params.diff_spatial_taps == 8 and params.hg_log2_buckets == 18
    ctx = vg.Context(0)
    scene = vg.Scene(1000, W, H, disocclusion_frac=0.02)
    view = vg.View(ctx, W, H, form, params)
    oview = po.OracleView(W, H, params, form)
    rview = None
    if with_reference_weights:
        rview = po.OracleView(W, H, params, form)
        rview.set_atrous_reference_weights(True)
    ob = OUT_PX[form]
    bufs, den = LISTS[form]
    dev = {k: torch.empty(N * c * np.dtype(dt).itemsize, dtype=torch.uint8, device="cuda")
           for k, (dt, c) in vg.FRAME_BUFFERS.items()}
    out_dev = {k: torch.zeros(ob * N, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
    errs = []
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            for k, arr in host.items():
                dev[k].copy_(torch.from_numpy(arr.view(np.uint8)))
            fp = scene.frame_params(f)
            view.run(fp, f, dev, out_dev)
            out_host = {k: np.zeros(ob * N, np.uint8) for k in ("diffuse", "specular")}
            oview.run(fp, f, host, out_host)
            torch.cuda.synchronize()
            names = bufs + (den if f > 0 else [])
            for name, words in names:
                ptr, nb = view.buffer(name)
                _compare(d2h(ptr, nb, np.uint8), oview.buffer(name, np.uint8), words, "frame %d %s" % (f, name), W)
            got_out = {}
            for k in ("diffuse", "specular"):
                got_out[k] = out_dev[k].cpu().numpy()
                _compare(got_out[k], out_host[k], OUT_WORDS[form], "frame %d output %s" % (f, k), W)
            for name, dt in (("hg_storage", np.uint32), ("hg_decay", np.uint8), ("hg_query_count", np.uint32)):
                ptr, nb = view.buffer(name)
                msg = first_mismatch(d2h(ptr, nb, dt), oview.buffer(name, dt))
                assert msg is None, "frame %d %s: %s" % (f, name, msg)
            cnt = int(oview.buffer("hg_query_count", np.uint32)[0])
            ptr, nb = view.buffer("hg_queries")
            msg = first_mismatch(d2h(ptr, cnt * 32, np.uint32), oview.buffer("hg_queries", np.uint32)[: cnt * 8])
            assert msg is None, "frame %d hg_queries: %s" % (f, msg)
            if rview is not None:
                ref_out = {k: np.zeros(ob * N, np.uint8) for k in ("diffuse", "specular")}
                rview.run(fp, f, host, ref_out)
                if f > 0:
                    e = []
                    for k in ("diffuse", "specular"):
                        g = got_out[k].view(np.float32).reshape(N, 4)[:, :3]
                        r = ref_out[k].view(np.float32).reshape(N, 4)[:, :3]
                        err, same = rel_l2(g, r)
                        assert same, "frame %d %s: non-finite values differ from the reference-weight oracle" % (f, k)
                        e.append(err)
                    errs.append(tuple(e))
                    assert max(e) <= REF_WEIGHTS_TOL, "frame %d: rel L2 vs reference-weight a-trous %.3g / %.3g" % (
                        f, e[0], e[1])
    finally:
        view.close()
        oview.close()
        if rview is not None:
            rview.close()
        ctx.close()
    return errs


def test_config1_fullsize_f32_64_frames_bitexact_and_reference_weights():
    errs = _run("f32", 64, True)
    d = np.array(errs)
    print("1920x1080 f32, rel L2 vs reference-weight a-trous over %d denoised frames: diffuse max %.2e mean %.2e, "
          "specular max %.2e mean %.2e" % (len(errs), d[:, 0].max(), d[:, 0].mean(), d[:, 1].max(), d[:, 1].mean()))


def test_config1_fullsize_reference_form_8_frames_bitexact():
    _run("ref", 8, False)


def test_config2_4k_f16_8_frames_bitexact():
    _run("f16", 8, False, W=3840, H=2160)
