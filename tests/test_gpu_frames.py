"""GPU parity: whole frames through vlt_frame_run vs the CPU oracle, buffer by buffer.

Every resident buffer (reservoirs, AO, denoiser history, variance, hash grid) and
every output is compared bit for bit after each frame. Integer/byte fields and the
binary32 records are exact because the kernels and the oracle follow the same
numeric contract; NaNs (if any) compare equal to NaNs.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, dev_zeros, first_mismatch, to_np, upload

pytestmark = pytest.mark.gpu

STATE_BUFFERS = [
    ("diff_reservoir", np.uint32, 4),
    ("spec_hit_pos", np.uint32, 4),
    ("spec_reservoir", np.uint32, 2),
    ("spec_radiance", np.uint32, 1),
    ("ao_history", np.uint32, 1),
    ("ao_filtered", np.uint16, 1),
    ("raw_diffuse", np.uint32, 1),
    ("raw_specular", np.uint32, 1),
    ("spec_ray_len", np.uint16, 1),
]
DENOISE_BUFFERS = [
    ("hist_color", np.uint32, 2),
    ("hist_moments", np.uint32, 1),
    ("hist_len", np.uint8, 1),
    ("variance", np.uint32, 1),
]


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def run_and_compare(ctx, W, H, params, frames, seed=11, disocc=0.02, check_hg=True):
    scene = vg.Scene(seed, W, H, disocclusion_frac=disocc)
    view = vg.View(ctx, W, H, "ref", params)
    oview = po.OracleView(W, H, params)
    n = W * H
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            dev = upload(host)
            fp = scene.frame_params(f)
            out_dev = {k: dev_zeros(4 * n) for k in ("diffuse", "specular")}
            view.run(fp, f, dev, out_dev)
            out_host = {k: np.zeros(n, np.uint32) for k in ("diffuse", "specular")}
            oview.run(fp, f, host, out_host)
            import torch

            torch.cuda.synchronize()
            names = list(STATE_BUFFERS)
            if params.denoise and f > 0:
                names += DENOISE_BUFFERS
            for name, dt, rec in names:
                ptr, nb = view.buffer(name)
                got = d2h(ptr, nb, dt)
                exp = oview.buffer(name, dt)
                assert got.shape == exp.shape, name
                msg = first_mismatch(got, exp, W, rec)
                assert msg is None, "frame %d %s: %s" % (f, name, msg)
            for k in ("diffuse", "specular"):
                got = to_np(out_dev[k][: 4 * n], np.uint32)
                msg = first_mismatch(got, out_host[k], W)
                assert msg is None, "frame %d output %s: %s" % (f, k, msg)
            if check_hg and params.hg_enable:
                for name, dt in (("hg_storage", np.uint32), ("hg_decay", np.uint8), ("hg_query_count", np.uint32)):
                    ptr, nb = view.buffer(name)
                    got = d2h(ptr, nb, dt)
                    exp = oview.buffer(name, dt)
                    msg = first_mismatch(got, exp)
                    assert msg is None, "frame %d %s: %s" % (f, name, msg)
                cnt = int(oview.buffer("hg_query_count", np.uint32)[0])
                ptr, nb = view.buffer("hg_queries")
                got = d2h(ptr, cnt * 32, np.uint32)
                exp = oview.buffer("hg_queries", np.uint32)[: cnt * 8]
                msg = first_mismatch(got, exp)
                assert msg is None, "frame %d hg_queries: %s" % (f, msg)
        return view, oview
    finally:
        view.close()
        oview.close()


def test_reference_preset_8_frames_320x180(ctx):
    run_and_compare(ctx, 320, 180, vg.params_reference(), 8)


def test_plain_config0_8_frames_320x180(ctx):
    run_and_compare(ctx, 320, 180, vg.params_plain(0), 8, seed=5)


def test_plain_config1_preset_small(ctx):
    # Two spatial passes of 8 taps, 2^22-cell grid keyed by position and normal
    # octant, one query per pixel — at a size the oracle finishes in seconds.
    run_and_compare(ctx, 256, 144, vg.params_plain(1), 5, seed=3)


@pytest.mark.parametrize("W,H", [(17, 9), (1, 1), (33, 7), (2, 64)])
def test_odd_sizes(ctx, W, H):
    run_and_compare(ctx, W, H, vg.params_reference(), 4, seed=W * 100 + H)


def test_no_denoise_and_fast_history(ctx):
    p = vg.params_reference()
    p.denoise = 0
    run_and_compare(ctx, 96, 64, p, 3, seed=2)
    p = vg.params_reference()
    p.fast_history_clamp = 1
    p.disocclusion_fix = 0
    p.atrous_iterations = 0
    run_and_compare(ctx, 96, 64, p, 4, seed=4)


def test_device_scene_matches_host():
    import torch

    W, H = 320, 180
    scene = vg.Scene(99, W, H, disocclusion_frac=0.02)
    n = W * H
    for f in (0, 3):
        host = scene.generate_host(f)
        dev = {k: torch.zeros(v.nbytes, dtype=torch.uint8, device="cuda") for k, v in host.items()}
        scene.generate_device(f, dev)
        torch.cuda.synchronize()
        for k, v in host.items():
            got = dev[k].cpu().numpy().view(v.dtype)
            assert np.array_equal(got.view(np.uint32), v.view(np.uint32)), "frame %d buffer %s" % (f, k)
    assert n > 0
