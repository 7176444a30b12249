"""Precision of the float storage forms against the binary64 denoiser.

Each frame the binary64 restatement of the denoiser is fed with the raw lighting
the GPU form produced (so both work on the same resampled samples) and its output
is compared with the form's denoised output. This isolates what the form's storage
and binary32 arithmetic do to the continuous part of the path (history, moments,
variance, edge-stopping weights). Random resampling decisions are not compared this
way: a selection flips on a one-ulp difference of its probability, so per-pixel
errors between differently rounded resamplers measure noise, not precision.

Bounds: for the f32 form, the first three denoised frames, before any
near-threshold reprojection decision can differ, must agree to 1e-5 relative L2, and
later frames, where a rare validity flip changes a pixel's history, to 5e-3. The f16
form (binary16 history with centered moments) must agree to 1e-3 on every frame.
The binary64 image reductions on the GPU (vlt_image_stats) are checked against numpy.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, dev_zeros, upload

pytestmark = pytest.mark.gpu

BOUNDS = {"f32": (1e-5, 5e-3), "f16": (1e-3, 1e-3)}
DT = {"f32": np.float32, "f16": np.float16}
OUT_PX = {"f32": 16, "f16": 8}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("form", ["f32", "f16"])
@pytest.mark.parametrize("preset", ["reference", "plain0"])
def test_form_against_binary64_denoiser(form, preset):
    import torch

    W, H, frames = 320, 180, 8
    n = W * H
    p = vg.params_reference() if preset == "reference" else vg.params_plain(0)
    ctx = vg.Context(0)
    view = vg.View(ctx, W, H, form, p)
    d64 = po.Denoiser64(W, H, p)
    scene = vg.Scene(11, W, H, disocclusion_frac=0.02)
    dt = DT[form]
    errs = []
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            fp = scene.frame_params(f)
            out = {k: dev_zeros(OUT_PX[form] * n) for k in ("diffuse", "specular")}
            view.run(fp, f, upload(host), out)
            torch.cuda.synchronize()
            ptr, nb = view.buffer("raw_diffuse")
            rd = d2h(ptr, nb, dt).reshape(n, 4).astype(np.float32)
            ptr, nb = view.buffer("raw_specular")
            rs = d2h(ptr, nb, dt).reshape(n, 4).astype(np.float32)
            od, os_ = d64.frame(fp, host, rd[:, :3].copy(), rs[:, :3].copy(), rs[:, 3].copy(), f > 0)
            if f == 0:
                continue
            gd = out["diffuse"].cpu().numpy().view(dt).reshape(n, 4)[:, :3].astype(np.float64)
            gs = out["specular"].cpu().numpy().view(dt).reshape(n, 4)[:, :3].astype(np.float64)
            errs.append((rel_l2(gd, od), rel_l2(gs, os_)))
    finally:
        view.close()
        d64.close()
        ctx.close()
    early, late = BOUNDS[form]
    for k, (ed, es) in enumerate(errs):
        bound = early if k < 3 else late
        assert ed <= bound and es <= bound, "%s/%s frame %d: rel L2 %.3g / %.3g > %.0e" % (form, preset, k + 1, ed,
                                                                                         es, bound)
    print("%s %s rel L2 vs binary64 per denoised frame (diffuse/specular): %s" % (
        form, preset, " ".join("%.1e/%.1e" % e for e in errs)))


def test_image_stats_binary64_reduction():
    import torch

    lib = vg.lib()
    n = 100003
    rng = np.random.default_rng(5)
    a = rng.lognormal(-1.0, 1.5, (n, 4)).astype(np.float32)
    b = (a * (1.0 + 1e-3 * rng.standard_normal((n, 4)))).astype(np.float16)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = lib.vlt_image_stats(C.c_void_p(da.data_ptr()), 0, C.c_void_p(db.data_ptr()), 1, n,
                             C.c_void_p(out.data_ptr()), None)
    assert st == 0
    got = out.cpu().numpy()
    a3 = a[:, :3].astype(np.float64)
    b3 = b[:, :3].astype(np.float64)
    exp = np.concatenate([a3.sum(0), b3.sum(0), [((a3 - b3) ** 2).sum(), (b3 ** 2).sum()]])
    assert np.allclose(got, exp, rtol=1e-12, atol=0), (got, exp)
