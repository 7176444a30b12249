"""GPU parity of traced mode (params.trace = 1) against the oracle, with the synthetic
scene as the caller's ray tracer.

Each frame: vlt_frame_trace produces the rays (hash-grid update rays, diffuse
candidates or, every 4th frame, the re-trace of last frame's diffuse samples, and the
re-trace of last frame's specular samples); the rays must equal the oracle's bit for
bit; the scene traces them on the GPU (and on the host for the oracle, which must
give the same hits); vlt_frame_run shades the hits (sun, screen-space cache of last
frame's denoised diffuse, world-space hash grid with query recording), validates,
updates the cache and runs the rest of the frame. Every resident buffer, the hash
grid and its query list, and the outputs are compared byte for byte.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po
from tests.helpers import d2h, first_mismatch, upload

pytestmark = pytest.mark.gpu

OUT_PX = {"ref": 4, "f32": 16, "f16": 8}
STATE = {
    "ref": ["diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance", "ao_history", "ao_filtered",
            "raw_diffuse", "raw_specular", "hist_color", "hist_moments", "hist_len"],
    "f32": ["diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance", "ao_history", "ao_filtered",
            "raw_diffuse", "raw_specular", "hist_record", "hist_len"],
    "f16": ["diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance", "ao_history", "ao_filtered",
            "raw_diffuse", "raw_specular", "hist_record", "hist_len"],
}


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def traced_params(base=None, **kw):
    p = base if base is not None else vg.params_reference()
    p.trace = 1
    p.diff_validate = 1
    p.spec_validate = 1
    p.hg_log2_buckets = 10
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def words_equal(got, exp, what, W=None):
    assert got.nbytes == exp.nbytes, "%s: %d vs %d bytes" % (what, got.nbytes, exp.nbytes)
    g, e = got.view(np.uint32), exp.view(np.uint32)
    gf, ef = g.view(np.float32), e.view(np.float32)
    same = (g == e) | (np.isnan(gf) & np.isnan(ef))
    if not same.all():
        i = int(np.nonzero(~same)[0][0])
        raise AssertionError("%s: %d words differ; first word %d: gpu 0x%08x oracle 0x%08x" % (
            what, int((~same).sum()), i, int(g[i]), int(e[i])))


def run_traced(ctx, form, W, H, params, frames, seed=5):
    import torch

    n = W * H
    scene = vg.Scene(seed, W, H, disocclusion_frac=0.02)
    view = vg.View(ctx, W, H, form, params)
    oview = po.OracleView(W, H, params, form)
    nq = view.cache_ray_capacity
    rays = {"cache": torch.zeros(max(nq, 1) * 32, dtype=torch.uint8, device="cuda"),
            "diffuse": torch.zeros(n * 32, dtype=torch.uint8, device="cuda"),
            "spec_validate": torch.zeros(n * 32, dtype=torch.uint8, device="cuda")}
    hits = {k: torch.zeros(t.numel() * 2, dtype=torch.uint8, device="cuda") for k, t in rays.items()}
    kinds = []
    try:
        for f in range(frames):
            host = scene.generate_host(f)
            dev = upload(host)
            fp = scene.frame_params(f)
            counts = view.trace(fp, f, dev, rays)
            orays, ocounts = oview.trace(fp, f, host)
            assert counts == ocounts, "frame %d ray counts %r vs %r" % (f, counts, ocounts)
            kinds.append(counts["diffuse_kind"])
            dev_in = dict(dev)
            host_in = dict(host)
            for k, name in (("cache", "cache_hits"), ("diffuse", "diffuse_hits"),
                            ("spec_validate", "spec_validate_hits")):
                c = counts[k]
                if not c:
                    continue
                torch.cuda.synchronize()
                words_equal(rays[k][: 32 * c].cpu().numpy(), orays[k][: 8 * c], "frame %d %s rays" % (f, k))
                scene.trace_device(fp, rays[k], c, hits[k])
                ohits = scene.trace_host(fp, orays[k], c)
                torch.cuda.synchronize()
                words_equal(hits[k][: 64 * c].cpu().numpy(), ohits, "frame %d %s hits" % (f, k))
                dev_in[name] = hits[k]
                host_in[name] = ohits
            ob = OUT_PX[form]
            out_dev = {k: torch.zeros(ob * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
            out_host = {k: np.zeros(ob * n, np.uint8) for k in ("diffuse", "specular")}
            view.run(fp, f, dev_in, out_dev)
            oview.run(fp, f, host_in, out_host)
            torch.cuda.synchronize()
            for name in STATE[form]:
                try:
                    exp = oview.buffer(name)
                except KeyError:
                    continue
                ptr, nb = view.buffer(name)
                words_equal(d2h(ptr, nb), exp, "frame %d %s" % (f, name)) if nb % 4 == 0 else \
                    np.testing.assert_array_equal(d2h(ptr, nb), exp, "frame %d %s" % (f, name))
            for k in out_dev:
                words_equal(out_dev[k].cpu().numpy(), out_host[k], "frame %d output %s" % (f, k))
            if not params.hg_enable:
                continue
            for name, dt in (("hg_storage", np.uint32), ("hg_decay", np.uint8), ("hg_query_count", np.uint32)):
                ptr, nb = view.buffer(name)
                msg = first_mismatch(d2h(ptr, nb, dt), oview.buffer(name, dt))
                assert msg is None, "frame %d %s: %s" % (f, name, msg)
            qc = min(int(oview.buffer("hg_query_count", np.uint32)[0]), params.hg_max_queries or n)
            ptr, _ = view.buffer("hg_queries")
            msg = first_mismatch(d2h(ptr, qc * 32, np.uint32), oview.buffer("hg_queries", np.uint32)[: qc * 8])
            assert msg is None, "frame %d hg_queries: %s" % (f, msg)
            # hash_grid_visualize over this frame's surfaces, both debug views
            sptr, _ = view.buffer("hg_storage")
            for code in (0, 1):
                vis = torch.zeros(4 * n, dtype=torch.uint8, device="cuda")
                assert vg.lib().vlt_hg_visualize(C.byref(fp), W, H, params.hg_log2_buckets, params.hg_key_mode,
                                                 C.c_void_p(dev["depth"].data_ptr()),
                                                 C.c_void_p(dev["gbuffer"].data_ptr()), C.c_void_p(sptr), code,
                                                 C.c_void_p(vis.data_ptr()), None) == 0
                ovis = np.zeros(n, np.uint32)
                ost = oview.buffer("hg_storage", np.uint32)
                po.lib().vlto_hg_visualize(C.byref(fp), W, H, params.hg_log2_buckets, params.hg_key_mode,
                                           po.ptr(host["depth"]), po.ptr(host["gbuffer"]), po.ptr(ost), code,
                                           po.ptr(ovis))
                torch.cuda.synchronize()
                msg = first_mismatch(vis.cpu().numpy().view(np.uint32), ovis, W)
                assert msg is None, "frame %d hg_visualize(%d): %s" % (f, code, msg)
    finally:
        view.close()
        oview.close()
    return kinds


FORMS = ["ref", "f32", "f16"]


@pytest.mark.parametrize("form", FORMS)
def test_traced_frames_match_oracle(ctx, form):
    kinds = run_traced(ctx, form, 96, 64, traced_params(), 9)
    assert kinds == [1, 1, 1, 1, 2, 1, 1, 1, 2]  # validation frames 4 and 8


@pytest.mark.parametrize("form", FORMS)
def test_traced_variants(ctx, form):
    # no validation, plain knobs (two spatial passes), with the post passes
    p = traced_params(vg.params_plain(1), diff_validate=0, spec_validate=0, post=2, hg_log2_buckets=11)
    run_traced(ctx, form, 80, 48, p, 5, seed=9)
    # no denoiser: the screen-space cache reads the raw lighting
    p = traced_params(denoise=0)
    run_traced(ctx, form, 48, 32, p, 5, seed=4)
    # no hash grid: no world-space cache, no queries
    p = traced_params(hg_enable=0)
    run_traced(ctx, form, 40, 24, p, 5, seed=6)


def test_traced_odd_sizes(ctx):
    for W, H in ((17, 9), (1, 1), (3, 40)):
        run_traced(ctx, "f32", W, H, traced_params(), 5, seed=W * H)


def test_traced_api_contract(ctx):
    import torch

    W, H = 16, 8
    sc = vg.Scene(1, W, H)
    dev = upload(sc.generate_host(0))
    fp = sc.frame_params(0)
    v = vg.View(ctx, W, H, "ref", traced_params())
    try:
        # phase two without phase one
        with pytest.raises(vg.VltError):
            v.run(fp, 0, dev)
        rays = {k: torch.zeros(max(v.cache_ray_capacity, W * H) * 32, dtype=torch.uint8, device="cuda")
                for k in ("cache", "diffuse", "spec_validate")}
        counts = v.trace(fp, 0, dev, rays)
        assert counts["cache"] == 0 and counts["spec_validate"] == 0 and counts["diffuse_kind"] == 1
        # hits missing for the diffuse rays
        with pytest.raises(vg.VltError):
            v.run(fp, 0, dev)
        # a batch takes no traced view
        b = vg.Batch(ctx)
        try:
            with pytest.raises(vg.VltError):
                b.run([v], [fp], [0], [dev])
        finally:
            b.close()
        torch.cuda.synchronize()
    finally:
        v.close()
    # validation needs traced mode
    p = vg.params_reference()
    p.diff_validate = 1
    with pytest.raises(vg.VltError):
        vg.View(ctx, W, H, "ref", p)
    # a plain view has no traced phase
    v = vg.View(ctx, W, H, "ref", vg.params_reference())
    try:
        with pytest.raises(vg.VltError):
            v.trace(fp, 0, dev, {"diffuse": torch.zeros(W * H * 32, dtype=torch.uint8, device="cuda")})
    finally:
        v.close()
