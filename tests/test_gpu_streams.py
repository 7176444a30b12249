"""Streams inside a frame: a plain frame runs its hash-grid, specular and AO chains on
the view's side streams, joined back into the caller's stream by events. Its results
must equal those of the same frame run on one stream (per-pass timers on), and the
call must be capturable in a CUDA graph on the caller's stream: a view whose frames
are captured and replayed must match a view that runs them directly, bit for bit.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import d2h, upload

pytestmark = pytest.mark.gpu

OUT_PX = {"ref": 4, "f32": 16, "f16": 8}
NAMES = ["diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance", "ao_history",
         "ao_filtered", "raw_diffuse", "raw_specular", "hist_color", "hist_moments", "hist_record", "hist_len",
         "hg_storage", "hg_decay", "hg_queries", "hg_query_count", "taa_history", "color"]


@pytest.fixture(scope="module")
def ctx():
    c = vg.Context(0)
    yield c
    c.close()


def state_of(view):
    import torch

    torch.cuda.synchronize()
    res = {}
    for name in NAMES:
        try:
            ptr, nb = view.buffer(name)
        except KeyError:
            continue
        res[name] = d2h(ptr, nb)
    return res


def same_state(a, b, what):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), "%s: %s differs" % (what, k)


def params(post):
    p = vg.params_plain(1)
    p.hg_log2_buckets = 10
    p.post = post
    return p


@pytest.mark.parametrize("form", ["ref", "f32", "f16"])
def test_side_streams_match_one_stream(ctx, form):
    import torch

    W, H = 96, 64
    n = W * H
    p = params(2)
    scene = vg.Scene(17, W, H, disocclusion_frac=0.03)
    a = vg.View(ctx, W, H, form, p)
    b = vg.View(ctx, W, H, form, p)
    b.set_timing(True)  # per-pass timers: the frame runs on one stream
    try:
        for f in range(5):
            dev = upload(scene.generate_host(f))
            fp = scene.frame_params(f)
            outs = []
            for v in (a, b):
                o = {k: torch.zeros(OUT_PX[form] * n, dtype=torch.uint8, device="cuda")
                     for k in ("diffuse", "specular", "color", "taa")}
                v.run(fp, f, dev, o)
                outs.append(o)
            same_state(state_of(a), state_of(b), "frame %d" % f)
            torch.cuda.synchronize()
            for k in outs[0]:
                assert torch.equal(outs[0][k], outs[1][k]), "frame %d output %s" % (f, k)
        b.read_timing()
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("form", ["ref", "f32"])
def test_frame_captured_in_cuda_graph(ctx, form):
    import torch

    W, H = 80, 48
    n = W * H
    p = params(0)
    scene = vg.Scene(23, W, H, disocclusion_frac=0.02)
    direct = vg.View(ctx, W, H, form, p)
    graphed = vg.View(ctx, W, H, form, p)
    s = torch.cuda.Stream()
    try:
        for f in range(4):
            dev = upload(scene.generate_host(f))
            fp = scene.frame_params(f)
            out_d = {k: torch.zeros(OUT_PX[form] * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
            out_g = {k: torch.zeros_like(t) for k, t in out_d.items()}
            direct.run(fp, f, dev, out_d)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                graphed.run(fp, f, dev, out_g, stream=s.cuda_stream)
            g.replay()
            torch.cuda.synchronize()
            same_state(state_of(direct), state_of(graphed), "frame %d" % f)
            for k in out_d:
                assert torch.equal(out_d[k], out_g[k]), "frame %d output %s" % (f, k)
    finally:
        direct.close()
        graphed.close()


def test_bound_frame_pointers_match_run(ctx):
    """View.run_bound (pointers bound once to a reused staging slot, as the benchmark's
    end-to-end leg uses them) gives the frames View.run gives."""
    import torch

    W, H = 72, 40
    n = W * H
    p = params(0)
    scene = vg.Scene(29, W, H, disocclusion_frac=0.02)
    a = vg.View(ctx, W, H, "f32", p)
    b = vg.View(ctx, W, H, "f32", p)
    keys = [k for k in vg.FRAME_BUFFERS if k != "shadow_mask"]
    first = scene.generate_host(0)
    sizes = [first[k].nbytes for k in keys]
    offs = [sum((sz + 255) // 256 * 256 for sz in sizes[:j]) for j in range(len(keys))]
    slot = torch.zeros(offs[-1] + sizes[-1], dtype=torch.uint8, device="cuda")
    out_b = torch.zeros(32 * n, dtype=torch.uint8, device="cuda")
    bind = vg.FrameBinding({k: slot[o:o + sz] for k, o, sz in zip(keys, offs, sizes)},
                           {"diffuse": out_b[:16 * n], "specular": out_b[16 * n:]})
    try:
        for f in range(4):
            host = scene.generate_host(f)
            fp = scene.frame_params(f)
            out_a = {k: torch.zeros(16 * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
            a.run(fp, f, upload(host), out_a)
            for k, o, sz in zip(keys, offs, sizes):
                slot[o:o + sz].copy_(torch.from_numpy(host[k].view(np.uint8)))
            b.run_bound(bind, fp, f)
            torch.cuda.synchronize()
            same_state(state_of(a), state_of(b), "frame %d" % f)
            assert torch.equal(out_a["diffuse"], out_b[:16 * n]) and torch.equal(out_a["specular"], out_b[16 * n:])
    finally:
        a.close()
        b.close()
