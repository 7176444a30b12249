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


def _seq_outputs(n, px, frames):
    import torch

    return [{k: torch.zeros(px * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
            for _ in range(frames)]


@pytest.mark.parametrize("form", ["ref", "f32", "f16"])
def test_frame_sequence_matches_frame_by_frame(ctx, form):
    """vlt_frames_run (frame k's denoiser beside frame k + 1's resampling passes) gives
    every frame's outputs and the final state that vlt_frame_run gives frame by frame,
    across two sequence calls; a frame that asks for raw outputs in the middle runs
    unpipelined (the side streams join first)."""
    import torch

    W, H = 96, 64
    n = W * H
    p = params(0)
    scene = vg.Scene(31, W, H, disocclusion_frac=0.03)
    a = vg.View(ctx, W, H, form, p)
    b = vg.View(ctx, W, H, form, p)
    px = OUT_PX[form]
    try:
        frames = [upload(scene.generate_host(f)) for f in range(11)]
        fps = [scene.frame_params(f) for f in range(11)]
        out_a = _seq_outputs(n, px, 11)
        out_b = _seq_outputs(n, px, 11)
        for f in (4, 9):  # raw outputs requested: these frames run unpipelined
            for o in (out_a[f], out_b[f]):
                o["raw_diffuse"] = torch.zeros(px * n, dtype=torch.uint8, device="cuda")
                o["raw_specular"] = torch.zeros(px * n, dtype=torch.uint8, device="cuda")
        for f in range(11):
            a.run(fps[f], f, frames[f], out_a[f])
        for lo, hi in ((0, 6), (6, 11)):
            seq = vg.FrameSequence(fps[lo:hi], list(range(lo, hi)), frames[lo:hi], out_b[lo:hi])
            b.run_sequence(seq)
            assert b.launches > 0
        torch.cuda.synchronize()
        same_state(state_of(a), state_of(b), "after 11 frames")
        for f in range(11):
            for k in out_a[f]:
                assert torch.equal(out_a[f][k], out_b[f][k]), "frame %d output %s" % (f, k)
    finally:
        a.close()
        b.close()


def test_frame_sequence_with_post_passes_and_graph(ctx):
    """A view with final lighting and TAA runs its sequence frame by frame (equal to
    vlt_frame_run); a pipelined sequence captured in a CUDA graph on the caller's
    stream replays to the same results (the side streams join before the capture
    ends)."""
    import torch

    W, H = 80, 48
    n = W * H
    scene = vg.Scene(37, W, H, disocclusion_frac=0.02)
    frames = [upload(scene.generate_host(f)) for f in range(6)]
    fps = [scene.frame_params(f) for f in range(6)]
    # post passes: unpipelined inside the sequence
    p2 = params(2)
    a = vg.View(ctx, W, H, "f32", p2)
    b = vg.View(ctx, W, H, "f32", p2)
    try:
        out_a = _seq_outputs(n, 16, 6)
        out_b = _seq_outputs(n, 16, 6)
        for f in range(6):
            a.run(fps[f], f, frames[f], out_a[f])
        b.run_sequence(vg.FrameSequence(fps, list(range(6)), frames, out_b))
        torch.cuda.synchronize()
        same_state(state_of(a), state_of(b), "post = 2")
        for f in range(6):
            for k in out_a[f]:
                assert torch.equal(out_a[f][k], out_b[f][k]), "post = 2, frame %d output %s" % (f, k)
    finally:
        a.close()
        b.close()
    # captured: frames 0-2 directly, frames 3-5 as one captured sequence
    p0 = params(0)
    direct = vg.View(ctx, W, H, "f32", p0)
    graphed = vg.View(ctx, W, H, "f32", p0)
    s = torch.cuda.Stream()
    try:
        out_d = _seq_outputs(n, 16, 6)
        out_g = _seq_outputs(n, 16, 6)
        for f in range(6):
            direct.run(fps[f], f, frames[f], out_d[f])
        graphed.run_sequence(vg.FrameSequence(fps[:3], [0, 1, 2], frames[:3], out_g[:3]))
        torch.cuda.synchronize()
        seq = vg.FrameSequence(fps[3:], [3, 4, 5], frames[3:], out_g[3:])
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            graphed.run_sequence(seq, stream=s.cuda_stream)
        g.replay()
        torch.cuda.synchronize()
        same_state(state_of(direct), state_of(graphed), "captured sequence")
        for f in range(6):
            for k in out_d[f]:
                assert torch.equal(out_d[f][k], out_g[f][k]), "captured, frame %d output %s" % (f, k)
    finally:
        direct.close()
        graphed.close()


def test_frame_sequence_refuses_bad_frames(ctx):
    """A sequence with one invalid frame runs none of its frames; a traced view refuses
    sequences."""
    import torch

    W, H = 64, 32
    n = W * H
    scene = vg.Scene(41, W, H)
    frames = [upload(scene.generate_host(f)) for f in range(3)]
    fps = [scene.frame_params(f) for f in range(3)]
    v = vg.View(ctx, W, H, "f32", params(0))
    try:
        before = state_of(v)
        bad = dict(frames[2])
        del bad["spec_hit_pos"]
        with pytest.raises(vg.VltError) as e:
            v.run_sequence(vg.FrameSequence(fps, [0, 1, 2], frames[:2] + [bad], _seq_outputs(n, 16, 3)))
        assert e.value.status == 1
        same_state(before, state_of(v), "refused sequence")
    finally:
        v.close()
    pt = params(0)
    pt.trace = 1
    t = vg.View(ctx, W, H, "f32", pt)
    try:
        with pytest.raises(vg.VltError) as e:
            t.run_sequence(vg.FrameSequence(fps[:1], [0], frames[:1]))
        assert e.value.status == 1
    finally:
        t.close()
