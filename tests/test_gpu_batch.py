"""Batched frames (vlt_batch_run) against the same views run one by one (vlt_frame_run).

Every view of a batch must end each frame with exactly the state and outputs it has
when it runs alone: the batched kernels run the same per-pixel bodies, and views
never share buffers. The mix covers both storage forms, different parameter sets and
sizes, a view that joins after the others (so its pass sequence differs: no history,
no denoiser), CUDA-graph replay on a non-default stream, and the tile-shape
autotuner (which changes block shapes between frames).
"""
import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import d2h, upload

pytestmark = pytest.mark.gpu

BUFFERS = ["diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance", "ao_history",
           "ao_filtered", "raw_diffuse", "raw_specular", "hist_len", "hg_storage", "hg_decay", "hg_query_count",
           "color", "taa_history"]
REF_ONLY = ["hist_color", "hist_moments", "variance", "spec_ray_len"]
F32_ONLY = ["hist_record", "fallback_record"]


def small_plain1():
    p = vg.params_plain(1)
    p.hg_log2_buckets = 12
    return p


def with_post(p, post):
    p.post = post
    return p


def view_specs():
    # (width, height, form, params, seed, first frame)
    return [
        (96, 64, "ref", with_post(vg.params_reference(), 2), 1, 0),
        (160, 90, "f32", with_post(vg.params_plain(0), 1), 2, 0),
        (33, 17, "f32", vg.params_reference(), 3, 0),
        (128, 72, "ref", small_plain1(), 4, 0),
        (64, 64, "f32", small_plain1(), 5, 2),  # joins at frame 2
        (1, 1, "ref", vg.params_reference(), 6, 1),
        (48, 40, "f16", with_post(vg.params_plain(0), 2), 7, 0),
        (20, 12, "f16", vg.params_reference(), 8, 1),
    ]


def out_bytes(form, n):
    return {"ref": 4, "f32": 16, "f16": 8}[form] * n


def state_of(view, form):
    import torch

    torch.cuda.synchronize()
    names = BUFFERS + (REF_ONLY if form == "ref" else F32_ONLY)
    res = {}
    for name in names:
        try:
            ptr, nb = view.buffer(name)
        except KeyError:
            continue
        res[name] = d2h(ptr, nb)
    return res


def run_pair(frames, graphs=True, autotune=False, use_stream=True, chunk_pixels=None):
    import torch

    ctx = vg.Context(0)
    specs = view_specs()
    scenes = [vg.Scene(seed, w, h, disocclusion_frac=0.02) for (w, h, form, p, seed, f0) in specs]
    alone = [vg.View(ctx, w, h, form, p) for (w, h, form, p, seed, f0) in specs]
    batched = [vg.View(ctx, w, h, form, p) for (w, h, form, p, seed, f0) in specs]
    batch = vg.Batch(ctx)
    batch.set_graphs(graphs)
    if chunk_pixels:
        batch.set_chunk_pixels(chunk_pixels)
    if autotune:
        batch.autotune()
    stream = torch.cuda.Stream() if use_stream else None
    sh = stream.cuda_stream if stream is not None else 0
    try:
        for f in range(frames):
            active = [k for k, s in enumerate(specs) if f >= s[5]]
            fps, inputs, outs_a, outs_b, idx = [], [], [], [], []
            for k in active:
                w, h, form, p, seed, f0 = specs[k]
                lf = f - f0
                host = scenes[k].generate_host(lf)
                dev = upload(host)
                fp = scenes[k].frame_params(lf)
                n = w * h
                names = ("diffuse", "specular", "raw_diffuse", "raw_specular") + ("color", "taa")[:p.post]
                oa = {o: torch.zeros(out_bytes(form, n), dtype=torch.uint8, device="cuda") for o in names}
                ob = {o: torch.zeros_like(t) for o, t in oa.items()}
                torch.cuda.synchronize()
                alone[k].run(fp, lf, dev, oa)
                fps.append(fp)
                inputs.append(dev)
                outs_a.append(oa)
                outs_b.append(ob)
                idx.append(lf)
            torch.cuda.synchronize()
            if stream is not None:
                with torch.cuda.stream(stream):
                    batch.run([batched[k] for k in active], fps, idx, inputs, outs_b, stream=sh)
                stream.synchronize()
            else:
                batch.run([batched[k] for k in active], fps, idx, inputs, outs_b, stream=0)
            torch.cuda.synchronize()
            for j, k in enumerate(active):
                form = specs[k][2]
                sa, sb = state_of(alone[k], form), state_of(batched[k], form)
                assert sa.keys() == sb.keys()
                for name in sa:
                    assert np.array_equal(sa[name], sb[name]), "frame %d view %d %s differs" % (f, k, name)
                for o in outs_a[j]:
                    assert torch.equal(outs_a[j][o], outs_b[j][o]), "frame %d view %d output %s differs" % (f, k, o)
        return batch.stats(), batch.tile_table() if autotune else None
    finally:
        batch.close()
        for v in alone + batched:
            v.close()
        ctx.close()


def test_batch_matches_alone_with_graphs():
    stats, _ = run_pair(6, graphs=True)
    assert stats["frames"] == 6
    assert stats["graph_captures"] >= 1
    assert stats["graph_replays"] >= 1  # frames 3.. repeat frame 2's launch sequence
    assert stats["last_launches"] < stats["last_jobs"]


def test_batch_matches_alone_default_stream_no_graphs():
    stats, _ = run_pair(4, graphs=False, use_stream=False)
    assert stats["graph_captures"] == 0


def test_batch_chunked_matches_alone():
    # chunks of at most 10k pixels: the larger views run in chunks of their own
    stats, _ = run_pair(4, graphs=True, chunk_pixels=10000)
    assert stats["last_chunks"] >= 4


def test_batch_autotune_keeps_results():
    stats, table = run_pair(12, graphs=True, autotune=True)
    assert table, "tuner saw no 2D pass"
    for name, t in table.items():
        assert tuple(t["tile"]) in [(32, 4), (16, 8), (32, 8), (16, 16), (64, 4)], name
        assert any(v > 0 for v in t["ns_per_kpix"]), name


def test_batch_rejects_bad_calls():
    import torch

    ctx = vg.Context(0)
    v = vg.View(ctx, 16, 8, "ref", vg.params_reference())
    batch = vg.Batch(ctx)
    try:
        sc = vg.Scene(1, 16, 8)
        dev = upload(sc.generate_host(0))
        fp = sc.frame_params(0)
        with pytest.raises(vg.VltError):
            batch.run([v, v], [fp, fp], [0, 0], [dev, dev])  # same view twice
        bad = dict(dev)
        bad.pop("depth")
        with pytest.raises(vg.VltError):
            batch.run([v], [fp], [0], [bad])
        torch.cuda.synchronize()
    finally:
        batch.close()
        v.close()
        ctx.close()
