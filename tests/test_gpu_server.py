"""Serving loop (vlt_server_*): continuous batching of view-sessions.

Sessions arrive over time, are admitted in arrival order as the HBM budget frees
up, and their frames run batched with whatever else is live. Every frame's outputs
must be bit-identical to running the session alone through vlt_frame_run.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import upload

pytestmark = pytest.mark.gpu


def out_bytes(form, n):
    return {"ref": 4, "f32": 16, "f16": 8}[form] * n


def test_server_mix_equals_alone_and_respects_budget():
    import torch

    ctx = vg.Context(0)
    # (arrival step, width, height, form, params, seed, frames)
    plan = [
        (0, 96, 64, "ref", vg.params_reference(), 11, 4),
        (0, 80, 48, "f32", vg.params_plain(0), 12, 5),
        (1, 64, 64, "f32", vg.params_reference(), 13, 3),
        (2, 48, 32, "ref", vg.params_plain(0), 14, 4),
        (6, 72, 40, "f32", vg.params_reference(), 15, 2),
        (7, 56, 40, "f16", vg.params_plain(0), 16, 3),
    ]
    bytes_each = [vg.View.device_bytes(w, h, form, p) for (_, w, h, form, p, _, _) in plan]
    # Room for the two largest sessions only: later arrivals wait for memory.
    budget = sorted(bytes_each)[-1] + sorted(bytes_each)[-2]
    server = vg.Server(ctx, budget)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    sess = {}      # plan index -> session id
    sent = {}      # plan index -> frames submitted
    done = {}      # plan index -> frames completed
    results = {}   # (plan index, frame) -> (diffuse, specular) host bytes
    keep = {}
    scenes = [vg.Scene(seed, w, h, disocclusion_frac=0.02) for (_, w, h, _, _, seed, _) in plan]
    outs = {}
    max_live = 0
    try:
        step = 0
        while len(done) < len(plan) or any(done[k] < plan[k][6] for k in done):
            for k, (arr, w, h, form, p, seed, nf) in enumerate(plan):
                if arr == step and k not in sess:
                    sess[k] = server.open(w, h, form, p)
                    sent[k] = 0
                    done[k] = 0
            # keep one frame queued per open session whose previous frame completed
            for k in sess:
                if sent[k] < plan[k][6] and sent[k] == done[k]:
                    f = sent[k]
                    w, h, form = plan[k][1], plan[k][2], plan[k][3]
                    dev = upload(scenes[k].generate_host(f))
                    o = {x: torch.zeros(out_bytes(form, w * h), dtype=torch.uint8, device="cuda")
                         for x in ("diffuse", "specular")}
                    fp = scenes[k].frame_params(f)
                    torch.cuda.synchronize()
                    keep[(k, f)] = (dev, fp)
                    outs[(k, f)] = o
                    server.submit(sess[k], fp, f, dev, o, tag=(k << 16) | f)
                    sent[k] += 1
                    if sent[k] == plan[k][6]:
                        server.close_session(sess[k])
            with torch.cuda.stream(stream):
                server.step(sh)
            for s_id, tag, lat, step_ms in server.poll(wait=True):
                k, f = tag >> 16, tag & 0xFFFF
                assert lat > 0.0 and step_ms > 0.0
                o = outs.pop((k, f))
                results[(k, f)] = (o["diffuse"].cpu().numpy(), o["specular"].cpu().numpy())
                keep.pop((k, f))
                done[k] += 1
            st = server.stats()
            max_live = max(max_live, st["sessions_live"])
            assert st["bytes_in_use"] <= budget
            step += 1
            assert step < 200, "server made no progress"
        st = server.stats()
        assert st["sessions_closed"] == len(plan)
        assert st["frames_done"] == sum(x[6] for x in plan)
        assert max_live == 2
    finally:
        server.close()

    # The same sessions alone.
    for k, (arr, w, h, form, p, seed, nf) in enumerate(plan):
        view = vg.View(ctx, w, h, form, p)
        sc = vg.Scene(seed, w, h, disocclusion_frac=0.02)
        for f in range(nf):
            dev = upload(sc.generate_host(f))
            o = {x: torch.zeros(out_bytes(form, w * h), dtype=torch.uint8, device="cuda") for x in ("diffuse", "specular")}
            view.run(sc.frame_params(f), f, dev, o)
            torch.cuda.synchronize()
            a_d, a_s = o["diffuse"].cpu().numpy(), o["specular"].cpu().numpy()
            b_d, b_s = results[(k, f)]
            assert np.array_equal(a_d, b_d), "session %d frame %d diffuse differs" % (k, f)
            assert np.array_equal(a_s, b_s), "session %d frame %d specular differs" % (k, f)
        view.close()
    ctx.close()


def test_server_rejects_oversized_session():
    ctx = vg.Context(0)
    server = vg.Server(ctx, 1 << 20)
    try:
        with pytest.raises(vg.VltError):
            server.open(1920, 1080, "f32", vg.params_reference())
    finally:
        server.close()
        ctx.close()
