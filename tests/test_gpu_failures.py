"""Host-side failure paths: device allocations that fail, and sessions closed while
their frames are still queued.

Failures are injected on the host (VLT_FAIL_DEVICE_ALLOC=1 makes the library's
device allocations fail before cudaMalloc is called); no GPU is faulted or
exhausted. A failed view creation must return VLT_ERR_OUT_OF_MEMORY and leave
nothing allocated; a server whose admission fails keeps the session first in line
and admits it once allocation succeeds again; a session closed with frames queued
runs them to completion and is then freed.
"""
import numpy as np
import pytest

import violet_gb300 as vg
from tests.helpers import upload

pytestmark = pytest.mark.gpu

VLT_ERR_OUT_OF_MEMORY = 2
VLT_ERR_BAD_STATE = 6


def _frame(scene, f, n, form="f32"):
    import torch

    ob = {"ref": 4, "f32": 16, "f16": 8}[form]
    dev = upload(scene.generate_host(f))
    out = {k: torch.zeros(ob * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
    return dev, scene.frame_params(f), out


def test_view_create_reports_out_of_memory_and_leaks_nothing(monkeypatch):
    import torch

    ctx = vg.Context(0)
    try:
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        monkeypatch.setenv("VLT_FAIL_DEVICE_ALLOC", "1")
        for form in ("ref", "f32", "f16"):
            with pytest.raises(vg.VltError) as ei:
                vg.View(ctx, 640, 360, form, vg.params_plain(1))
            assert ei.value.status == VLT_ERR_OUT_OF_MEMORY
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, "a failed view creation left device memory allocated"
        monkeypatch.delenv("VLT_FAIL_DEVICE_ALLOC")
        v = vg.View(ctx, 640, 360, "f32", vg.params_plain(1))  # allocation works again
        v.close()
    finally:
        ctx.close()


def test_server_admission_survives_allocation_failure(monkeypatch):
    import torch

    W, H = 96, 64
    n = W * H
    p = vg.params_reference()
    ctx = vg.Context(0)
    server = vg.Server(ctx, 1 << 34)
    scene = vg.Scene(31, W, H, disocclusion_frac=0.02)
    try:
        monkeypatch.setenv("VLT_FAIL_DEVICE_ALLOC", "1")
        sid = server.open(W, H, "f32", p)
        dev, fp, out = _frame(scene, 0, n)
        server.submit(sid, fp, 0, dev, out, tag=7)
        assert server.step() == 0  # admission failed: nothing to run
        st = server.stats()
        assert st["admit_failures"] >= 1 and st["last_admit_status"] == VLT_ERR_OUT_OF_MEMORY
        assert st["sessions_waiting"] == 1 and st["sessions_live"] == 0 and st["bytes_in_use"] == 0
        monkeypatch.delenv("VLT_FAIL_DEVICE_ALLOC")
        assert server.step() == 1  # admitted on the next step, frame issued
        done = server.poll(wait=True)
        assert [d[1] for d in done] == [7]
        got = (out["diffuse"].cpu().numpy(), out["specular"].cpu().numpy())
    finally:
        server.close()
    view = vg.View(ctx, W, H, "f32", p)
    dev, fp, o = _frame(scene, 0, n)
    view.run(fp, 0, dev, o)
    torch.cuda.synchronize()
    assert np.array_equal(o["diffuse"].cpu().numpy(), got[0])
    assert np.array_equal(o["specular"].cpu().numpy(), got[1])
    view.close()
    ctx.close()


def test_session_closed_with_frames_queued_runs_them_then_frees():
    import torch

    W, H = 80, 48
    n = W * H
    p = vg.params_plain(0)
    ctx = vg.Context(0)
    bytes_one = vg.View.device_bytes(W, H, "f32", p)
    server = vg.Server(ctx, bytes_one)  # room for one session: the second waits
    scene = vg.Scene(41, W, H, disocclusion_frac=0.02)
    frames = [_frame(scene, f, n) for f in range(3)]
    try:
        a = server.open(W, H, "f32", p)
        b = server.open(W, H, "f32", p)
        for f, (dev, fp, out) in enumerate(frames):
            server.submit(a, fp, f, dev, out, tag=f)
        server.close_session(a)  # three frames still queued
        with pytest.raises(vg.VltError) as ei:
            server.submit(a, frames[0][1], 3, frames[0][0], None, tag=99)
        assert ei.value.status == VLT_ERR_BAD_STATE
        tags = []
        for _ in range(10):
            server.step()
            tags += [d[1] for d in server.poll(wait=True) if d[0] == a]
            if len(tags) == 3:
                break
        assert tags == [0, 1, 2]
        server.poll(wait=True)
        st = server.stats()
        assert st["sessions_closed"] == 1
        # the closed session's memory went to the waiting one
        assert st["sessions_live"] == 1 and st["sessions_waiting"] == 0 and st["bytes_in_use"] == bytes_one
        results = [(o["diffuse"].cpu().numpy(), o["specular"].cpu().numpy()) for _, _, o in frames]
        server.close_session(b)
        server.step()
        server.poll(wait=True)
        assert server.stats()["sessions_closed"] == 2 and server.stats()["bytes_in_use"] == 0
    finally:
        server.close()
    view = vg.View(ctx, W, H, "f32", p)
    for f in range(3):
        dev, fp, o = _frame(scene, f, n)
        view.run(fp, f, dev, o)
        torch.cuda.synchronize()
        assert np.array_equal(o["diffuse"].cpu().numpy(), results[f][0]), "frame %d" % f
        assert np.array_equal(o["specular"].cpu().numpy(), results[f][1]), "frame %d" % f
    view.close()
    ctx.close()
