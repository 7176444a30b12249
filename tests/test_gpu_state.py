"""Export and import of a view's temporal state (vlt_view_export_state /
vlt_view_import_state): a view that imports another view's state mid-sequence must
continue exactly as the exporting view does, in every storage form, through host and
device blobs, with the post passes and in traced mode; mismatched views and damaged
blobs are refused."""
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


def run_frame(view, scene, f, form, n):
    import torch

    dev = upload(scene.generate_host(f))
    out = {k: torch.zeros(OUT_PX[form] * n, dtype=torch.uint8, device="cuda") for k in ("diffuse", "specular")}
    view.run(scene.frame_params(f), f, dev, out)
    return out


@pytest.mark.parametrize("form", ["ref", "f32", "f16"])
@pytest.mark.parametrize("where", ["host", "device"])
def test_imported_view_continues_identically(ctx, form, where):
    import torch

    W, H = 64, 40
    n = W * H
    p = vg.params_reference()
    p.post = 2
    p.hg_log2_buckets = 10
    scene = vg.Scene(21, W, H, disocclusion_frac=0.02)
    a = vg.View(ctx, W, H, form, p)
    b = vg.View(ctx, W, H, form, p)
    try:
        for f in range(3):
            run_frame(a, scene, f, form, n)
        blob = a.export_state() if where == "host" else a.export_state(
            torch.empty(a.state_bytes, dtype=torch.uint8, device="cuda"))
        b.import_state(blob)
        sa, sb = state_of(a), state_of(b)
        assert sa.keys() == sb.keys()
        for k in sa:
            assert np.array_equal(sa[k], sb[k]), "after import: %s" % k
        for f in range(3, 7):
            oa = run_frame(a, scene, f, form, n)
            ob = run_frame(b, scene, f, form, n)
            torch.cuda.synchronize()
            for k in oa:
                assert torch.equal(oa[k], ob[k]), "frame %d output %s" % (f, k)
            sa, sb = state_of(a), state_of(b)
            for k in sa:
                assert np.array_equal(sa[k], sb[k]), "frame %d %s" % (f, k)
    finally:
        a.close()
        b.close()


def test_state_import_refuses_mismatch(ctx):
    W, H = 32, 16
    p = vg.params_reference()
    a = vg.View(ctx, W, H, "f32", p)
    q = vg.params_reference()
    q.atrous_iterations = 4
    others = [vg.View(ctx, W, H, "f32", q), vg.View(ctx, W, H, "ref", p), vg.View(ctx, W + 1, H, "f32", p)]
    try:
        scene = vg.Scene(3, W, H)
        run_frame(a, scene, 0, "f32", W * H)
        blob = a.export_state()
        for o in others:
            padded = np.zeros(max(o.state_bytes, blob.nbytes), np.uint8)
            padded[: blob.nbytes] = blob
            with pytest.raises(vg.VltError):
                o.import_state(padded)
        bad = blob.copy()
        bad[:4] = 0  # magic
        with pytest.raises(vg.VltError):
            a.import_state(bad)
        with pytest.raises(vg.VltError):
            a.import_state(blob[:100])  # too short
        a.import_state(blob)  # the intact blob still loads
    finally:
        a.close()
        for o in others:
            o.close()


def _header_fields():
    """Byte offsets of StateHeader fields (api.cu): six u32, vlt_params, u64 pool
    bytes, u32 frames and flags, eight i32 slot indices, u64 screen-cache offset, then
    the u64 buffer table in ViewBuffers order."""
    import ctypes as C

    pool = (24 + C.sizeof(vg._ffi.Params) + 7) & ~7
    return {"diff_prev": pool + 16, "spec_prev": pool + 20, "prev_den_stride": pool + 40,
            "prev_den_off": pool + 48, "table": pool + 56}


@pytest.mark.parametrize("damage", ["slot_index", "spec_slot_index", "group_offset", "fixed_offset",
                                    "screen_cache", "screen_stride"])
def test_state_import_refuses_damaged_table(ctx, damage):
    W, H = 32, 16
    p = vg.params_reference()
    a = vg.View(ctx, W, H, "ref", p)
    try:
        scene = vg.Scene(3, W, H)
        for f in range(2):
            run_frame(a, scene, f, "ref", W * H)
        blob = a.export_state()
        before = state_of(a)
        hf = _header_fields()
        bad = blob.copy()
        table = bad[hf["table"]:].view(np.uint64)
        if damage == "slot_index":
            bad[hf["diff_prev"]:hf["diff_prev"] + 4].view(np.int32)[0] = 7
        elif damage == "spec_slot_index":
            bad[hf["spec_prev"]:hf["spec_prev"] + 4].view(np.int32)[0] = -1
        elif damage == "group_offset":
            table[0] = table[3]  # diff_rsv[0] pointed at ao[0]: not a permutation of its group
        elif damage == "fixed_offset":
            table[5] += 256  # ao_filtered moved inside the pool
        elif damage == "screen_cache":
            bad[hf["prev_den_off"]:hf["prev_den_off"] + 8].view(np.uint64)[0] = 12345
        else:
            bad[hf["prev_den_stride"]:hf["prev_den_stride"] + 4].view(np.int32)[0] = 3
        with pytest.raises(vg.VltError) as ei:
            a.import_state(bad)
        assert ei.value.status == 1  # VLT_ERR_INVALID_ARG
        assert "state blob" in str(ei.value)
        after = state_of(a)  # a refused blob leaves the view as it was
        for k in before:
            assert np.array_equal(before[k], after[k]), k
        a.import_state(blob)
    finally:
        a.close()


def test_state_export_refused_while_a_traced_frame_is_pending(ctx):
    import torch

    W, H = 16, 8
    p = vg.params_reference()
    p.trace = 1
    v = vg.View(ctx, W, H, "f32", p)
    try:
        scene = vg.Scene(4, W, H)
        dev = upload(scene.generate_host(0))
        rays = {k: torch.zeros(max(v.cache_ray_capacity, W * H) * 32, dtype=torch.uint8, device="cuda")
                for k in ("cache", "diffuse", "spec_validate")}
        v.trace(scene.frame_params(0), 0, dev, rays)
        with pytest.raises(vg.VltError):
            v.export_state()
    finally:
        v.close()
