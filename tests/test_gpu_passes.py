"""GPU parity of every per-pass C-ABI entry point (the drop-in replacements of the
reference's individual render-graph nodes) against the oracle's per-pass functions.

Inputs: frame 3 of a seeded scene, with the resident state (reservoirs, AO and
denoiser history, hash grid) of an oracle view that has run frames 0..2, so every
pass sees realistic history. Outputs are compared bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import violet_gb300 as vg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

W, H = 96, 64
N = W * H
V = C.c_void_p


def vp(x):
    return V(x) if isinstance(x, int) else V(x.data_ptr() if x is not None else None)


@pytest.fixture(scope="module")
def world():
    import torch  # noqa: F401

    P = vg.params_reference()
    scene = vg.Scene(31, W, H, disocclusion_frac=0.05)
    ov = po.OracleView(W, H, P)
    frames = []
    for f in range(3):
        h = scene.generate_host(f)
        ov.run(scene.frame_params(f), f, h)
        frames.append(h)
    h3 = scene.generate_host(3)
    state = {k: ov.buffer(k) for k in ("diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance",
                                       "ao_history", "hist_color", "hist_moments", "hist_len", "raw_diffuse",
                                       "raw_specular", "spec_ray_len", "hg_storage", "hg_decay")}
    ov.close()
    return {"P": P, "fp": scene.frame_params(3), "prev": frames[2], "cur": h3, "state": state}


_KEEP = []  # device copies stay alive for the module: a freed temporary's block would be reused


def D(a):
    """numpy -> device tensor (bytes)."""
    import torch

    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()
    _KEEP.append(t)
    return t


def Z(nbytes):
    import torch

    return torch.zeros(max(int(nbytes), 16), dtype=torch.uint8, device="cuda")


def back(t, nbytes, dtype=np.uint8):
    import torch

    torch.cuda.synchronize()
    return t[:nbytes].cpu().numpy().view(dtype)


def host(nbytes, dtype=np.uint8):
    return np.zeros(nbytes, np.uint8).view(dtype)


def same(got, exp, what):
    got = np.asarray(got).reshape(-1)
    exp = np.asarray(exp).reshape(-1)
    bad = np.nonzero(got != exp)[0]
    assert bad.size == 0, "%s: %d mismatches, first at %d: 0x%x vs 0x%x" % (what, bad.size, bad[0], int(got[bad[0]]),
                                                                          int(exp[bad[0]]))


def u8(a):
    return np.ascontiguousarray(a).view(np.uint8).reshape(-1)


@pytest.mark.parametrize("has_new", [1, 0])
def test_diff_temporal_and_spatial(world, has_new):
    lib, ol = vg.lib(), po.lib()
    P, fp, prev, cur, st = world["P"], world["fp"], world["prev"], world["cur"], world["state"]
    out_o = host(16 * N, np.uint32)
    ol.vlto_ind_diff_temporal_resample(C.byref(fp), W, H, C.byref(P), po.ptr(prev["depth"]), po.ptr(cur["depth"]),
                                       po.ptr(cur["diff_hit_pos_normal"]), po.ptr(cur["diff_hit_radiance"]),
                                       po.ptr(cur["diff_source_pdf"]), po.ptr(st["diff_reservoir"]), po.ptr(out_o),
                                       777, 1, has_new)
    out_g = Z(16 * N)
    rc = lib.vlt_ind_diff_temporal_resample(C.byref(fp), W, H, C.byref(P), vp(D(prev["depth"])), vp(D(cur["depth"])),
                                            vp(D(cur["diff_hit_pos_normal"])), vp(D(cur["diff_hit_radiance"])),
                                            vp(D(cur["diff_source_pdf"])), vp(D(st["diff_reservoir"])), vp(out_g), 777,
                                            1, has_new, None)
    assert rc == 0
    same(back(out_g, 16 * N, np.uint32), out_o, "diff temporal")
    # spatial on top of the temporal result
    ao = st["ao_history"].view(np.uint32)
    aof_o = host(2 * N, np.uint16)
    ol.vlto_ao_filter(W, H, po.ptr(cur["depth"]), po.ptr(ao), po.ptr(aof_o))
    sp_o, li_o = host(16 * N, np.uint32), host(4 * N, np.uint32)
    ol.vlto_ind_diff_spatial_resample(C.byref(fp), W, H, C.byref(P), po.ptr(cur["gbuffer"]), po.ptr(cur["depth"]),
                                      po.ptr(aof_o), po.ptr(out_o), po.ptr(sp_o), po.ptr(li_o), 4242)
    sp_g, li_g = Z(16 * N), Z(4 * N)
    rc = lib.vlt_ind_diff_spatial_resample(C.byref(fp), W, H, C.byref(P), vp(D(cur["gbuffer"])), vp(D(cur["depth"])),
                                           vp(D(aof_o)), vp(out_g), vp(sp_g), vp(li_g), 4242, None)
    assert rc == 0
    same(back(sp_g, 16 * N, np.uint32), sp_o, "diff spatial reservoir")
    same(back(li_g, 4 * N, np.uint32), li_o, "diff spatial lighting")


@pytest.mark.parametrize("has_new,has_prev", [(1, 1), (0, 1), (1, 0)])
def test_ao_gen_and_filter(world, has_new, has_prev):
    lib, ol = vg.lib(), po.lib()
    fp, cur, st = world["fp"], world["cur"], world["state"]
    prev_ao = st["ao_history"].view(np.uint32)
    ao_o = host(4 * N, np.uint32)
    ol.vlto_ao_gen(C.byref(fp), W, H, po.ptr(cur["diff_hit_pos_normal"]), po.ptr(cur["depth"]), po.ptr(prev_ao),
                   po.ptr(ao_o), has_new, has_prev, C.c_float(2.0))
    ao_g = Z(4 * N)
    rc = lib.vlt_ao_gen(C.byref(fp), W, H, vp(D(cur["diff_hit_pos_normal"])), vp(D(cur["depth"])), vp(D(prev_ao)),
                        vp(ao_g), has_new, has_prev, C.c_float(2.0), None)
    assert rc == 0
    same(back(ao_g, 4 * N, np.uint32), ao_o, "ao gen")
    f_o = host(2 * N, np.uint16)
    ol.vlto_ao_filter(W, H, po.ptr(cur["depth"]), po.ptr(ao_o), po.ptr(f_o))
    f_g = Z(2 * N)
    assert lib.vlt_ao_filter(W, H, vp(D(cur["depth"])), vp(ao_g), vp(f_g), None) == 0
    same(back(f_g, 2 * N, np.uint16), f_o, "ao filter")


@pytest.mark.parametrize("chain", [False, True])
def test_spec_temporal_and_spatial(world, chain):
    lib, ol = vg.lib(), po.lib()
    P, fp, prev, cur, st = world["P"], world["fp"], world["prev"], world["cur"], world["state"]
    rs_o, hp_o, rd_o = host(8 * N, np.uint32), host(16 * N, np.float32), host(4 * N, np.uint32)
    ol.vlto_ind_spec_temporal_resample(C.byref(fp), W, H, C.byref(P), po.ptr(prev["depth"]), po.ptr(prev["gbuffer"]),
                                       po.ptr(cur["depth"]), po.ptr(cur["gbuffer"]),
                                       po.ptr(st["spec_reservoir"].view(np.uint32)),
                                       po.ptr(st["spec_hit_pos"].view(np.float32)),
                                       po.ptr(st["spec_radiance"].view(np.uint32)), po.ptr(cur["spec_hit_pos"]),
                                       po.ptr(cur["spec_hit_radiance"]), po.ptr(rs_o), po.ptr(hp_o), po.ptr(rd_o),
                                       99, 1)
    rs_g, hp_g, rd_g = Z(8 * N), Z(16 * N), Z(4 * N)
    rc = lib.vlt_ind_spec_temporal_resample(C.byref(fp), W, H, C.byref(P), vp(D(prev["depth"])),
                                            vp(D(prev["gbuffer"])), vp(D(cur["depth"])), vp(D(cur["gbuffer"])),
                                            vp(D(st["spec_reservoir"])), vp(D(st["spec_hit_pos"])),
                                            vp(D(st["spec_radiance"])), vp(D(cur["spec_hit_pos"])),
                                            vp(D(cur["spec_hit_radiance"])), vp(rs_g), vp(hp_g), vp(rd_g), 99, 1, None)
    assert rc == 0
    same(back(rs_g, 8 * N, np.uint32), rs_o, "spec temporal reservoir")
    same(back(hp_g, 16 * N, np.uint32), hp_o.view(np.uint32), "spec temporal hit pos")
    same(back(rd_g, 4 * N, np.uint32), rd_o, "spec temporal radiance")
    li_o, rl_o = host(4 * N, np.uint32), host(2 * N, np.uint16)
    ors, ohp, ord_ = (host(8 * N, np.uint32), host(16 * N, np.float32), host(4 * N, np.uint32)) if chain else (
        None, None, None)
    ol.vlto_ind_spec_spatial_resample(C.byref(fp), W, H, C.byref(P), po.ptr(cur["gbuffer"]), po.ptr(cur["depth"]),
                                      po.ptr(rs_o), po.ptr(hp_o), po.ptr(rd_o), po.ptr(li_o), po.ptr(rl_o),
                                      po.ptr(ors), po.ptr(ohp), po.ptr(ord_), 5)
    li_g, rl_g = Z(4 * N), Z(2 * N)
    grs, ghp, grd = (Z(8 * N), Z(16 * N), Z(4 * N)) if chain else (None, None, None)
    rc = lib.vlt_ind_spec_spatial_resample(C.byref(fp), W, H, C.byref(P), vp(D(cur["gbuffer"])), vp(D(cur["depth"])),
                                           vp(rs_g), vp(hp_g), vp(rd_g), vp(li_g), vp(rl_g), vp(grs), vp(ghp),
                                           vp(grd), 5, None)
    assert rc == 0
    same(back(li_g, 4 * N, np.uint32), li_o, "spec spatial lighting")
    same(back(rl_g, 2 * N, np.uint16), rl_o, "spec spatial ray length")
    if chain:
        same(back(grs, 8 * N, np.uint32), ors, "spec spatial reservoir")
        same(back(ghp, 16 * N, np.uint32), ohp.view(np.uint32), "spec spatial hit pos")
        same(back(grd, 4 * N, np.uint32), ord_, "spec spatial radiance")


@pytest.mark.parametrize("fast", [0, 1])
def test_denoiser_passes(world, fast):
    lib, ol = vg.lib(), po.lib()
    P, fp, prev, cur, st = world["P"], world["fp"], world["prev"], world["cur"], world["state"]
    hc, hm, hl = st["hist_color"].view(np.uint32), st["hist_moments"].view(np.uint32), st["hist_len"]
    fast_hist = np.ascontiguousarray(hc[::-1])  # any plausible colour history
    c_o, m_o, l_o, f_o = host(8 * N, np.uint32), host(4 * N, np.uint32), host(N), host(8 * N, np.uint32)
    ol.vlto_denoise_temporal(C.byref(fp), W, H, C.byref(P), po.ptr(cur["depth"]), po.ptr(cur["gbuffer"]),
                             po.ptr(st["raw_diffuse"].view(np.uint32)), po.ptr(st["raw_specular"].view(np.uint32)),
                             po.ptr(st["spec_ray_len"].view(np.uint16)), po.ptr(prev["depth"]),
                             po.ptr(prev["gbuffer"]), po.ptr(hc), po.ptr(hm), po.ptr(hl), po.ptr(fast_hist),
                             po.ptr(c_o), po.ptr(m_o), po.ptr(l_o), po.ptr(f_o), 1, fast)
    c_g, m_g, l_g, f_g = Z(8 * N), Z(4 * N), Z(N), Z(8 * N)
    rc = lib.vlt_denoise_temporal(C.byref(fp), W, H, C.byref(P), vp(D(cur["depth"])), vp(D(cur["gbuffer"])),
                                  vp(D(st["raw_diffuse"])), vp(D(st["raw_specular"])), vp(D(st["spec_ray_len"])),
                                  vp(D(prev["depth"])), vp(D(prev["gbuffer"])), vp(D(hc)), vp(D(hm)), vp(D(hl)),
                                  vp(D(fast_hist)), vp(c_g), vp(m_g), vp(l_g), vp(f_g), 1, fast, None)
    assert rc == 0
    same(back(c_g, 8 * N, np.uint32), c_o, "dn temporal colour")
    same(back(m_g, 4 * N, np.uint32), m_o, "dn temporal moments")
    same(back(l_g, N), l_o, "dn temporal history length")
    if fast:
        same(back(f_g, 8 * N, np.uint32), f_o, "dn temporal fast history")
    # disocclusion fix
    fc_o, fm_o = host(8 * N, np.uint32), host(4 * N, np.uint32)
    ol.vlto_denoise_disocclusion_fix(W, H, po.ptr(cur["depth"]), po.ptr(cur["gbuffer"]), po.ptr(l_o), po.ptr(c_o),
                                     po.ptr(m_o), po.ptr(fc_o), po.ptr(fm_o))
    fc_g, fm_g = Z(8 * N), Z(4 * N)
    assert lib.vlt_denoise_disocclusion_fix(W, H, vp(D(cur["depth"])), vp(D(cur["gbuffer"])), vp(l_g), vp(c_g),
                                            vp(m_g), vp(fc_g), vp(fm_g), None) == 0
    same(back(fc_g, 8 * N, np.uint32), fc_o, "dn fix colour")
    same(back(fm_g, 4 * N, np.uint32), fm_o, "dn fix moments")
    assert (l_o > 0).any() and (l_o < 4).any(), "test input should contain short-history pixels"
    if fast:
        ol.vlto_denoise_fast_history_clamp(W, H, po.ptr(f_o), po.ptr(fc_o))
        assert lib.vlt_denoise_fast_history_clamp(W, H, vp(f_g), vp(fc_g), None) == 0
        same(back(fc_g, 8 * N, np.uint32), fc_o, "dn fast clamp")
    # fallback / variance
    bc_o, v_o = host(8 * N, np.uint32), host(4 * N, np.uint32)
    ol.vlto_denoise_spatial_fallback(W, H, po.ptr(cur["depth"]), po.ptr(cur["gbuffer"]), po.ptr(l_o), po.ptr(fc_o),
                                     po.ptr(fm_o), po.ptr(bc_o), po.ptr(v_o))
    bc_g, v_g = Z(8 * N), Z(4 * N)
    assert lib.vlt_denoise_spatial_fallback(W, H, vp(D(cur["depth"])), vp(D(cur["gbuffer"])), vp(l_g), vp(fc_g),
                                            vp(fm_g), vp(bc_g), vp(v_g), None) == 0
    same(back(bc_g, 8 * N, np.uint32), bc_o, "dn fallback colour")
    same(back(v_g, 4 * N, np.uint32), v_o, "dn fallback variance")
    # a-trous at two step sizes
    for step in (1, 4):
        ac_o, av_o = host(8 * N, np.uint32), host(4 * N, np.uint32)
        ol.vlto_denoise_atrous(W, H, po.ptr(cur["depth"]), po.ptr(cur["gbuffer"]), po.ptr(bc_o), po.ptr(v_o),
                               po.ptr(ac_o), po.ptr(av_o), step)
        ac_g, av_g = Z(8 * N), Z(4 * N)
        assert lib.vlt_denoise_atrous(W, H, vp(D(cur["depth"])), vp(D(cur["gbuffer"])), vp(bc_g), vp(v_g), vp(ac_g),
                                      vp(av_g), step, None) == 0
        same(back(ac_g, 8 * N, np.uint32), ac_o, "a-trous colour (step %d)" % step)
        same(back(av_g, 4 * N, np.uint32), av_o, "a-trous variance (step %d)" % step)


def test_hash_grid_passes(world):
    import torch

    lib, ol = vg.lib(), po.lib()
    P, fp, cur, st = world["P"], world["fp"], world["cur"], world["state"]
    lb, mq = P.hg_log2_buckets, P.hg_max_queries
    nc = 16 << lb
    storage = st["hg_storage"].view(np.uint32).copy()
    decay = st["hg_decay"].copy()
    # decay
    ol.vlto_hg_decay(lb, po.ptr(decay), po.ptr(storage))
    s_g, d_g = D(st["hg_storage"]), D(st["hg_decay"])
    assert lib.vlt_hg_decay(lb, vp(d_g), vp(s_g), None) == 0
    same(back(s_g, 16 * nc, np.uint32), storage, "hg decay storage")
    same(back(d_g, nc), decay, "hg decay bytes")
    # emission
    q_o, qc_o = host(32 * mq, np.uint32), host(4, np.uint32)
    ol.vlto_hg_emit_queries(C.byref(fp), W, H, lb, 0, mq, po.ptr(cur["depth"]), po.ptr(cur["diff_hit_pos_normal"]),
                            po.ptr(cur["diff_hit_radiance"]), po.ptr(q_o), po.ptr(qc_o))
    q_g, qc_g = Z(32 * mq), Z(4)
    assert lib.vlt_hg_emit_queries(C.byref(fp), W, H, lb, 0, mq, vp(D(cur["depth"])),
                                   vp(D(cur["diff_hit_pos_normal"])), vp(D(cur["diff_hit_radiance"])), vp(q_g),
                                   vp(qc_g), None) == 0
    same(back(qc_g, 4, np.uint32), qc_o, "hg query count")
    same(back(q_g, 32 * N, np.uint32), q_o[: 8 * N], "hg queries")
    # a query buffer that is not 32-byte aligned takes the 16-byte store path
    q_u = Z(32 * mq + 16)
    assert lib.vlt_hg_emit_queries(C.byref(fp), W, H, lb, 0, mq, vp(D(cur["depth"])),
                                   vp(D(cur["diff_hit_pos_normal"])), vp(D(cur["diff_hit_radiance"])),
                                   C.c_void_p(q_u.data_ptr() + 16), vp(qc_g), None) == 0
    same(back(q_u[16:], 32 * N, np.uint32), q_o[: 8 * N], "hg queries (unaligned buffer)")
    # select
    sel_o = host(4 * nc, np.uint32)
    ol.vlto_hg_query_select(lb, mq, po.ptr(q_o), po.ptr(qc_o), po.ptr(storage), po.ptr(sel_o), 0xC0FFEE)
    sel_g = Z(4 * nc)
    scratch = Z(lib.vlt_hg_select_scratch_bytes(lb, mq))
    assert lib.vlt_hg_query_select(lb, mq, vp(q_g), vp(qc_g), vp(s_g), vp(sel_g), 0xC0FFEE, vp(scratch), None) == 0
    same(back(s_g, 16 * nc, np.uint32), storage, "hg select storage")
    same(back(sel_g, 4 * nc, np.uint32), sel_o, "hg selection")
    # compact (order unspecified: compare as sets)
    nmax = min(mq, nc)
    idx_o, adr_o, cnt_o = host(4 * nmax, np.uint32), host(4 * nmax, np.uint32), host(4, np.uint32)
    ol.vlto_hg_query_compact(lb, mq, po.ptr(sel_o), po.ptr(idx_o), po.ptr(adr_o), po.ptr(cnt_o))
    idx_g, adr_g, cnt_g = Z(4 * nmax), Z(4 * nmax), Z(4)
    assert lib.vlt_hg_query_compact(lb, mq, vp(sel_g), vp(idx_g), vp(adr_g), vp(cnt_g), None) == 0
    n = int(cnt_o[0])
    assert int(back(cnt_g, 4, np.uint32)[0]) == n and n > 0
    go = sorted(zip(back(adr_g, 4 * n, np.uint32).tolist(), back(idx_g, 4 * n, np.uint32).tolist()))
    oo = sorted(zip(adr_o[:n].tolist(), idx_o[:n].tolist()))
    assert go == oo, "hg compact sets differ"
    # update (from the GPU's own compacted order)
    ol.vlto_hg_update(po.ptr(q_o), po.ptr(idx_o), po.ptr(adr_o), po.ptr(cnt_o), po.ptr(storage), po.ptr(decay))
    assert lib.vlt_hg_update(mq, vp(q_g), vp(idx_g), vp(adr_g), vp(cnt_g), vp(s_g), vp(d_g), None) == 0
    same(back(s_g, 16 * nc, np.uint32), storage, "hg update storage")
    same(back(d_g, nc), decay, "hg update decay")
    # find: positions/normals of every 7th query
    qs = q_o[: 8 * N].reshape(-1, 8)[::7]
    pos = np.ascontiguousarray(qs[:, :3]).view(np.float32).reshape(-1)
    nrm = np.zeros((qs.shape[0], 3), np.float32)
    nrm[:, 2] = 1.0
    nrm = nrm.reshape(-1)
    m = qs.shape[0]
    a_o, r_o = host(4 * m, np.uint32), host(16 * m, np.float32)
    ol.vlto_hg_find(C.byref(fp), lb, 0, po.ptr(storage), m, po.ptr(pos), po.ptr(nrm), po.ptr(a_o), po.ptr(r_o))
    a_g, r_g = Z(4 * m), Z(16 * m)
    assert lib.vlt_hg_find(C.byref(fp), lb, 0, vp(s_g), m, vp(D(pos)), vp(D(nrm)), vp(a_g), vp(r_g), None) == 0
    same(back(a_g, 4 * m, np.uint32), a_o, "hg find address")
    same(back(r_g, 16 * m, np.uint32), r_o.view(np.uint32), "hg find radiance")
    assert (a_o != 0xFFFFFFFF).mean() > 0.5
    torch.cuda.synchronize()
