#!/usr/bin/env python3
"""Throughput of the full ReSTIR GI + ReLAX + hash-grid-update frame on GB300.

Workload: one 1920x1080 view, seeded synthetic scene with 2% disocclusion pixels per
frame, plain-method knobs (temporal M cap 20, two spatial passes of 8 taps at 16 px
for diffuse and specular, 32-frame history, 5 a-trous iterations, 2^22-cell hash
grid keyed by position and normal octant with one query per pixel), FP32 storage
form (VLT_FORM_F32: float reservoirs, AO, lighting and denoiser records), binary32
arithmetic. A step is one frame of that view. The reference-storage-form
(R11G11B10/half/M8W24 records) throughput of the same frames is reported beside it.

  value : Mpix/s with every frame's inputs already resident in HBM (CUDA events on
          the launching stream around exactly --steps frames; frames are distinct and
          each frame's inputs plus resident state exceed the 129 MB L2);
  e2e   : the same through the public C ABI with host inputs: per step the frame's
          inputs are copied from pinned host memory and the denoised outputs read
          back, inside the timed region (a copy stream overlaps frame f+2's upload
          and frame f's read-back with frame f+1's compute);
  roofline: the dominant pass (per-pass CUDA-event timers of the library) against
          the measured HBM copy bandwidth; issue_roofline: the same launch against
          the SMs' warp-instruction issue rate (the bound of that pass);
  cpu_baseline: the CPU oracle (restatement of the reference's passes) on the
          host cores, on a bounded sample of the same workload.

`--impl reference` times the reference's algorithm on the host cores instead (the
reference itself is HLSL + a Rust/Vulkan host and cannot run on this machine; its
CPU restatement is the stand-in). Under torchrun each rank runs an independent
replica (the path does not shard within a view); rank 0 prints one JSON line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpix/s full ReSTIR GI+ReLAX frame, batched vs plain, rel-L2≤1e-3; p99 frame ms"
W_DEFAULT, H_DEFAULT = 1920, 1080
WORKLOAD = "restir_gi_relax_hashgrid_1920x1080_plain"

# Algorithmic bytes per pixel (per cell for hg_decay/hg_compact) of each pass:
# inputs read once + outputs written once, counted from the record layouts of
# include/vlt.h (unused G-buffer layers are not counted; the per-frame surface planes
# are an implementation choice and count as the G-buffer/depth reads they replace).
PASS_BYTES_PER_PIXEL_REF = {
    "surface": 4 + 12 + 48,
    "hg_emit": 16 + 32,
    "hg_select": 32 + 4,
    "hg_update": 4 + 16 + 16 + 1,
    "ao_gen": 8 + 4 + 4 + 4,
    "ao_filter": 4 + 4 + 2,
    "diff_temporal": 4 + 4 + 8 + 4 + 4 + 16 + 16,
    "diff_spatial": 4 + 4 + 2 + 16 + 16 + 4,
    "spec_temporal": 4 + 4 + 8 + 8 + 28 + 20 + 28,
    "spec_spatial": 4 + 8 + 28 + 28,
    "dn_temporal": 4 + 8 + 4 + 4 + 2 + 4 + 4 + 8 + 4 + 1 + 8 + 4 + 1,
    "dn_fix": 1 + 8 + 4 + 8 + 4,
    "dn_fallback": 1 + 8 + 4 + 8 + 4,
    "dn_fast_clamp": 8 + 8 + 8,
    "dn_atrous": 4 + 4 + 4 + 8 + 4 + 8 + 4,
    # G-buffer layers 0, 1, 3 + R8 shadow + diffuse + specular + colour
    "final_lighting": 12 + 1 + 4 + 4 + 4,
    # depth + source + history (each read once) + next history
    "taa": 4 + 4 + 4 + 4,
}
# FP32 form: float2 AO history, float filtered AO, 48-byte diffuse records, float4
# lighting, 32-byte denoiser records {diffuse.rgb|aux, specular.rgb|aux}, float
# history length.
PASS_BYTES_PER_PIXEL_F32 = dict(
    PASS_BYTES_PER_PIXEL_REF,
    ao_gen=8 + 4 + 8 + 8,
    ao_filter=4 + 8 + 4,
    diff_temporal=4 + 4 + 8 + 4 + 4 + 48 + 48,
    diff_spatial=4 + 4 + 4 + 48 + 48 + 16,
    dn_temporal=4 + 8 + 16 + 16 + 4 + 4 + 32 + 4 + 32 + 4,
    dn_fix=4 + 32 + 32,
    dn_fast_clamp=32 + 32 + 32,
    dn_fallback=4 + 32 + 32,
    dn_atrous=4 + 4 + 4 + 32 + 32,
    final_lighting=12 + 1 + 16 + 16 + 16,
    taa=4 + 16 + 16 + 16,
)
PASS_BYTES_PER_PIXEL = {"ref": PASS_BYTES_PER_PIXEL_REF, "f32": PASS_BYTES_PER_PIXEL_F32}

# The whole frame's fused minimum per pixel (each input read once, each piece of
# persistent state read once and written once, each output written once), from the
# record layouts: inputs depth 4 + G-buffer 16 + previous depth 4 + previous G-buffer
# 16 + diffuse candidate 12 + its source pdf 4 + specular candidate 20 = 76; state
# (read + write) diffuse reservoir 48 (f32) / 17 (f16), specular reservoir 28 / 24, AO
# history 8 / 4, denoiser history record + length 33 / 17; outputs (diffuse +
# specular) 32 / 16. Hash grid per frame: the decay bytes read and written (2 per
# cell) plus 37 bytes per updated cell (cell radiance 12 read and 12 written, decay
# byte 1, the query's radiance 12 read).
FRAME_BYTES_PER_PIXEL = {"f32": 76 + 2 * (48 + 28 + 8 + 33) + 32, "f16": 76 + 2 * (17 + 24 + 4 + 17) + 16}
FRAME_BYTES_PER_CELL = 2
FRAME_BYTES_PER_UPDATED_CELL = 37
FORM = "f32"
PASS_BYTES_PER_CELL = {"hg_decay": 2, "hg_compact": 4}
# DRAM bytes per launch unit measured with ncu at 960x540, f32 (dram__bytes_read.sum +
# dram__bytes_write.sum; the a-trous from one-pass counters, profiles/dn_atrous_f32_540p.md;
# the specular spatial pass from its --set full capture, mean of its two launches,
# profiles/spec_spatial_f32_540p.md).
MEASURED_TRAFFIC_PER_UNIT = {"dn_atrous": 64.25, "spec_spatial": (36.013e6 + 0.507e6 + 34.377e6 + 0.322e6) / 2 / (960 * 540)}
# Warp instructions per launch unit measured with ncu (smsp__inst_executed.sum of a
# --set full capture / pixels, mean of two launches): the issue roofline of a pass
# that is bound by instruction issue or latency rather than by HBM.
MEASURED_WARP_INSTRUCTIONS_PER_UNIT = {"dn_atrous": (20.716e6 + 20.666e6) / 2 / (960 * 540),
                                       "spec_spatial": (40.168e6 + 43.590e6) / 2 / (960 * 540)}
ISSUE_SLOTS_PER_SM_CLOCK = 4  # one warp instruction per scheduler per clock, 4 schedulers per SM


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        import torch

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, ws, device=None):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# The knobs of the plain 1920x1080 workload (vlt_params_plain(1)); kept here as values
# so that the CPU reference arm builds them without loading the product library
# (tests/test_scene.py checks them against the library's preset).
WORKLOAD_KNOBS = {
    "diff_m_cap": 20, "spec_m_cap": 20, "use_input_pdf": 1, "diff_spatial_passes": 2, "diff_spatial_taps": 8,
    "diff_spatial_radius_px": 16.0, "spec_spatial_passes": 2, "spec_spatial_taps": 8, "spec_spatial_radius_px": 16.0,
    "ao_radius": 2.0, "denoise": 1, "disocclusion_fix": 1, "fast_history_clamp": 0, "atrous_iterations": 5,
    "history_max_frames": 32.0, "hg_enable": 1, "hg_decay": 1, "hg_log2_buckets": 18, "hg_key_mode": 1,
    "hg_max_queries": 0, "post": 0, "trace": 0, "diff_validate": 0, "spec_validate": 0,
}


def workload_params(vg):
    return vg.params_plain(1)


def workload_params_struct():
    from violet_gb300 import _ffi

    p = _ffi.Params()
    for k, v in WORKLOAD_KNOBS.items():
        setattr(p, k, v)
    return p


def input_bytes_per_pixel(vg, params):
    import numpy as np

    return sum(np.dtype(dt).itemsize * c for k, (dt, c) in vg.FRAME_BUFFERS.items()
               if k != "shadow_mask" or params.post >= 1)


def input_buffers(vg, params, w, h, dev):
    """Device buffers for one frame's inputs (the shadow mask only when the final
    lighting runs)."""
    import numpy as np
    import torch

    return {k: torch.empty(w * h * c * np.dtype(dt).itemsize, dtype=torch.uint8, device=dev)
            for k, (dt, c) in vg.FRAME_BUFFERS.items() if k != "shadow_mask" or params.post >= 1}


def cpu_sample(width, height, frames, seed, threads=None):
    """Times the CPU oracle on `frames` frames of the workload; returns (Mpix/s of
    frames 1.., threads used)."""
    import numpy as np  # noqa: F401

    import violet_gb300 as vg
    from oracle import pyoracle as po

    if threads:
        po.set_threads(threads)
    params = workload_params(vg)
    scene = vg.Scene(seed, width, height, disocclusion_frac=0.02)
    ov = po.OracleView(width, height, params, FORM)
    times = []
    for f in range(frames):
        host = scene.generate_host(f)
        fp = scene.frame_params(f)
        t0 = time.perf_counter()
        ov.run(fp, f, host)
        times.append(time.perf_counter() - t0)
    ov.close()
    steady = times[1:] if len(times) > 1 else times
    return width * height * len(steady) / sum(steady) / 1e6, po.threads(), times


def run_reference(args, ws, rank):
    """The reference's algorithm on the host cores: the CPU restatement of its passes
    (the oracle, all host threads), on the same 1920x1080 workload as the GPU arm (same
    scene seed, knobs and frames), one frame per step. The frames are synthesised by
    the oracle's host build of the scene generator, outside the timed spans; only the
    restatement's frame calls are timed. This process loads the oracle's libraries
    only."""
    if rank != 0:
        return
    from oracle import pyoracle as po
    from oracle import pyscene

    W, H = args.width, args.height
    params = workload_params_struct()
    scene = pyscene.Scene(1000, W, H, disocclusion_frac=0.02)
    ov = po.OracleView(W, H, params, FORM)
    out = {k: np.zeros(16 * W * H, np.uint8) for k in ("diffuse", "specular")}
    for f in range(args.warmup):
        ov.run(scene.frame_params(f), f, scene.generate_host(f), out)
    total = 0.0
    for k in range(args.steps):
        f = args.warmup + k
        host, fp = scene.generate_host(f), scene.frame_params(f)
        t0 = time.perf_counter()
        ov.run(fp, f, host, out)
        total += time.perf_counter() - t0
    ov.close()
    value = args.steps * W * H / total / 1e6
    cores = po.threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "storage": FORM,
                   "parallelism": "single view", "knobs": dict(WORKLOAD_KNOBS)},
        "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": cores, "kind": "port",
                         "sample": "%d frames of the %dx%d workload after %d warm-up frames (frame synthesis not "
                                   "timed)" % (args.steps, W, H, args.warmup)},
        "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference runs HLSL through DXC/Vulkan from a Rust host; neither a Vulkan stack nor cargo "
                "exists on this machine, so its passes run as the CPU restatement (checked bit for bit against "
                "the reference's shaders compiled as C++) on all host threads",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch

    import violet_gb300 as vg

    vg.lib()  # raises if libvlt.so is missing: there is no fallback path
    assert torch.cuda.is_available(), "bench.py needs a GPU"
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    W, H = args.width, args.height
    n = W * H
    params = workload_params(vg)
    scene = vg.Scene(1000 + rank, W, H, disocclusion_frac=0.02)
    nframes = args.warmup + args.steps
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    # Distinct frames, generated on the device and kept resident in HBM.
    frames, fps = [], []
    for f in range(nframes):
        bufs = input_buffers(vg, params, W, H, dev)
        scene.generate_device(f, bufs, sh)
        frames.append(bufs)
        fps.append(scene.frame_params(f))
    out_px = 16 if FORM == "f32" else 4
    out = {k: torch.empty(n * out_px, dtype=torch.uint8, device=dev) for k in ("diffuse", "specular")}
    ctx = vg.Context(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def device_resident(form, o, clocks=None):
        """Warm-up frames, then exactly --steps timed frames; returns (ms, launches)."""
        v = vg.View(ctx, W, H, form, params)
        for f in range(args.warmup):
            v.run(fps[f], f, frames[f], o, sh)
        torch.cuda.synchronize()
        barrier(ws)
        if clocks:
            clocks.start()
            time.sleep(0.3)
        nl = 0
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(args.steps):
            f = args.warmup + k
            v.run(fps[f], f, frames[f], o, sh)
            nl += v.launches
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1)
        barrier(ws)
        v.close()
        return max_over_ranks(t, ws, dev), nl

    # ---- device-resident throughput of the reference storage form (side figure)
    out_ref = {k: torch.empty(n * 4, dtype=torch.uint8, device=dev) for k in ("diffuse", "specular")}
    ms_ref, _ = device_resident("ref", out_ref)
    value_ref = ws * args.steps * n / (ms_ref / 1e3) / 1e6
    del out_ref

    # ---- device-resident throughput (headline)
    clocks = ClockSampler(local)
    ms, launches = device_resident(FORM, out, clocks)
    clk = clocks.stop()
    value = ws * args.steps * n / (ms / 1e3) / 1e6
    view = vg.View(ctx, W, H, FORM, params)

    # ---- the same frames as one pipelined sequence (vlt_frames_run: frame f's
    # denoiser beside frame f + 1's resampling passes), device-resident
    pipelined = None
    if not args.no_pipelined:
        pv = vg.View(ctx, W, H, FORM, params)
        outs_p = [out] * nframes  # every frame writes the same output buffers, as above
        warm = vg.FrameSequence(fps[:args.warmup], list(range(args.warmup)), frames[:args.warmup],
                                outs_p[:args.warmup])
        timed = vg.FrameSequence(fps[args.warmup:], list(range(args.warmup, nframes)), frames[args.warmup:],
                                 outs_p[args.warmup:])
        pv.run_sequence(warm, sh)
        torch.cuda.synchronize()
        barrier(ws)
        e0.record(stream)
        pv.run_sequence(timed, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_p = max_over_ranks(e0.elapsed_time(e1), ws, dev)
        barrier(ws)
        pipelined = {"value": ws * args.steps * n / (ms_p / 1e3) / 1e6, "unit": "Mpix/s",
                     "ms_per_step": ms_p / args.steps, "launches": pv.launches,
                     "definition": "the same --steps frames as one vlt_frames_run call after --warmup frames "
                                   "in another; results equal frame-by-frame vlt_frame_run"}
        pv.close()

    # ---- per-pass timers (separate run: the event records cost a little time)
    view.reset(sh)
    for f in range(args.warmup):
        view.run(fps[f], f, frames[f], out, sh)
    view.set_timing(True)
    view.read_timing()
    prof_frames = min(args.steps, 8)
    for k in range(prof_frames):
        f = args.warmup + k
        view.run(fps[f], f, frames[f], out, sh)
    passes = view.read_timing()
    view.set_timing(False)
    dom = max(passes, key=lambda k: passes[k][1])
    dl, dms = passes[dom]
    avg_s = dms / dl / 1e3
    if dom in PASS_BYTES_PER_CELL:
        units = 16 << params.hg_log2_buckets
        per_unit = PASS_BYTES_PER_CELL[dom]
    else:
        units = n
        per_unit = PASS_BYTES_PER_PIXEL[FORM][dom]
    alg_bytes = per_unit * units
    peaks = measured_peaks()
    if peaks and peaks.get("hbm_gbs"):
        peak, peak_src = float(peaks["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst)"
    else:
        peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    achieved = alg_bytes / avg_s / 1e9
    traffic = MEASURED_TRAFFIC_PER_UNIT.get(dom)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic * units if traffic else None, "kernel": dom,
                "alg_bytes_per_launch": alg_bytes, "launch_ms": avg_s * 1e3, "peak_source": peak_src}
    # The whole frame against HBM: the fused-minimum bytes of a frame (inputs, state
    # read and written, outputs, and the hash grid's decay bytes and updated cells,
    # counted on the last profiled frame) over the headline frame time.
    cells = 16 << params.hg_log2_buckets
    ptr_u, _ = view.buffer("hg_compact_count")
    torch.cuda.synchronize()
    ubuf = torch.zeros(1, dtype=torch.int32, device=dev)
    ctypes.CDLL("libcudart.so.13").cudaMemcpy(ctypes.c_void_p(ubuf.data_ptr()), ctypes.c_void_p(ptr_u),
                                              ctypes.c_size_t(4), 3)
    upd = int(ubuf.cpu().item())
    frame_bytes = FRAME_BYTES_PER_PIXEL[FORM] * n + FRAME_BYTES_PER_CELL * cells + FRAME_BYTES_PER_UPDATED_CELL * upd
    frame_gbs = frame_bytes / (ms / args.steps / 1e3) / 1e9
    roofline["frame"] = {"bytes_per_frame": frame_bytes, "bytes_per_pixel": FRAME_BYTES_PER_PIXEL[FORM],
                         "hash_grid_cells": cells, "updated_cells": upd, "achieved": frame_gbs,
                         "frac": frame_gbs / peak, "unit": "GB/s",
                         "definition": "fused-minimum bytes per frame / headline ms per frame"}
    # The same launch against the SMs' instruction-issue rate at the sampled clock.
    issue = None
    wi = MEASURED_WARP_INSTRUCTIONS_PER_UNIT.get(dom)
    if wi:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
        ipeak = sms * ISSUE_SLOTS_PER_SM_CLOCK * mhz * 1e6 / 1e9
        iach = wi * units / avg_s / 1e9
        issue = {"bound": "issue", "achieved": iach, "peak": ipeak, "unit": "G warp-instructions/s",
                 "frac": iach / ipeak, "kernel": dom, "warp_instructions_per_unit": wi, "sm_count": sms,
                 "sm_mhz": mhz, "source": "smsp__inst_executed.sum per pixel (ncu, 960x540 f32)"}
    pass_table = {}
    for k, (nl, tot) in sorted(passes.items()):
        if k in PASS_BYTES_PER_CELL:
            b = PASS_BYTES_PER_CELL[k] * (16 << params.hg_log2_buckets)
        else:
            b = PASS_BYTES_PER_PIXEL[FORM].get(k, 0) * n
        pass_table[k] = {"launches": nl, "ms_per_frame": tot / prof_frames,
                         "alg_gbs": (b * nl / (tot / 1e3) / 1e9) if tot > 0 and b else None}

    # ---- end to end through the C ABI with host buffers
    # Each frame's inputs sit in one pinned host buffer and go up with one copy; the
    # outputs come back with one copy; vlt_frame_run gets pointers bound once per
    # staging slot. Frames are pipelined over two slots: the copy stream uploads frame
    # f+2's inputs and reads back frame f's outputs while the compute stream runs
    # frame f+1. Every frame's upload and read-back is inside the timed region.
    keys = list(frames[0].keys())
    sizes = [frames[0][k].numel() for k in keys]
    offs, tot_in = [], 0
    for sz in sizes:  # each input 256-byte aligned inside the slot
        offs.append(tot_in)
        tot_in += (sz + 255) // 256 * 256
    host = []
    for f in range(nframes):
        hf = torch.empty(tot_in, dtype=torch.uint8, pin_memory=True)
        for k, o, sz in zip(keys, offs, sizes):
            hf[o:o + sz].copy_(frames[f][k])
        host.append(hf)
    out_bytes = n * out_px
    out_host = torch.empty(2 * out_bytes, dtype=torch.uint8, pin_memory=True)
    view.reset(sh)
    copy_stream = torch.cuda.Stream(device=dev)
    stage = [torch.empty(tot_in, dtype=torch.uint8, device=dev) for _ in range(2)]
    outd = [torch.empty(2 * out_bytes, dtype=torch.uint8, device=dev) for _ in range(2)]
    bind = [vg.FrameBinding({k: stage[s_][o:o + sz] for k, o, sz in zip(keys, offs, sizes)},
                            {"diffuse": outd[s_][:out_bytes], "specular": outd[s_][out_bytes:]}) for s_ in range(2)]
    ready = [torch.cuda.Event() for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]

    def upload(f, slot):
        with torch.cuda.stream(copy_stream):
            stage[slot].copy_(host[f], non_blocking=True)
            ready[slot].record(copy_stream)

    def e2e_frames(f0, f1):
        upload(f0, f0 % 2)
        if f0 + 1 < f1:
            upload(f0 + 1, (f0 + 1) % 2)
        for f in range(f0, f1):
            s = f % 2
            stream.wait_event(ready[s])
            view.run_bound(bind[s], fps[f], f, sh)
            done[s].record(stream)
            copy_stream.wait_event(done[s])
            with torch.cuda.stream(copy_stream):
                out_host.copy_(outd[s], non_blocking=True)
            if f + 2 < f1:
                upload(f + 2, s)

    e2e_frames(0, args.warmup)
    torch.cuda.synchronize()
    barrier(ws)
    e0.record(copy_stream)
    t0 = time.perf_counter()
    e2e_frames(args.warmup, args.warmup + args.steps)
    e1.record(copy_stream)
    torch.cuda.synchronize()
    e2e_event_ms = e0.elapsed_time(e1)
    e2e_wall_ms = (time.perf_counter() - t0) * 1e3
    e2e_ms = max(e2e_event_ms, e2e_wall_ms)
    barrier(ws)
    e2e_ms = max_over_ranks(e2e_ms, ws, dev)
    e2e_value = ws * args.steps * n / (e2e_ms / 1e3) / 1e6
    # The host link on its own, after the timed region: three uploads of one frame's
    # packed inputs, then three read-backs of its outputs, on the copy stream.
    l0, l1, l2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.cuda.stream(copy_stream):
        l0.record(copy_stream)
        for _ in range(3):
            stage[0].copy_(host[0], non_blocking=True)
        l1.record(copy_stream)
        for _ in range(3):
            out_host.copy_(outd[0], non_blocking=True)
        l2.record(copy_stream)
    torch.cuda.synchronize()
    link = {"h2d_gbs": 3 * tot_in / (l0.elapsed_time(l1) / 1e3) / 1e9,
            "d2h_gbs": 3 * out_host.numel() / (l1.elapsed_time(l2) / 1e3) / 1e9,
            "definition": "pinned host <-> device copies alone on the copy stream, after the timed region"}
    view.close()
    ctx.close()
    del frames, host

    batched = None
    if not args.no_batched:
        batched = batched_leg(args, ws, dev)
        # Small views (widths 256..640), where a plain frame is too short to fill the GPU
        # and batching the views into one launch per pass should pay.
        batched["small_views"] = batched_leg(args, ws, dev, w_max=640.0)

    precision = None
    if not args.no_precision:
        precision = precision_leg(args, ws, dev)
        if rank == 0 and not args.no_fp64:
            precision["against_fp64"] = fp64_precision_leg(args, dev)

    post = None
    if not args.no_post:
        post = post_leg(args, ws, dev)

    traced = None
    if not args.no_traced:
        traced = traced_leg(args, ws, dev)

    serving = None
    if not args.no_serving:
        serving = serving_leg(args, ws, dev)
        if not args.no_serving_sweep:
            # Latency/throughput across the per-step pixel budget (shorter runs), and one
            # run where the HBM budget alone gates admission.
            sweep = []
            for mpix in (6.0, 12.0, 24.0, 0.0):
                r = serving_leg(args, ws, dev, seconds=args.sweep_seconds, step_mpix=mpix)
                sweep.append({k: r[k] for k in ("step_pixel_budget_mpix", "hbm_budget_gb", "value", "latency_ms",
                                                "latency_ms_by_class", "admission_wait_ms", "time_to_first_frame_ms",
                                                "frames_per_step", "sessions_admitted", "peak_bytes_in_use_gb")})
            r = serving_leg(args, ws, dev, seconds=args.sweep_seconds, step_mpix=0.0, hbm_gb=args.sweep_hbm_gb)
            sweep.append({k: r[k] for k in ("step_pixel_budget_mpix", "hbm_budget_gb", "value", "latency_ms",
                                            "latency_ms_by_class", "admission_wait_ms", "time_to_first_frame_ms",
                                            "frames_per_step", "sessions_admitted", "peak_bytes_in_use_gb")})
            serving["sweep"] = sweep

    cpu = None
    if rank == 0 and not args.no_cpu:
        mpix, cores, times = cpu_sample(W, H, args.cpu_frames, 1000)
        cpu = {"value": mpix, "unit": "Mpix/s", "cores": cores, "kind": "port",
               "sample": "frames 1-%d of the same 1920x1080 workload (frame 0, without history, excluded); "
                         "%.1f s of CPU work" % (args.cpu_frames - 1, sum(times))}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "width": W, "height": H, "storage": FORM,
                       "parallelism": "replicas" if ws > 1 else "single view",
                       "l2": "inputs+state per frame > L2 (distinct frames, no flush)",
                       "knobs": {k: getattr(params, k) for k, _ in params._fields_}},
            "e2e": {"value": e2e_value, "unit": "Mpix/s", "h2d_bytes_per_step": tot_in,
                    "d2h_bytes_per_step": 2 * out_px * n,
                    "event_ms_per_step": e2e_event_ms / args.steps, "wall_ms_per_step": e2e_wall_ms / args.steps,
                    "host_link": link},
            "ref_storage_form": {"value": value_ref, "unit": "Mpix/s", "ms_per_step": ms_ref / args.steps},
            "pipelined": pipelined,
            "gpu_launches": launches,
            "roofline": roofline,
            "issue_roofline": issue,
            "passes": pass_table,
            "cpu_baseline": cpu,
            "clocks": clk,
            "batched": batched,
            "serving": serving,
            "precision": precision,
            "post_passes": post,
            "traced": traced,
        }
        print(json.dumps(line), flush=True)


def batch_view_set(n_views, seed, w_max=2560.0):
    """Resolutions drawn log-uniformly from 256x144 to w_max (by width; 2560x1440 by
    default), aspect 16:9, 4:3 or 1:1, each view with its own scene seed."""
    rng = np.random.default_rng(seed)
    views = []
    for k in range(n_views):
        w = float(np.exp(rng.uniform(np.log(256.0), np.log(w_max))))
        aspect = [16.0 / 9.0, 4.0 / 3.0, 1.0][int(rng.integers(0, 3))]
        w = int(round(w / 2.0)) * 2
        h = max(2, int(round(w / aspect / 2.0)) * 2)
        views.append((w, h, 7000 + k))
    return views


def batched_leg(args, ws, dev, w_max=2560.0):
    """Many views of uneven size per step: every view's frames run one by one
    through vlt_frame_run (plain), then the same frames through vlt_batch_run
    (batched persistent kernels, CUDA graphs, autotuned tiles). Inputs are resident;
    both arms time the same steps after the same warm-up frames."""
    import torch

    import violet_gb300 as vg

    specs = batch_view_set(args.batch_views, 42, w_max)
    frames_total = args.batch_frames
    warm = 3
    params = workload_params(vg)
    ctx = vg.Context(dev.index)
    # A created stream: CUDA graphs cannot capture the legacy default stream.
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    total_px = sum(w * h for w, h, _ in specs)
    per_frame_in = sum(input_bytes_per_pixel(vg, params) * w * h for w, h, _ in specs)
    state = sum(vg.View.device_bytes(w, h, "f32", params) for w, h, _ in specs)
    need = per_frame_in * frames_total + state + total_px * 64
    if need > 150e9:
        return {"skipped": "needs %.0f GB of HBM" % (need / 1e9)}
    scenes = [vg.Scene(seed, w, h, disocclusion_frac=0.02) for w, h, seed in specs]
    frames = []
    for f in range(frames_total):
        fr = []
        for k, (w, h, seed) in enumerate(specs):
            bufs = input_buffers(vg, params, w, h, dev)
            scenes[k].generate_device(f, bufs, sh)
            fr.append(bufs)
        frames.append(fr)
    fps = [[scenes[k].frame_params(f) for k in range(len(specs))] for f in range(frames_total)]
    outs = [{o: torch.empty(w * h * 16, dtype=torch.uint8, device=dev) for o in ("diffuse", "specular")}
            for w, h, _ in specs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = frames_total - warm

    def plain_arm(form):
        """Each view's frame through vlt_frame_run, view after view."""
        views = [vg.View(ctx, w, h, form, params) for w, h, _ in specs]
        for f in range(warm):
            for k, v in enumerate(views):
                v.run(fps[f][k], f, frames[f][k], outs[k], sh)
        torch.cuda.synchronize()
        barrier(ws)
        e0.record(stream)
        for f in range(warm, frames_total):
            for k, v in enumerate(views):
                v.run(fps[f][k], f, frames[f][k], outs[k], sh)
        e1.record(stream)
        torch.cuda.synchronize()
        t = max_over_ranks(e0.elapsed_time(e1), ws, dev)
        for v in views:
            v.close()
        return t

    def batched_arm(form):
        """The same frames through vlt_batch_run, after tuning the launch shapes on
        the same views (results do not depend on the shapes)."""
        views = [vg.View(ctx, w, h, form, params) for w, h, _ in specs]
        batch = vg.Batch(ctx)
        batch.autotune()
        for f in range(2 * vg._ffi.TILE_CANDIDATES + 1):
            ff = f % frames_total
            batch.run(views, fps[ff], [ff] * len(views), frames[ff], outs, stream=sh)
        tiles = batch.tile_table()
        for v in views:
            v.reset(sh)
        for f in range(warm):
            batch.run(views, fps[f], [f] * len(views), frames[f], outs, stream=sh)
        torch.cuda.synchronize()
        st0 = batch.stats()
        barrier(ws)
        e0.record(stream)
        for f in range(warm, frames_total):
            batch.run(views, fps[f], [f] * len(views), frames[f], outs, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        t = max_over_ranks(e0.elapsed_time(e1), ws, dev)
        st1 = batch.stats()
        batch.close()
        for v in views:
            v.close()
        return t, st0, st1, tiles

    plain_ms = plain_arm("f32")
    b32_ms, _, _, _ = batched_arm("f32")
    batch_ms, st0, st1, tiles = batched_arm(args.batch_form)
    ctx.close()
    del frames
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    px = ws * total_px * steps
    return {
        "workload": "%d views, %d frames each, widths log-uniform 256..%d, aspect 16:9/4:3/1:1" % (
            len(specs), frames_total, int(w_max)),
        "storage": args.batch_form, "views": len(specs), "frames": frames_total, "timed_steps": steps,
        "mpix_per_step": total_px / 1e6,
        "value": px / (batch_ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": batch_ms / steps,
        "plain_value": px / (plain_ms / 1e3) / 1e6, "plain_ms_per_step": plain_ms / steps,
        "plain_storage": "f32",
        "speedup_vs_plain": plain_ms / batch_ms,
        "batched_f32_value": px / (b32_ms / 1e3) / 1e6,
        "speedup_batching_alone": plain_ms / b32_ms,
        "launches_per_step": st1["last_launches"], "view_passes_per_step": st1["last_jobs"],
        "graph_replays": st1["graph_replays"] - st0["graph_replays"],
        "graph_captures": st1["graph_captures"] - st0["graph_captures"],
        "arena_bytes": st1["arena_bytes"],
        "tiles": {k: list(v["tile"]) + (["persistent"] if v["persistent"] else []) for k, v in tiles.items()},
        "sizes": [[w, h] for w, h, _ in specs],
    }


def precision_leg(args, ws, dev):
    """3840x2160, --precision-frames frames: device-resident throughput of the f16 and
    f32 storage forms on the same frames, then both forms in lockstep with binary64
    image reductions on the GPU between their denoised outputs (energy ratio and
    relative L2 per frame; the latter includes resampling decisions that diverge
    between differently stored reservoirs, so it bounds the divergence, not the
    precision, which the binary64 denoiser test measures). Frame inputs: a ring of
    16 consecutive frames walked forth and back (each frame's inputs are far larger
    than L2)."""
    import numpy as np
    import torch

    import violet_gb300 as vg

    W, H = 3840, 2160
    n = W * H
    ring = 16
    params = workload_params(vg)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    sc = vg.Scene(4000, W, H, disocclusion_frac=0.02)
    pool = []
    for f in range(ring):
        bufs = input_buffers(vg, params, W, H, dev)
        sc.generate_device(f, bufs, sh)
        pool.append((bufs, sc.frame_params(f)))

    def ring_index(f):
        k = f % (2 * ring - 2)
        return k if k < ring else 2 * ring - 2 - k

    ctx = vg.Context(dev.index)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    frames = args.precision_frames
    warm = 3
    res = {}
    outs = {}
    for form in ("f32", "f16"):
        ob = 16 if form == "f32" else 8
        outs[form] = {o: torch.empty(n * ob, dtype=torch.uint8, device=dev) for o in ("diffuse", "specular")}
        v = vg.View(ctx, W, H, form, params)
        for f in range(warm):
            bufs, fp = pool[ring_index(f)]
            v.run(fp, f, bufs, outs[form], sh)
        torch.cuda.synchronize()
        barrier(ws)
        e0.record(stream)
        for f in range(warm, frames):
            bufs, fp = pool[ring_index(f)]
            v.run(fp, f, bufs, outs[form], sh)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1), ws, dev)
        res[form] = {"value": ws * n * (frames - warm) / (ms / 1e3) / 1e6, "unit": "Mpix/s",
                     "ms_per_frame": ms / (frames - warm), "device_bytes": vg.View.device_bytes(W, H, form, params)}
        v.close()
    # lockstep comparison of the two forms' outputs
    lib = vg.lib()
    v32 = vg.View(ctx, W, H, "f32", params)
    v16 = vg.View(ctx, W, H, "f16", params)
    st = torch.zeros(8, dtype=torch.float64, device=dev)
    energy, rel = {"diffuse": [], "specular": []}, {"diffuse": [], "specular": []}
    for f in range(min(frames, 32)):
        bufs, fp = pool[ring_index(f)]
        v32.run(fp, f, bufs, outs["f32"], sh)
        v16.run(fp, f, bufs, outs["f16"], sh)
        if f < 1:
            continue
        for o in ("diffuse", "specular"):
            lib.vlt_image_stats(ctypes.c_void_p(outs["f16"][o].data_ptr()), 1, ctypes.c_void_p(outs["f32"][o].data_ptr()),
                                0, n, ctypes.c_void_p(st.data_ptr()), ctypes.c_void_p(sh))
            stream.synchronize()
            s = st.cpu().numpy()
            energy[o].append(float(s[0:3].sum() / max(s[3:6].sum(), 1e-300)))
            rel[o].append(float(np.sqrt(s[6] / max(s[7], 1e-300))))
    v32.close()
    v16.close()
    ctx.close()
    del pool
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return {
        "workload": "3840x2160, %d frames (ring of %d consecutive frames walked forth and back), plain knobs" % (
            frames, ring),
        "f16": res["f16"], "f32": res["f32"], "f16_speedup": res["f16"]["value"] / res["f32"]["value"],
        "f16_vs_f32_energy_ratio": {o: {"mean": float(np.mean(v)), "max_dev": float(np.max(np.abs(np.array(v) - 1)))}
                                    for o, v in energy.items()},
        "f16_vs_f32_rel_l2": {o: {"mean": float(np.mean(v)), "max": float(np.max(v))} for o, v in rel.items()},
        "reductions": "binary64 on the GPU (vlt_image_stats)",
    }


FP64_OUTPUTS = ["diff_W", "spec_W", "ao", "raw_diffuse", "raw_specular", "ray_len", "hist_color", "hist_moments",
                "variance", "denoised_diffuse", "denoised_specular"]


def fp64_precision_leg(args, dev):
    """Per-output error of the FP32 and FP16 storage forms against the binary64
    replay of the whole back end (oracle/oracle64r.cpp): every frame the GPU view and
    the oracle's view of the same form run the same inputs (their outputs are
    checked bit for bit), and the replay, following the float form's decisions (the
    same selected samples, accepted taps and history lengths), recomputes every value
    in binary64 with unquantized storage. The differences are the form's arithmetic
    and storage alone. Plain knobs of the 1080p workload at 960x540 (1/16 of the 4K
    pixels of the precision workload; the binary64 replay runs on the host)."""
    import torch

    import violet_gb300 as vg
    from oracle import pyoracle as po

    W, H = args.fp64_width, args.fp64_height
    n = W * H
    params = workload_params(vg)
    ctx = vg.Context(dev.index)
    res = {}
    for form in ("f32", "f16"):
        ob = 16 if form == "f32" else 8
        dt = np.float32 if form == "f32" else np.float16
        scene = vg.Scene(4000, W, H, disocclusion_frac=0.02)
        view = vg.View(ctx, W, H, form, params)
        ov = po.OracleView(W, H, params, form)
        ov.enable_fp64()
        dev_in = input_buffers(vg, params, W, H, dev)
        out_dev = {k: torch.zeros(ob * n, dtype=torch.uint8, device=dev) for k in ("diffuse", "specular")}
        errs = {k: [] for k in FP64_OUTPUTS}
        flips, gpu_mismatch, decisions_equal, flips_by_pass = [], 0, True, {}
        for f in range(args.fp64_frames):
            host = scene.generate_host(f)
            for k, t in dev_in.items():
                t.copy_(torch.from_numpy(host[k].view(np.uint8)))
            fp = scene.frame_params(f)
            view.run(fp, f, dev_in, out_dev)
            out_host = {k: np.zeros(ob * n, np.uint8) for k in ("diffuse", "specular")}
            ov.run(fp, f, host, out_host)
            got = {k: out_dev[k].cpu().numpy() for k in out_dev}
            if any(not np.array_equal(got[k], out_host[k]) for k in got):
                gpu_mismatch += 1
            flips.append(ov.fp64_flips())
            for nm in ("diff_M", "spec_M", "hist_len"):
                ref = ov.fp64(nm)
                if form == "f16" and nm == "diff_M":
                    ref = np.minimum(ref, 255.0)  # the FP16 form stores M in a byte
                if f > 0 and not np.array_equal(ov.form_values(nm), ref):
                    decisions_equal = False
            for k, c in ov.fp64_flips_by_pass().items():
                flips_by_pass[k] = flips_by_pass.get(k, 0) + c
            if f == 0:
                continue  # no denoised output without history
            for nm in FP64_OUTPUTS:
                if nm.startswith("denoised_"):
                    a = got[nm.split("_")[1]].view(dt).reshape(n, 4)[:, :3].astype(np.float64)
                else:
                    a = ov.form_values(nm)
                b = ov.fp64(nm)
                m = np.isfinite(a).all(1) & np.isfinite(b).all(1)
                den = np.linalg.norm(b[m])
                errs[nm].append((float(np.linalg.norm(a[m] - b[m]) / den) if den > 0 else 0.0,
                                 float(np.max(np.abs(a[m] - b[m]))) if m.any() else 0.0,
                                 float(np.max(np.abs(b[m]))) if m.any() else 0.0, int((~m).sum())))
        view.close()
        ov.close()
        table = {}
        for nm, e in errs.items():
            e = np.array(e)
            table[nm] = {"rel_l2_mean": float(e[:, 0].mean()), "rel_l2_max": float(e[:, 0].max()),
                         "max_abs_err": float(e[:, 1].max()), "max_abs_value": float(e[:, 2].max()),
                         "nonfinite_pixels": int(e[:, 3].sum())}
        res[form] = {"per_output": table, "decision_flips_per_frame": {"mean": float(np.mean(flips)),
                                                                       "max": int(np.max(flips)),
                                                                       "pixels": n},
                     "decision_flips_by_pass": flips_by_pass,
                     "decisions_replayed_exactly": decisions_equal, "gpu_frames_not_bitexact_vs_oracle": gpu_mismatch,
                     "denoised_meets_1e-3": bool(max(table["denoised_diffuse"]["rel_l2_max"],
                                                     table["denoised_specular"]["rel_l2_max"]) <= 1e-3)}
    ctx.close()
    return {"workload": "%dx%d, %d frames, plain 1080p knobs; binary64 replay of the float form's decisions" % (
        W, H, args.fp64_frames), "f32": res["f32"], "f16": res["f16"]}


def traced_leg(args, ws, dev):
    """Traced mode (params.trace = 1, diffuse validation every 4th frame, specular
    validation every frame) on the headline workload: the back end's device time per
    frame, phase one (hash-grid selection/compaction and the rays) plus phase two
    (shading the hits and the rest of the frame); the synthetic scene traces the rays
    in between, outside the timed spans."""
    import torch

    import violet_gb300 as vg

    W, H = args.width, args.height
    n = W * H
    params = workload_params(vg)
    params.trace = 1
    params.diff_validate = 1
    params.spec_validate = 1
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    sc = vg.Scene(6000, W, H, disocclusion_frac=0.02)
    nfr = args.warmup + args.steps
    frames = []
    for f in range(nfr):
        bufs = input_buffers(vg, params, W, H, dev)
        sc.generate_device(f, bufs, sh)
        frames.append((bufs, sc.frame_params(f)))
    ctx = vg.Context(dev.index)
    v = vg.View(ctx, W, H, FORM, params)
    nq = v.cache_ray_capacity
    rays = {"cache": torch.empty(max(nq, 1) * 32, dtype=torch.uint8, device=dev),
            "diffuse": torch.empty(n * 32, dtype=torch.uint8, device=dev),
            "spec_validate": torch.empty(n * 32, dtype=torch.uint8, device=dev)}
    hits = {k: torch.empty(t.numel() * 2, dtype=torch.uint8, device=dev) for k, t in rays.items()}
    ob = 16 if FORM == "f32" else 4
    out = {o: torch.empty(n * ob, dtype=torch.uint8, device=dev) for o in ("diffuse", "specular")}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    total = 0.0
    launches = 0
    for f in range(nfr):
        bufs, fp = frames[f]
        ev[0].record(stream)
        counts = v.trace(fp, f, bufs, rays, sh)
        ev[1].record(stream)
        inp = dict(bufs)
        for k, name in (("cache", "cache_hits"), ("diffuse", "diffuse_hits"), ("spec_validate", "spec_validate_hits")):
            if counts[k]:
                sc.trace_device(fp, rays[k], counts[k], hits[k], sh)
                inp[name] = hits[k]
        ev[2].record(stream)
        v.run(fp, f, inp, out, sh)
        ev[3].record(stream)
        torch.cuda.synchronize()
        if f >= args.warmup:
            total += ev[0].elapsed_time(ev[1]) + ev[2].elapsed_time(ev[3])
            launches += v.launches
    v.close()
    ctx.close()
    del frames
    ms = max_over_ranks(total, ws, dev)
    return {"workload": "%dx%d %s storage, plain knobs, traced mode with validation" % (W, H, FORM),
            "value": ws * n * args.steps / (ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_frame": ms / args.steps,
            "timed": "vlt_frame_trace + vlt_frame_run device time (scene tracing excluded)",
            "launches_per_frame": launches / args.steps}


def post_leg(args, ws, dev):
    """The frame with the passes the reference renderer runs after the denoiser
    (final lighting and temporal AA, params.post = 2) on the headline workload:
    device-resident Mpix/s of the whole frame and per-pass times."""
    import torch

    import violet_gb300 as vg

    W, H = args.width, args.height
    n = W * H
    params = workload_params(vg)
    params.post = 2
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    sc = vg.Scene(5000, W, H, disocclusion_frac=0.02)
    nfr = args.warmup + args.steps
    frames = []
    for f in range(nfr):
        bufs = input_buffers(vg, params, W, H, dev)
        sc.generate_device(f, bufs, sh)
        frames.append((bufs, sc.frame_params(f)))
    ob = 16 if FORM == "f32" else 4
    out = {o: torch.empty(n * ob, dtype=torch.uint8, device=dev) for o in ("diffuse", "specular", "taa")}
    ctx = vg.Context(dev.index)
    v = vg.View(ctx, W, H, FORM, params)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for f in range(args.warmup):
        v.run(frames[f][1], f, frames[f][0], out, sh)
    torch.cuda.synchronize()
    barrier(ws)
    e0.record(stream)
    for f in range(args.warmup, nfr):
        v.run(frames[f][1], f, frames[f][0], out, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), ws, dev)
    v.reset(sh)
    for f in range(args.warmup):
        v.run(frames[f][1], f, frames[f][0], out, sh)
    v.set_timing(True)
    v.read_timing()
    for f in range(args.warmup, nfr):
        v.run(frames[f][1], f, frames[f][0], out, sh)
    passes = v.read_timing()
    v.close()
    ctx.close()
    del frames
    res = {"workload": "%dx%d %s storage, plain knobs, post = 2 (final lighting + TAA)" % (W, H, FORM),
           "value": ws * n * args.steps / (ms / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_frame": ms / args.steps}
    for k in ("final_lighting", "taa"):
        if k in passes:
            nl, tot = passes[k]
            b = PASS_BYTES_PER_PIXEL[FORM][k] * n
            res[k] = {"ms_per_frame": tot / nl, "alg_gbs": b * nl / (tot / 1e3) / 1e9}
    return res


SERVE_CLASSES = [("720p", 1280, 720, 0.3), ("1080p", 1920, 1080, 0.4), ("1440p", 2560, 1440, 0.2),
                 ("2160p", 3840, 2160, 0.1)]
POOL_FRAMES = 16


def serving_leg(args, ws, dev, seconds=None, step_mpix=None, hbm_gb=None):
    """Poisson arrivals of view-sessions through the server (vlt_server_*): each
    admitted session keeps one frame queued (the next is submitted when the last
    completes); every step batches the queued frames of all admitted sessions.
    Per-frame latency is submit-to-completion (a session's first frame is submitted
    when the session opens, so it includes the admission wait); the admission wait of
    a session is its first frame's latency minus the step that ran it; time to first
    frame is open-to-completion of that frame.
    Per-frame latency is submit-to-completion on the host clock. Frame inputs come
    from a pool of POOL_FRAMES consecutive frames per resolution class, walked
    forth and back, so the timed loop runs only the lighting path."""
    import numpy as np
    import torch

    import violet_gb300 as vg

    seconds = args.serve_seconds if seconds is None else seconds
    step_mpix = args.serve_step_mpix if step_mpix is None else step_mpix
    hbm_gb = args.serve_hbm_gb if hbm_gb is None else hbm_gb
    rng = np.random.default_rng(4242)
    params = workload_params(vg)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    pools = {}
    for name, w, h, _ in SERVE_CLASSES:
        sc = vg.Scene(900 + w, w, h, disocclusion_frac=0.02)
        frames = []
        for f in range(POOL_FRAMES):
            bufs = input_buffers(vg, params, w, h, dev)
            sc.generate_device(f, bufs, sh)
            frames.append((bufs, sc.frame_params(f)))
        pools[name] = frames
    torch.cuda.synchronize()
    ctx = vg.Context(dev.index)
    server = vg.Server(ctx, int(hbm_gb * 1e9), int(step_mpix * 1e6))
    # arrivals
    t_arr, classes, lengths = [], [], []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > seconds:
            break
        t_arr.append(t)
        k = int(rng.choice(len(SERVE_CLASSES), p=[c[3] for c in SERVE_CLASSES]))
        classes.append(k)
        lengths.append(int(rng.integers(30, 301)))
    form = args.serve_form
    out_px = {"ref": 4, "f32": 16, "f16": 8}[form]
    live = {}  # session id -> state
    lat_all, lat_cls = [], {c[0]: [] for c in SERVE_CLASSES}
    admit_wait, ttff = [], []
    frames_done = 0
    pix_done = 0
    nxt = 0
    barrier(ws)
    t0 = time.perf_counter()
    steps = 0
    while True:
        now = time.perf_counter() - t0
        while nxt < len(t_arr) and t_arr[nxt] <= now:
            name, w, h, _ = SERVE_CLASSES[classes[nxt]]
            sid = server.open(w, h, form, params)
            live[sid] = {"cls": name, "w": w, "h": h, "n": lengths[nxt], "sent": 0, "done": 0, "t_open": now,
                         "out": {o: torch.empty(w * h * out_px, dtype=torch.uint8, device=dev)
                                 for o in ("diffuse", "specular")}}
            nxt += 1
        if now > seconds:
            break
        for sid, st in live.items():
            if st["sent"] == st["done"] and st["sent"] < st["n"]:
                f = st["sent"]
                pi = f % (2 * POOL_FRAMES - 2)
                pi = pi if pi < POOL_FRAMES else 2 * POOL_FRAMES - 2 - pi
                bufs, fp = pools[st["cls"]][pi]
                server.submit(sid, fp, f, bufs, st["out"], tag=f)
                st["sent"] += 1
        issued = server.step(sh)
        if issued:
            steps += 1
        for sid, tag, lat, step_ms in server.poll(wait=True):
            st = live[sid]
            if st["done"] == 0:
                admit_wait.append(max(lat - step_ms, 0.0))
                ttff.append((time.perf_counter() - t0) * 1e3 - st["t_open"] * 1e3)
            st["done"] += 1
            lat_all.append(lat)
            lat_cls[st["cls"]].append(lat)
            frames_done += 1
            pix_done += st["w"] * st["h"]
            if st["done"] == st["n"]:
                server.close_session(sid)
        for sid in [k for k, v in live.items() if v["done"] == v["n"]]:
            del live[sid]
        if not issued and nxt < len(t_arr):
            time.sleep(max(0.0, min(0.002, t_arr[nxt] - (time.perf_counter() - t0))))
    elapsed = time.perf_counter() - t0
    stats = server.stats()
    server.close()
    ctx.close()
    del pools
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    def pct(x, q):
        return float(np.percentile(x, q)) if x else None

    waiting_open = [(elapsed - st["t_open"]) * 1e3 for st in live.values() if st["done"] == 0]
    return {
        "workload": "Poisson %.0f sessions/s for %.0f s; 720p/1080p/1440p/2160p with p=0.3/0.4/0.2/0.1; 30-300 "
                    "frames each; HBM budget %.0f GB; step pixel budget %s" % (
                        args.serve_rate, seconds, hbm_gb, ("%.1f Mpix" % step_mpix) if step_mpix else "off"),
        "hbm_budget_gb": hbm_gb, "step_pixel_budget_mpix": step_mpix or None,
        "admission_wait_ms": {"p50": pct(admit_wait, 50), "p99": pct(admit_wait, 99), "sessions": len(admit_wait),
                              "still_waiting_at_end": len(waiting_open),
                              "still_waiting_min_ms": min(waiting_open) if waiting_open else None},
        "time_to_first_frame_ms": {"p50": pct(ttff, 50), "p99": pct(ttff, 99)},
        "peak_bytes_in_use_gb": stats["bytes_in_use"] / 1e9,
        "admit_failures": stats.get("admit_failures", 0),
        "storage": form, "sessions_arrived": len(t_arr), "sessions_admitted": stats["sessions_admitted"],
        "sessions_completed": stats["sessions_closed"], "sessions_waiting_at_end": stats["sessions_waiting"],
        "frames": frames_done, "steps": steps, "frames_per_step": frames_done / max(steps, 1),
        "value": pix_done / elapsed / 1e6, "unit": "Mpix/s", "seconds": elapsed,
        "latency_ms": {"p50": pct(lat_all, 50), "p99": pct(lat_all, 99)},
        "latency_ms_by_class": {k: {"p50": pct(v, 50), "p99": pct(v, 99), "frames": len(v)}
                                for k, v in lat_cls.items()},
        "admit_wait_ms_mean": stats["admit_wait_ms_total"] / max(stats["sessions_admitted"], 1),
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=W_DEFAULT)
    ap.add_argument("--height", type=int, default=H_DEFAULT)
    ap.add_argument("--cpu-frames", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-hbm-gb", type=float, default=150.0)
    ap.add_argument("--serve-step-mpix", type=float, default=6.0)
    ap.add_argument("--no-serving-sweep", action="store_true")
    ap.add_argument("--sweep-seconds", type=float, default=15.0)
    ap.add_argument("--sweep-hbm-gb", type=float, default=12.0)
    ap.add_argument("--batch-views", type=int, default=48)
    ap.add_argument("--batch-frames", type=int, default=32)
    ap.add_argument("--batch-form", default="f16", choices=["ref", "f32", "f16"])
    ap.add_argument("--serve-form", default="f32", choices=["ref", "f32", "f16"])
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-post", action="store_true")
    ap.add_argument("--no-traced", action="store_true")
    ap.add_argument("--precision-frames", type=int, default=64)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-pipelined", action="store_true")
    ap.add_argument("--fp64-frames", type=int, default=32)
    ap.add_argument("--fp64-width", type=int, default=960)
    ap.add_argument("--fp64-height", type=int, default=540)
    args = ap.parse_args()
    if args.warmup < 3:
        log("warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        # Rank 0 alone times the host-side reference; other ranks exit without work.
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")))
        return
    ws, rank, local = dist_setup()
    try:
        run_ours(args, ws, rank, local)
    finally:
        if ws > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
