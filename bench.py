"""Benchmark: frames/s and Gsamples/s of the GB300 raycaster on the CT-like
shaded DVR workload (512^3 uint16, spacing 0.7/0.7/1.0, 4096-entry TF,
Phong, 1920x1080, 2 samples/voxel), with the CPU path timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one frame. `value` is frames/s with the volume, TF and entry/exit
images resident in HBM (device-timed with CUDA events on the library's
stream); `e2e` is the same metric through the C ABI with host entry/exit
images and a host RGBA8 frame (copies inside the timed region).
`--impl reference` times the CPU path (the FP32 restatement of
CPURaycaster in oracle/, all host threads) on a bounded sample of rows per
step. One process per GPU; N > 1 runs N independent replicas (the path does
not shard across GPUs).
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s & Gsamples/s, 512³ u16 @1080p; learned vs plain fps at PSNR≥40 dB"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(value: float, ws: int):
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _whole_job(ms_local: float, ws: int):
    """Replicas: the slowest rank's time per step, and the frames/s of all
    ranks together (each rank renders its own frame per step)."""
    ms = _barrier_max(ms_local, ws)
    return ms, 1000.0 / ms * ws


def _barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace('.', '').isdigit())}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(key: str = "dram_bytes_per_launch"):
    """Per-launch DRAM (or L2) bytes of the march kernel from the committed
    ncu summary (profiles/); None if absent."""
    p = os.path.join(ROOT, "profiles", "march_dvr_phong_512cube_u16_1080p.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get(key)
        except (OSError, ValueError):
            return None
    return None


def build_workload(small: bool, kind: str = "ct", volume_fn=None):
    """ct: 512^3 u16 shaded DVR 1080p; mip: the same volume and TF under MIP;
    blobs: 128^3 u8 plain DVR 512x512 (the CPU-runnable case). volume_fn:
    the volume generator (default: the library's)."""
    from voreen_gb300 import synth
    if kind == "blobs":
        return synth.config1(volume_fn=volume_fn)
    comp = synth.MIP if kind == "mip" else synth.DVR
    if small:
        return synth.config2(size=(256, 256, 256), image=(960, 540), compositing=comp, volume_fn=volume_fn)
    return synth.config2(compositing=comp, volume_fn=volume_fn)


def oracle_workload_params(w, shading=None):
    """The oracle's render parameters for workload w (the processor defaults
    of the library's vrc_render_params_default: iso 0.5, ERT 0.95, light
    0.4 / 0.8 / 0.6, shininess 60)."""
    import oracle
    return oracle.make_params(sampling_rate=w.sampling_rate, compositing=w.compositing,
                              shading=w.shading if shading is None else shading, iso_value=0.5, ert=0.95,
                              light_pos=list(w.light_pos)[:3], camera_pos=list(w.camera_pos))


def run_cpu(w, entry, exit_pts, target_s: float, start_row: int | None = None):
    """FP32 CPURaycaster restatement on all host cores over a band of rows
    sized to about target_s: centred, or starting at start_row (wrapping to
    the top). Returns (seconds, rows, samples, threads, first row)."""
    import oracle
    op = oracle_workload_params(w)
    tf = oracle.bake_tf(w.tf_keys, w.tf_width)
    ov = oracle.make_volume(w.voxels, w.spacing)
    H = w.height
    threads = os.cpu_count() or 1
    # calibrate on 2 centre rows, then size the band to ~target_s
    r0 = H // 2 - 1
    t0 = time.perf_counter()
    _, s, _ = oracle.render(ov, tf, w.domain, op, entry, exit_pts, 32, rows=(r0, r0 + 2), nthreads=threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    rows = int(max(2, min(H, 2 * target_s / dt)))
    if start_row is None:
        lo = max(0, H // 2 - rows // 2)
        bands = [(lo, lo + rows)]
    else:
        lo = start_row % H
        bands = [(lo, min(H, lo + rows))]
        if lo + rows > H:
            bands.append((0, lo + rows - H))
    t0 = time.perf_counter()
    total = 0
    for a, b in bands:
        _, s, _ = oracle.render(ov, tf, w.domain, op, entry, exit_pts, 32, rows=(a, b), nthreads=threads)
        total += int(s.sum())
    dt = time.perf_counter() - t0
    return dt, rows, total, threads, lo


def frame_parity(ctx, vol, tf, p, w, e_dev, x_dev, e_host, x_host, gpu_samples):
    """The benchmarked frame (same volume, TF, camera and entry/exit points),
    rendered as RGBA32F by the library and by the FP32 and FP64 oracles over
    the whole image: max |d| against each, and the rays where FP32 and FP64
    take different discrete decisions (count, their max |d|, how many of them
    exceed 1/255). Outside the timed region."""
    import torch
    import oracle
    from oracle import parity
    import voreen_gb300 as v
    out = torch.empty((w.height, w.width, 4), dtype=torch.float32, device=e_dev.device)
    _, st = v.render(ctx, vol, tf, p, e_dev, x_dev, v.OUT_RGBA32F, out)
    img = out.cpu().numpy()
    op = oracle_workload_params(w, shading=p.shading)
    op.compositing = p.compositing
    ov = oracle.make_volume(w.voxels, w.spacing)
    otf = oracle.bake_tf(w.tf_keys, w.tf_width)
    t0 = time.perf_counter()
    g32 = np.zeros((w.height, w.width), np.uint32)
    g64 = np.zeros((w.height, w.width), np.uint32)
    o32, s32, fh32 = oracle.render(ov, otf, w.domain, op, e_host, x_host, 32, signature=g32)
    o64, s64, fh64 = oracle.render(ov, otf, w.domain, op, e_host, x_host, 64, signature=g64)
    step = 1.0 / (max(w.dims) * w.sampling_rate)
    r = parity.report(img, o32, s32, fh32, o64, s64, fh64, p.compositing, step, shaded=p.shading != v.SHADE_NONE,
                      sig32=g32, sig64=g64)
    r.update({"frame": f"{w.width}x{w.height} full frame, RGBA32F", "bound": 1.0 / 255.0,
              "samples_equal_fp32": int(s32.sum()) == int(st.samples) == int(gpu_samples),
              "bit_equal_fp32": bool(np.array_equal(img.view(np.uint32), o32.view(np.uint32))),
              "oracle_seconds": time.perf_counter() - t0})
    return r


def run_batch(args, warmup, ws, rank, local):
    """64 requests (volumes 64^3..512^3, u8/u16/f32, images 256^2..2048^2,
    DVR + Phong) in one persistent launch replayed from a CUDA graph; tile
    shape, brick size and skip cell per request class from the autotuner."""
    import numpy as np
    import torch

    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild, synth
    from voreen_gb300.autotune import Autotuner
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = v.Context(dev)
    vols_raw, reqs = synth.config3(seed=1, n=64)
    tuner = Autotuner(ctx)
    brick_of, tuned = {}, []
    for r in reqs:
        vox, sp = vols_raw[r["volume"]]
        mn, mx = float(vox.min()), float(vox.max())
        norm = {np.dtype(np.uint8): 255.0, np.dtype(np.uint16): 65535.0}.get(vox.dtype, 1.0)
        tf_rgba = v.TransferFunction.bake(r["tf_keys"], r["tf_width"])
        p = v.default_params(r["width"], r["height"])
        pos, focus, near, far = r["camera"]
        p.camera = v.make_camera(pos, focus, near=near, far=far)
        p.light_position[:] = list(r["light"])
        p.shading = v.SHADE_PHONG
        p.entry_exit_mode = v.EE_ANALYTIC
        best = tuner.tune(vox, sp, tf_rgba, (mn / norm, mx / norm), p, tune_bricks=r["volume"] not in brick_of)
        brick_of.setdefault(r["volume"], best["brick"])
        p.tile_width, p.skip_cell_size = best["tile_width"], min(best["skip_cell"], brick_of[r["volume"]])
        tuned.append((r, p, tf_rgba, (mn / norm, mx / norm)))
    vols = {k: v.Volume(ctx, vox, sp, brick_size=brick_of[k]) for k, (vox, sp) in vols_raw.items() if k in brick_of}
    items, pixels = [], 0
    for r, p, tf_rgba, dom in tuned:
        tf = v.TransferFunction(ctx, tf_rgba, dom)
        out = torch.empty((r["height"], r["width"], 4), dtype=torch.uint8, device=f"cuda:{dev}")
        items.append((vols[r["volume"]], tf, p, out, v.OUT_RGBA8))
        pixels += r["width"] * r["height"]
    batch = v.Batch(ctx, items)
    for _ in range(warmup):
        batch.launch()
    st, lat = batch.stats()
    samples = st.samples
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 200))
    _barrier(ws)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for _ in range(steps):
            batch.launch()
        end.record(stream)
        end.synchronize()
    clocks = clk.summary()
    ms = _barrier_max(start.elapsed_time(end) / steps, ws)
    st, lat = batch.stats()
    vol_bytes = {k: vv.device_bytes for k, vv in vols.items()}
    line = {"metric": "aggregate Gsamples/s and per-request latency p50/p99, 64 batched requests",
            "value": samples / (ms * 1e-3) / 1e9 * ws, "unit": "Gsamples/s", "n_gpus": ws, "steps": steps,
            "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded procedural volumes)",
            "config": {"workload": "64 requests, volumes {64^3,128^3,256^3,384x256x200,512^3} x {u8,u16,f32}, "
                                   "images {256^2,512^2,1024^2,1920x1080,2048^2}, DVR + Phong, one captured launch",
                       "distinct_volumes": len(vols), "pixels_per_launch": pixels,
                       "l2": "inputs larger than L2 (%.0f MB of bricked volumes)" % (sum(vol_bytes.values()) / 1e6)},
            "requests_per_s": 64 * 1000.0 / ms * ws,
            "latency_ms": {"p50": st.latency_p50_ms, "p99": st.latency_p99_ms, "max": st.latency_max_ms},
            "samples_per_launch": samples, "autotuned_classes": len(tuner.table),
            "autotune": tuner.table, "gpu_launches": steps * st.kernels_per_launch,
            "clocks": clocks}
    if rank == 0:
        print(json.dumps(line))


def run_preint(args, warmup, ws, rank, local):
    """Pre-integrated classification on the CT-like workload (DVR + Phong,
    512^3 u16, 1080p): the exact table (1024 x 1024, the largest size the
    reference derives) built on the GPU against the same build by the CPU
    restatement on all host cores, and frames/s of the pre-integrated march
    against the TF march."""
    import torch

    import oracle
    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = v.Context(dev)
    w = build_workload(args.small)
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    p = w.params(entry_exit_mode=v.EE_ANALYTIC)
    res = v.PreIntegrationTable.resolution(w.tf_width)
    step = v.sampling_step(vol, p.sampling_rate)
    src = v.PreIntegrationTable.bake_source(w.tf_keys, res)
    builds = {}
    exact = None
    for integral in (False, True):
        t_gpu = []
        for k in range(3):
            t0 = time.perf_counter()
            tbl = v.PreIntegrationTable(ctx, src, step, integral)
            t_gpu.append(time.perf_counter() - t0)
            if k < 2:
                tbl.close()
        t0 = time.perf_counter()
        ref = oracle.preint_table(src, tbl.step, integral)
        t_cpu = time.perf_counter() - t0
        equal = bool(np.array_equal(tbl.download().view(np.uint32), ref.view(np.uint32)))
        builds["integral" if integral else "exact"] = {"gpu_ms": 1e3 * statistics.median(t_gpu),
                                                        "cpu_ms": 1e3 * t_cpu, "cpu_threads": os.cpu_count(),
                                                        "equal_to_cpu_build": equal}
        if integral:
            tbl.close()
        else:
            exact = tbl
    tf.set_preintegration(exact)
    out = torch.empty((w.height, w.width, 4), dtype=torch.uint8, device=f"cuda:{dev}")
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")

    def frames(q):
        for _ in range(warmup):
            v.render_async(ctx, vol, tf, q, None, None, out, v.OUT_RGBA8)
        ctx.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            v.render_async(ctx, vol, tf, q, None, None, out, v.OUT_RGBA8)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / args.steps

    with ClockSampler(dev) as clk:
        ms_tf = frames(p)
        p.classification = v.CLASSIFY_PREINTEGRATED
        ms_pi = frames(p)
    _, st = v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA8, out)
    line = {"metric": "pre-integrated DVR frames/s, 512^3 u16 @1080p; table build ms (GPU vs CPU)",
            "value": 1000.0 / ms_pi, "unit": "frames/s", "n_gpus": ws, "steps": args.steps, "warmup": warmup,
            "ms_per_step": ms_pi, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural CT-like shells)",
            "config": {"workload": w.name + " pre-integrated", "table": [res, res], "classification":
                       "pre-integrated-cpu (exact table)", "l2": "inputs larger than L2"},
            "tf_classification_frames_per_s": 1000.0 / ms_tf, "samples_per_frame": st.samples,
            "samples_fetched_per_frame": st.samples_fetched, "table_build": builds,
            "gpu_launches": args.steps * st.kernel_launches, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line))


def run_ingest(args, warmup, ws, rank, local):
    """Volume ingest: the 512^3 uint16 CT-like volume written as a .vvd + .raw
    pair (256 MiB, in the page cache after writing), loaded by
    vrc_volume_load_vvd (file -> two pinned 64 MiB chunks -> device ->
    bricks + min/max) against a plain host read of the raw file (what a CPU
    reader does) and an upload of the same voxels from host memory."""
    import shutil

    import torch

    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = v.Context(dev)
    w = build_workload(args.small)
    tmp = tempfile.mkdtemp(prefix="vrc_ingest_")
    try:
        path = os.path.join(tmp, "ct.vvd")
        raw = v.write_vvd(path, w.voxels, spacing=w.spacing)
        nbytes = os.path.getsize(raw)
        steps = max(3, min(args.steps, 20))

        def timed(fn):
            for _ in range(warmup):
                fn()
            ts = []
            for _ in range(steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            return statistics.median(ts)

        def load():
            vol = v.Volume.load_vvd(ctx, path)
            ctx.synchronize()
            vol.close()

        def host_read():
            np.fromfile(raw, np.uint16)

        def upload():
            vol = v.Volume(ctx, w.voxels, w.spacing)
            ctx.synchronize()
            vol.close()

        t_load, t_read, t_up = timed(load), timed(host_read), timed(upload)
        vol = v.Volume.load_vvd(ctx, path)
        ref = v.Volume(ctx, w.voxels, w.spacing)
        same = vol.minmax() == ref.minmax() and vol.device_bytes == ref.device_bytes
        line = {"metric": "volume ingest GB/s (.vvd raw file -> bricked device volume with min/max)",
                "value": nbytes / t_load / 1e9, "unit": "GB/s", "n_gpus": 1, "steps": steps, "warmup": warmup,
                "ms_per_step": t_load * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u16", "data": "synthetic (seeded procedural CT-like shells, written as .vvd + .raw)",
                "config": {"workload": f"{w.dims[0]}x{w.dims[1]}x{w.dims[2]} u16 .vvd ingest", "bytes": nbytes,
                           "page_cache": "warm (file just written)"},
                "host_read_gbs": nbytes / t_read / 1e9, "upload_from_host_memory_gbs": nbytes / t_up / 1e9,
                "loaded_equals_uploaded": bool(same), "device_bytes": vol.device_bytes}
        if rank == 0:
            print(json.dumps(line))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_upsampler_layers(args, warmup, ws, rank, local):
    """Every 3x3 convolution of the upsampler at 960 x 540 (random BF16
    weights and inputs), timed with CUDA events on the tcgen05 kernel (each
    output-channel split it supports) and on the mma.sync kernel (the decoder
    inputs fused on load); one JSON line with per-layer microseconds."""
    import ctypes as C

    import torch

    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild
    vbuild.build()
    torch.cuda.set_device(local if ws > 1 else 0)
    L = v.lib()
    H0, W0 = 540, 960
    layers = [("enc1a", 16, 0, 32, 0, [1]), ("enc1b", 32, 0, 32, 0, [1]), ("enc2a", 32, 0, 64, 1, [1]),
              ("enc2b", 64, 0, 64, 1, [1]), ("bota", 64, 0, 128, 2, [1, 2]), ("botb", 128, 0, 128, 2, [2, 4]),
              ("dec2a", 128, 64, 64, 1, [2]), ("dec2b", 64, 0, 64, 1, [1]), ("dec1a", 64, 32, 32, 0, [1]),
              ("dec1b", 32, 0, 32, 0, [1]), ("head", 32, 0, 16, 0, [1])]
    steps = max(3, args.steps)

    def timeit(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            fn()
        e.record()
        e.synchronize()
        return round(a.elapsed_time(e) / steps * 1e3, 1)

    def P(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    gen = torch.Generator(device="cuda").manual_seed(0)
    result, flops = {}, {}
    for name, c0, c1, cout, lvl, splits in layers:
        H, W = H0 >> lvl, W0 >> lvl
        cin = c0 + c1
        x0 = (torch.randn((1, H, W, c0), device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
        x1 = (torch.randn((1, H, W, c1), device="cuda", generator=gen) * 0.5).to(torch.bfloat16) if c1 else None
        xh = (torch.randn((1, H // 2, W // 2, c0), device="cuda", generator=gen) * 0.5).to(torch.bfloat16) if c1 else None
        w = (torch.randn((cout, 3, 3, cin), device="cuda", generator=gen) * 0.05).to(torch.bfloat16)
        b = torch.zeros(cout, device="cuda")
        of = 1 if name == "head" else 0
        act = 0 if of else 2
        y = torch.empty((1, H, W, cout), dtype=torch.float32 if of else torch.bfloat16, device="cuda")
        r = {}
        for sp in splits:
            wtc = torch.empty_like(w)
            L.vrc_nn_weights_tc(P(w), cout, c0, c1, sp, P(wtc), None)
            r[f"tcgen05_split{sp}"] = timeit(lambda: L.vrc_nn_conv3x3_tc(P(x0), c0, P(x1), c1, 1, H, W, P(wtc), P(b),
                                                                         cout, sp, act, P(y), of, None, None))
        if c1:
            r["mma_sync_upcat"] = timeit(lambda: L.vrc_nn_conv3x3_fwd_upcat(P(xh), c0, P(x1), c1, 1, H, W, P(w), P(b),
                                                                            cout, act, P(y), of, None))
            r["upsample_for_tcgen05"] = timeit(lambda: L.vrc_nn_upsample2(P(xh), 1, H // 2, W // 2, c0, 1.0, P(x0),
                                                                          None))
        else:
            r["mma_sync"] = timeit(lambda: L.vrc_nn_conv3x3_fwd(P(x0), 1, H, W, cin, P(w), P(b), cout, act, P(y), of,
                                                               None))
        result[name] = r
        flops[name] = 2 * H * W * cout * 9 * cin
    best = {k: min(t for n, t in r.items() if not n.startswith("upsample")) for k, r in result.items()}
    line = {"metric": "upsampler convolution microseconds per layer at 960x540 (tcgen05 vs mma.sync)",
            "value": sum(best.values()), "unit": "us (sum of the faster form per layer)", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "higher_is_better": False, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic (random BF16)", "config": {"workload": "U-Net 32/64/128 layers, 960x540"},
            "layers_us": result, "tflops_best": {k: round(flops[k] / (best[k] * 1e-6) / 1e12, 1) for k in best}}
    if rank == 0:
        print(json.dumps(line))


def run_learned(args, warmup, ws, rank, local):
    """Learned form on the CT-like workload: half-resolution, half-rate march +
    U-Net (trained weights voreen_gb300/weights/upsampler_ct.npz) + 64x64
    probe tile, against the plain full render of the same frames; PSNR and
    max |d| against the plain render on held-out volume seeds."""
    import random

    import torch

    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild, learned, synth
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = v.Context(dev)
    net = learned.UNet(seed=0)
    net.load(os.path.join(ROOT, "voreen_gb300", "weights", "upsampler_ct.npz"))
    w = build_workload(args.small)  # held-out: generator seed differs from the training volumes
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    p = w.params(entry_exit_mode=v.EE_ANALYTIC)
    lr = learned.LearnedRenderer(ctx, net)
    stream = lr.stream
    ref = torch.empty((w.height, w.width, 4), dtype=torch.float32, device=f"cuda:{dev}")
    for _ in range(warmup):
        lr.render(vol, tf, p)
        lr._render_plain(vol, tf, p, ref)
    torch.cuda.synchronize()
    ctx.synchronize()
    steps = max(3, min(args.steps, 200))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    infos = []
    for _ in range(steps):
        out, info = lr.render(vol, tf, p)
        infos.append(info)
    end.record(stream)
    end.synchronize()
    ms_learned = start.elapsed_time(end) / steps
    start.record(stream)
    for _ in range(steps):
        lr._render_plain(vol, tf, p, ref)
    end.record(stream)
    end.synchronize()
    ms_plain = start.elapsed_time(end) / steps
    stages = lr.stage_times(vol, tf, p, steps)
    # quality on a few held-out views of the same volume
    prng = random.Random(4242)
    quality = []
    for i in range(4):
        wv = learned.random_view(prng, w.voxels, w.spacing, 900 + i, w.width, w.height)
        tfv = v.TransferFunction(ctx, v.TransferFunction.bake(wv.tf_keys, wv.tf_width), wv.domain)
        pv = wv.params(entry_exit_mode=v.EE_ANALYTIC)
        o, inf = lr.render(vol, tfv, pv)
        r, _ = learned.plain_frame(ctx, vol, tfv, pv)
        x0, base, _ = learned.make_pair(ctx, vol, tfv, wv.params())
        quality.append({"psnr_learned": learned.psnr(o, r), "psnr_bilinear": learned.psnr(learned.bilinear_up2(base)[0], r),
                        "max_abs": float((o.clamp(0, 1) - r.clamp(0, 1)).abs().max()), "fallback": inf["fallback"]})
        tfv.close()
    line = {"metric": "learned vs plain frames/s at the PSNR bound (40 dB), 512^3 u16 @1080p",
            "value": 1000.0 / ms_learned, "unit": "frames/s", "n_gpus": ws, "steps": steps, "warmup": warmup,
            "ms_per_step": ms_learned, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network (fp32 accumulate), f32 march", "data": "synthetic (held-out seeded volume)",
            "config": {"workload": w.name, "input_march": [w.width // 2, w.height // 2, w.sampling_rate / 2],
                       "network": "U-Net 32/64/128, 3x3, leaky ReLU", "probe": "64x64 plain tile per frame"},
            "plain_frames_per_s": 1000.0 / ms_plain, "speedup_vs_plain": ms_plain / ms_learned,
            "fallback_rate": sum(1 for i in infos if i["fallback"]) / len(infos),
            "probe_psnr_median": statistics.median(i["probe_psnr"] for i in infos),
            "stage_ms": stages,
            "quality_held_out": quality}
    if rank == 0:
        print(json.dumps(line))


def run_large(args, warmup, ws, rank, local):
    """Large bricked volume: 2048x2048x1024 uint16 (8 GiB) of 500 sparse tubes
    generated on the device, 3840x2160, rate 1.5, Phong, 2-peak 4096-entry
    TF; plain kernel timing, empty-space statistics, a parity band of rows
    against the CPU oracle, and the learned form on the same frame."""
    import torch

    import oracle
    import voreen_gb300 as v
    from voreen_gb300 import build as vbuild, learned, synth
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    dims = (1024, 1024, 512) if args.small else (2048, 2048, 1024)
    image = (1920, 1080) if args.small else (3840, 2160)
    t0 = time.time()
    vox_d = v.synth_tubes_device(dims, 500, 5001)
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    ctx = v.Context(dev)
    t0 = time.time()
    placement = v.PLACE_HOST if args.placement == "host" else v.PLACE_DEVICE
    vol = v.Volume(ctx, vox_d, (1.0, 1.0, 1.0), placement=placement)
    ctx.synchronize()
    upload_s = time.time() - t0
    if placement == v.PLACE_HOST and args.cache_gb is not None:
        vol.set_cache_limit(int(args.cache_gb * 1e9))
    if placement == v.PLACE_HOST and args.lod:
        t0 = time.time()
        vol.set_lod(args.lod_level)
        lod_build_s = time.time() - t0
    lo, hi = vol.minmax()
    keys, domain = synth.tubes_tf(5002, 2, (lo, hi))
    tf_rgba = v.TransferFunction.bake(keys, 4096)
    tf = v.TransferFunction(ctx, tf_rgba, domain)
    pos, focus, near, far = synth.orbit_camera(dims, (1.0, 1.0, 1.0), 30.0, 25.0, 1.2)
    p = v.default_params(*image)
    p.sampling_rate, p.shading, p.entry_exit_mode = 1.5, v.SHADE_PHONG, v.EE_ANALYTIC
    p.skip_cell_size = args.skip_cell  # 0: the library default (2^3 cells for this volume)
    p.camera = v.make_camera(pos, focus, near=near, far=far)
    p.light_position[:] = [*pos, 1.0]
    out = torch.empty((image[1], image[0], 4), dtype=torch.float32, device=f"cuda:{dev}")
    t0 = time.time()
    _, st = v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F, out)
    first_ms = (time.time() - t0) * 1e3  # host placement: includes filling the device brick cache
    # host placement: per-frame wall time and bricks read without a cache slot
    # while the cache refines towards the view's working set
    settle = []
    if placement == v.PLACE_HOST:
        for _ in range(6):
            t0 = time.time()
            _, sk = v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F, out)
            settle.append({"ms": (time.time() - t0) * 1e3, "kernel_ms": sk.kernel_ms, "missed": vol.cache_info()[2]})
    steady = [v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F, out)[1] for _ in range(3)]
    kms = [x.kernel_ms for x in steady]
    launches_per_frame = steady[-1].kernel_launches  # steady frames reuse occupancy and cache plan
    for _ in range(warmup):
        v.render_async(ctx, vol, tf, p, None, None, out, v.OUT_RGBA32F)
    ctx.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    steps = max(3, min(args.steps, 100))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for _ in range(steps):
            v.render_async(ctx, vol, tf, p, None, None, out, v.OUT_RGBA32F)
        end.record(stream)
        end.synchronize()
    clocks = clk.summary()
    ms = start.elapsed_time(end) / steps
    cache = None
    if placement == v.PLACE_HOST:
        cached, reach, missed_timed = vol.cache_info()
        # one frame with the cache off: every brick read over the host link
        vol.set_cache_limit(0)
        lod_on = bool(args.lod)
        if lod_on:
            vol.set_lod(False)
        _, su = v.render(ctx, vol, tf, p, None, None, v.OUT_RGBA32F, out)
        vol.set_cache_limit(int(args.cache_gb * 1e9) if args.cache_gb is not None else 2**62)
        if lod_on:
            vol.set_lod(args.lod_level)
        nb = int(np.prod(vol.brick_minmax()[2]))
        cache = {"bricks_cached": cached, "bricks_reachable": reach, "bricks_total": nb,
                 "cache_bytes": cached * (vol.host_bytes // nb), "first_frame_ms_with_fill": first_ms,
                 "uncached_kernel_ms": su.kernel_ms, "cache_limit_gb": args.cache_gb, "lod": bool(args.lod),
                 "lod_level": args.lod_level if args.lod else 0,
                 "frames_after_first": settle, "missed_in_last_timed_frame": missed_timed}
        if args.lod:
            cache["lod_build_s"] = lod_build_s
    b_alg = st.samples * 16 + st.samples_shaded * 48 + image[0] * image[1] * 4
    k_ms = statistics.median(kms)
    peak, peak_kind = measured_peaks()
    # parity band: 2 centre rows against the FP32 CPU oracle on the same entry/exit points
    e, x = v.entry_exit(ctx, vol, p)
    img_b, _ = v.render(ctx, vol, tf, w_params := p, None, None, v.OUT_RGBA32F)
    host = vox_d.cpu().numpy()
    ov = oracle.make_volume(host, (1.0, 1.0, 1.0))
    op = oracle.make_params(sampling_rate=1.5, shading=1, light_pos=pos, camera_pos=pos)
    r0 = image[1] // 2
    t1 = time.time()
    o32, s32, _ = oracle.render(ov, tf_rgba, domain, op, e, x, 32, rows=(r0, r0 + 2))
    cpu_s = time.time() - t1
    band = np.abs(img_b[r0:r0 + 2] - o32[r0:r0 + 2])
    # learned form on the same frame (weights trained on the tube family,
    # 1024x1024x512 volumes of 125 tubes): at the 40 dB bound, and with the
    # bound at 0 (never falls back) for the network's own speed and PSNR
    net = learned.UNet(seed=0)
    net.load(os.path.join(ROOT, "voreen_gb300", "weights", "upsampler_tubes.npz"))
    learned_res = {}
    for bound in (40.0, 0.0):
        lr = learned.LearnedRenderer(ctx, net, psnr_bound=bound)
        for _ in range(2):
            lr.render(vol, tf, p)
        torch.cuda.synchronize()
        ctx.synchronize()
        start.record(lr.stream)
        infos = [lr.render(vol, tf, p)[1] for _ in range(10)]
        end.record(lr.stream)
        end.synchronize()
        ms_l = start.elapsed_time(end) / 10
        o_l, _ = lr.render(vol, tf, p)
        learned_res[bound] = {"frames_per_s": 1000.0 / ms_l, "speedup_vs_plain": ms / ms_l,
                              "fallback_rate": sum(1 for i in infos if i["fallback"]) / len(infos),
                              "psnr_vs_plain": learned.psnr(o_l, out), "psnr_bound": bound}
        if bound == 0.0:
            learned_res[bound]["stage_ms"] = lr.stage_times(vol, tf, p, 5)
    line = {"metric": "frames/s & Gsamples/s, large bricked volume 2048x2048x1024 u16 @3840x2160",
            "value": 1000.0 / ms, "unit": "frames/s", "n_gpus": ws, "steps": steps, "warmup": warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (500 seeded tubes generated on the device)",
            "config": {"workload": f"{dims[0]}x{dims[1]}x{dims[2]} u16 tubes, {image[0]}x{image[1]}, rate 1.5, "
                                   "Phong, 2-peak TF", "l2": "inputs larger than L2"},
            "gsamples_per_s": st.samples / (ms * 1e-3) / 1e9, "samples_per_frame": st.samples,
            "samples_fetched_per_frame": st.samples_fetched, "shaded_samples_per_frame": st.samples_shaded,
            "skip_runs_per_frame": st.skip_runs, "kernel_ms": k_ms,
            "roofline": {"bound": "hbm", "achieved": b_alg / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": b_alg / (k_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": b_alg},
            "volume": {"voxels_bytes": int(host.nbytes), "device_bytes": vol.device_bytes,
                       "host_bytes": vol.host_bytes, "placement": args.placement, "generate_s": gen_s,
                       "upload_s": upload_s, "upload_gbs": host.nbytes / upload_s / 1e9, "brick_cache": cache},
            "parity_band": {"rows": [r0, r0 + 2], "max_abs": float(band.max()), "oracle_samples":
                            int(s32[r0:r0 + 2].sum()), "cpu_seconds": cpu_s},
            "learned": {"at_bound": learned_res[40.0], "without_fallback": learned_res[0.0],
                        "weights": "upsampler_tubes.npz (held-out tube views: 34.0 dB learned, 32.7 dB bilinear)"},
            "gpu_launches": steps * launches_per_frame, "clocks": clocks}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="256^3 / 960x540 variant for quick checks")
    ap.add_argument("--workload", default="ct",
                    choices=["ct", "mip", "blobs", "batch", "learned", "large", "preint", "upsampler_layers",
                             "ingest"],
                    help="ct: 512^3 u16 shaded DVR 1080p (default); mip: the same under MIP; blobs: 128^3 u8 "
                         "DVR 512x512; batch: 64 mixed requests in one launch; learned: upsampler vs plain; "
                         "large: 2048x2048x1024 u16 at 3840x2160; preint: pre-integrated classification; "
                         "upsampler_layers: the learned path's convolutions, tcgen05 vs mma.sync; "
                         "ingest: .vvd volume loading")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--cache-gb", type=float, default=None,
                    help="large workload, host placement: device brick cache budget (default: free memory)")
    ap.add_argument("--lod", action="store_true",
                    help="large workload, host placement: sample uncached bricks from a coarser level")
    ap.add_argument("--lod-level", type=int, default=1,
                    help="with --lod: the level sampled for uncached bricks (k: 2^-k resolution, 1..6)")
    ap.add_argument("--placement", default="device", choices=["device", "host"],
                    help="large workload: brick pool in HBM or in pinned host memory read over NVLink-C2C")
    ap.add_argument("--skip-cell", type=int, default=0, help="empty-space cell edge (0 = library default)")
    ap.add_argument("--shading", default="phong", choices=["phong", "none"], help="exploration only")
    ap.add_argument("--no-skip", action="store_true", help="disable empty-space skipping (exploration only)")
    ap.add_argument("--profile", action="store_true",
                    help="device frames only (no e2e, no CPU baseline): the command line for ncu captures")
    args = ap.parse_args()
    warmup = max(3, args.warmup)
    ws, rank, local = _dist()
    if args.impl == "reference" and rank != 0:
        return  # the CPU reference runs on rank 0 only
    if ws > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    import numpy as np

    import voreen_gb300 as v

    if args.workload == "batch":
        if rank == 0 or ws > 1:
            run_batch(args, warmup, ws, rank, local)
        return
    if args.workload == "learned":
        run_learned(args, warmup, ws, rank, local)
        return
    if args.workload == "large":
        run_large(args, warmup, ws, rank, local)
        return
    if args.workload == "preint":
        run_preint(args, warmup, ws, rank, local)
        return
    if args.workload == "upsampler_layers":
        run_upsampler_layers(args, warmup, ws, rank, local)
        return
    if args.workload == "ingest":
        run_ingest(args, warmup, ws, rank, local)
        return

    if args.impl == "reference":
        import oracle
        w = build_workload(args.small, args.workload, volume_fn=oracle.synth_volume)
    else:
        w = build_workload(args.small, args.workload)
    shading = w.shading if args.shading == "phong" else v.SHADE_NONE
    npix = w.width * w.height
    bpv = w.voxels.dtype.itemsize
    comp_name = {v.DVR: "dvr", v.MIP: "mip", v.ISO: "iso"}[w.compositing]
    config = {"workload": w.name, "volume": list(w.dims), "dtype_volume": str(w.voxels.dtype),
              "spacing": list(w.spacing), "image": [w.width, w.height], "sampling_rate": w.sampling_rate,
              "tf_width": w.tf_width, "shading": "phong" if shading == v.SHADE_PHONG else "none",
              "compositing": comp_name, "ert": 0.95 if w.compositing == v.DVR else None,
              "camera": "orbit 1.25 x box diagonal" if args.workload != "blobs" else "orbit 2.5 x box diagonal",
              "l2": "inputs larger than L2 (bricked volume > 129 MB)" if w.voxels.nbytes > 129e6 else
                    "flush: 256 MB buffer written between timed frames", "replicas": ws}
    flush_l2 = w.voxels.nbytes <= 129e6

    if args.impl == "reference":
        if rank != 0:
            return
        # the CPU arm loads nothing of the product: volume, TF bake, camera
        # and entry/exit all come from oracle/
        import oracle
        from oracle import camera as ocam
        inv = ocam.inverse_mvp(w.camera_pos, w.camera_focus, (0.0, 1.0, 0.0), w.fovy, w.near, w.far, w.width,
                               w.height, w.dims, w.spacing)
        e, x = oracle.entry_exit(inv, w.width, w.height)
        # each step renders a band of centre rows sized so the whole run takes
        # about 150 s of CPU time (at least 2 rows a step): a bounded sample
        per_step = min(args.cpu_seconds, max(0.02, 150.0 / (warmup + args.steps)))
        # bands cycle down the frame, so the timed steps cover its rows evenly
        # (centre rows carry the longest rays): full-frame time = H x the
        # summed seconds over the summed rows
        sum_dt, sum_rows, sum_samples, next_row = 0.0, 0, 0, 0
        for i in range(warmup + args.steps):
            dt, rows, samples, threads, lo = run_cpu(w, e, x, per_step / 2 if i < warmup else per_step,
                                                     start_row=next_row)
            if i >= warmup:
                sum_dt, sum_rows, sum_samples = sum_dt + dt, sum_rows + rows, sum_samples + samples
                next_row = (lo + rows) % w.height
        t_frame = sum_dt * w.height / sum_rows
        rates = [sum_samples / sum_dt / 1e9]
        fps = 1.0 / t_frame
        line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": ws,
                "steps": args.steps, "warmup": warmup, "ms_per_step": t_frame * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
                "gsamples_per_s": statistics.median(rates),
                "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": f"bands of about {rows} rows per step cycling down the {w.width}x{w.height} "
                                           f"frame ({sum_rows} rows timed in all), extrapolated to a full frame; "
                                           f"FP32 CPURaycaster restatement, OpenMP over x per row"},
                "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    p = w.params(skip_cell_size=args.skip_cell, empty_space_skipping=0 if args.no_skip else 1, shading=shading)
    import torch
    from voreen_gb300 import build as vbuild
    vbuild.build()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = v.Context(dev)
    vol = v.Volume(ctx, w.voxels, w.spacing)
    tf = v.TransferFunction(ctx, v.TransferFunction.bake(w.tf_keys, w.tf_width), w.domain)
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    # device-resident inputs: entry/exit images in HBM, RGBA8 frame in HBM
    e_host, x_host = v.entry_exit(ctx, vol, p)
    e_dev = torch.from_numpy(e_host).to(f"cuda:{dev}")
    x_dev = torch.from_numpy(x_host).to(f"cuda:{dev}")
    out_dev = torch.empty((w.height, w.width, 4), dtype=torch.uint8, device=f"cuda:{dev}")
    torch.cuda.synchronize()

    # per-frame stats (sample counts, kernel time) from untimed frames
    _, st = v.render(ctx, vol, tf, p, e_dev, x_dev, v.OUT_RGBA8, out_dev)
    samples, shaded = st.samples, st.samples_shaded
    kernel_ms = []
    for _ in range(3):
        _, st = v.render(ctx, vol, tf, p, e_dev, x_dev, v.OUT_RGBA8, out_dev)
        kernel_ms.append(st.kernel_ms)
    launches_per_frame = st.kernel_launches  # steady state: the occupancy bits are reused across frames

    if args.profile:
        for _ in range(args.steps):
            v.render_async(ctx, vol, tf, p, e_dev, x_dev, out_dev, v.OUT_RGBA8)
        ctx.synchronize()
        print(json.dumps({"profile_run": True, "samples_per_frame": samples, "kernel_ms": kernel_ms}))
        return
    for _ in range(warmup):
        v.render_async(ctx, vol, tf, p, e_dev, x_dev, out_dev, v.OUT_RGBA8)
    torch.cuda.synchronize()
    ctx.synchronize()
    _barrier(ws)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    if flush_l2:
        # the volume fits in L2: write a 256 MB buffer before each frame and
        # time each frame on its own
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(stream):
            if flush_l2:
                for a, b in evs:
                    flush.fill_(1)
                    a.record(stream)
                    v.render_async(ctx, vol, tf, p, e_dev, x_dev, out_dev, v.OUT_RGBA8)
                    b.record(stream)
            else:
                start.record(stream)
                for _ in range(args.steps):
                    v.render_async(ctx, vol, tf, p, e_dev, x_dev, out_dev, v.OUT_RGBA8)
                end.record(stream)
        torch.cuda.synchronize()
        ctx.synchronize()
    clocks = clk.summary()
    if flush_l2:
        ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    else:
        ms = start.elapsed_time(end) / args.steps
    ms, value = _whole_job(ms, ws)

    # e2e: host entry/exit in, host RGBA8 frame out, through the C ABI
    e_pin = torch.from_numpy(e_host).pin_memory().numpy()
    x_pin = torch.from_numpy(x_host).pin_memory().numpy()
    o_pin = torch.empty((w.height, w.width, 4), dtype=torch.uint8).pin_memory().numpy()
    for _ in range(2):
        v.render(ctx, vol, tf, p, e_pin, x_pin, v.OUT_RGBA8, o_pin)
    _barrier(ws)
    t0 = time.perf_counter()
    k_e2e = max(3, args.steps // 2)
    e2e_kms = [v.render(ctx, vol, tf, p, e_pin, x_pin, v.OUT_RGBA8, o_pin)[1].kernel_ms for _ in range(k_e2e)]
    e2e_ms = (time.perf_counter() - t0) * 1e3 / k_e2e
    e2e_ms = _barrier_max(e2e_ms, ws)

    b_alg = samples * 8 * bpv + shaded * 24 * bpv + npix * 4
    fetched_b = st.samples_fetched * 8 * bpv + shaded * 24 * bpv + npix * 4
    k_ms = statistics.median(kernel_ms)
    peak, peak_kind = measured_peaks()
    achieved = b_alg / (k_ms * 1e-3) / 1e9
    traffic = load_traffic() if (args.workload == "ct" and not args.small) else None
    l2_peak = v.measure_l2_read(ctx)
    l2_traffic = load_traffic("l2_bytes_per_launch") if (args.workload == "ct" and not args.small) else None

    line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
            "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": f"synthetic (seeded procedural {w.dims[0]}x{w.dims[1]}x{w.dims[2]} "
                                    f"{w.voxels.dtype} {'Gaussian blobs' if args.workload == 'blobs' else 'CT-like shells'})",
            "config": config,
            "gsamples_per_s": samples / (ms * 1e-3) / 1e9 * ws,
            "samples_per_frame": samples, "shaded_samples_per_frame": shaded,
            "samples_fetched_per_frame": st.samples_fetched, "skip_runs_per_frame": st.skip_runs,
            "kernel_ms": k_ms,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": b_alg,
                         "note": f"algorithmic bytes = {8 * bpv} B/sample + {24 * bpv} B/shaded sample + 4 B/pixel, "
                                 "counting every reference sample, also those the empty-space skipping jumps "
                                 "(so frac can pass 1); fetched_* counts only the samples the kernel read",
                         "fetched_bytes_per_launch": fetched_b,
                         "achieved_fetched": fetched_b / (k_ms * 1e-3) / 1e9,
                         "frac_fetched": fetched_b / (k_ms * 1e-3) / 1e9 / peak},
            "roofline_l2": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                            "frac": achieved / l2_peak if l2_peak > 0 else None,
                            "peak_kind": "measured in this run: 48 MB L2-resident 16-byte reads (vrc_measure_l2_read)",
                            "traffic": l2_traffic},
            "e2e": {"value": 1000.0 / e2e_ms * ws, "unit": "frames/s", "h2d_bytes_per_step": 2 * npix * 16,
                    "d2h_bytes_per_step": npix * 4, "kernel_ms": statistics.median(e2e_kms),
                    "note": "pinned host entry/exit read and RGBA8 frame written in place by the march (mapped)"},
            "gpu_launches": launches_per_frame * args.steps,
            "clocks": clocks,
            "volume_upload_bytes": int(w.voxels.nbytes), "volume_device_bytes": vol.device_bytes}

    if rank == 0 and ws == 1:
        dt, rows, s_cpu, threads, lo = run_cpu(w, e_host, x_host, args.cpu_seconds)
        cpu_fps = 1.0 / (dt * w.height / rows)
        line["cpu_baseline"] = {"value": cpu_fps, "unit": "frames/s", "cores": threads, "kind": "port",
                                "sample": f"{rows} centre rows ({s_cpu} samples) of the same frame, extrapolated "
                                          f"to {w.width}x{w.height}; FP32 CPURaycaster restatement",
                                "gsamples_per_s": s_cpu / dt / 1e9}
        line["parity"] = frame_parity(ctx, vol, tf, p, w, e_dev, x_dev, e_host, x_host, samples)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
