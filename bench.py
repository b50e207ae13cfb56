"""Benchmark: full-sensor 24 MP develops per second on one GB300.

Workload (the reference's full-sensor configuration): 6048x4024 RGGB u16
14-bit synthetic mosaic, ~5% clipped in Gaussian blobs; Opposed highlight;
AMaZE; masked RL capture sharpening, 10 iterations, sigma 0.7; optics (Poly5
distortion -0.02/0.005, PA vignetting, linear TCA 1.0003/0.9997); exact area
reduction to 2560x1703; WB + camera matrix; exposure +0.5 EV, 16-knot tone
curve, 8-band HSL; sRGB 8-bit + histogram.

A step is one complete develop of one mosaic. `value` is measured with the
mosaic already resident in HBM (rd_develop_device -> rd_spatial ->
rd_render_device); `e2e` goes through the host-buffer C ABI (rd_develop from
pinned host memory -> rd_spatial -> rd_render into host memory), copies
included. L2 is flushed before every timed step (outside the step's events).

Multi-GPU: images are independent, so N GPUs run N replicas; value = N x
per-GPU develops/s (max step time over ranks).

`--impl reference` times the reference algorithm on the host cores: the
reference is Rust and cannot be built here, so its CPU restatement (the
oracle) runs on a bounded band of the same workload per step.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "24MP develops/s"
UNIT = "develops/s"
KERNEL_FAMILIES = 15  # RD_KERNEL_FAMILIES of include/rd_gpu.h


def dist_setup(gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float) -> float:
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi takes a moment to start; begin the timed region once it samples.
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.02)
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes per pixel of one launch, measured with ncu on the 4096x3072 case of this workload
# (dram__bytes_read.sum + dram__bytes_write.sum); the traffic grows with the pixel count, so the
# bench workload's traffic is this figure times its pixels.
MEASURED_TRAFFIC_BPP = {
    "amaze": (34.1, "profiles/amaze_kernel_4096x3072.md"),
    "rl_iteration": (10.3, "profiles/rl_step_kernel_4096x3072.md"),
    "rl_mask": (17.1, "profiles/rl_prep_step_kernel_4096x3072.md"),
    "optics_gather": (25.0, "profiles/optics_lut_kernel_4096x3072.md"),
    "area_reduce": (14.9, "profiles/area_kernel_4096x3072.md"),
}


# Algorithmic FP32 operations per output pixel of AMaZE, from the oracle census
# (profiles/amaze_fp32_census.md), and the non-FMA FP32 issue rate of the GPU
# at its maximum SM clock (152 SMs x 128 lanes x 2.07 GHz).
AMAZE_FP32_OPS_PER_PX = 478.18
FP32_PEAK_TOPS = 152 * 128 * 2.07e9 / 1e12


# Algorithmic bytes per launch of each kernel family, per pixel of the image it covers.
def family_bytes(name: str, N: int, n: int, H: int, tw: int) -> float | None:
    table = {
        "amaze": 14.0 * N,          # u16 mosaic in, planar f32 RGB out
        "rl_iteration": 12.0 * N,   # estimate in, guide in, estimate out
        "rl_mask": 20.0 * N,        # guide + mask preparation: RGB in, guide + refined mask out
        "rl_apply": 36.0 * N,
        "vignetting": 4.0 * N,      # multiplier plane out
        "optics_gather": 28.0 * N,  # RGB + multiplier in, RGB out
        "area_reduce": 12.0 * N + 12.0 * n,  # RGB in, reduced RGB out (one pass)
        "wb_matrix": 24.0 * n,
        "color_output": 15.0 * n,
        "opposed": 6.0 * N,
        "mhc_bilinear": 14.0 * N,
        "rcd": 14.0 * N,
    }
    return table.get(name)


def family_timing(lib, h, family: str) -> tuple[float, int]:
    """Total ms and launch count of one kernel family since the last reset."""
    nm, ms, cnt = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_uint64()
    for f in range(KERNEL_FAMILIES):
        lib.rd_ctx_kernel_timing(h, f, ctypes.byref(nm), ctypes.byref(ms), ctypes.byref(cnt))
        if nm.value and nm.value.decode() == family:
            return ms.value, int(cnt.value)
    raise KeyError(family)


def rl_shape_record(W: int, H: int, radius: float) -> dict | None:
    """Row segments per strip of the RL iteration that the first (warm-up)
    develop of this shape picked by timing, beside the occupancy heuristic's."""
    from rohditor_gb300 import rl_launch_shape

    s = rl_launch_shape(W, H, radius)
    if s is None:
        return None
    return {"segments": s.segments, "default_segments": s.default_segments,
            "tuned_iteration_ms": round(s.best_ms, 4), "default_iteration_ms": round(s.default_ms, 4)}


def run_ours(args, world, rank, local, pg):
    from rohditor_gb300 import Device
    from rohditor_gb300 import _ffi
    from rohditor_gb300.workloads import full_24mp

    dev = Device(local)
    lib = dev.lib
    h = dev.handle
    wl = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight,
                   width=args.width, height=args.height)
    W, H = wl.width, wl.height
    tw, th = wl.target
    N, n = W * H, tw * th
    sensor = wl.sensor.to_c()
    detail = wl.capture.to_c()
    optics = wl.optics.to_c()
    color = wl.color.to_c()
    wb = np.ascontiguousarray(wl.color.wb_gains, dtype=np.float32)
    cam = np.ascontiguousarray(wl.color.camera_to_rec2020, dtype=np.float32)
    wbp = wb.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    camp = cam.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    d_mosaic = wl.mosaic_device(dev)
    # Pinned host copy of the same mosaic and pinned host outputs for the end-to-end leg.
    mos_bytes = 2 * N
    h_mosaic = ctypes.c_void_p()
    dev.check(lib.rd_host_alloc(mos_bytes, ctypes.byref(h_mosaic)))
    dev.check(lib.rd_copy_to_host(h, h_mosaic, ctypes.c_void_p(d_mosaic), mos_bytes))
    h_out = ctypes.c_void_p()
    dev.check(lib.rd_host_alloc(3 * n, ctypes.byref(h_out)))
    hist = np.zeros(1024, dtype=np.uint64)
    clipped = np.zeros(6, dtype=np.uint64)

    def step_device():
        src, base = ctypes.c_void_p(), ctypes.c_void_p()
        dev.check(lib.rd_develop_device(h, ctypes.c_void_p(d_mosaic), W, ctypes.byref(sensor), ctypes.byref(detail),
                                        None, ctypes.byref(src), None))
        dev.check(lib.rd_spatial(h, src, ctypes.byref(optics), tw, th, wbp, camp, ctypes.byref(base), None))
        dev.check(lib.rd_render_device(h, base, ctypes.byref(color), None))
        lib.rd_source_release(src)
        lib.rd_base_release(base)

    def step_e2e():
        src, base = ctypes.c_void_p(), ctypes.c_void_p()
        dev.check(lib.rd_develop(h, ctypes.cast(h_mosaic, ctypes.POINTER(ctypes.c_uint16)), W, ctypes.byref(sensor),
                                 ctypes.byref(detail), None, ctypes.byref(src), None))
        dev.check(lib.rd_spatial(h, src, ctypes.byref(optics), tw, th, wbp, camp, ctypes.byref(base), None))
        dev.check(lib.rd_render(h, base, ctypes.byref(color), ctypes.cast(h_out, ctypes.POINTER(ctypes.c_uint8)),
                                hist.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                clipped.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None))
        lib.rd_source_release(src)
        lib.rd_base_release(base)

    def timed(step, steps):
        total = 0.0
        per = []
        for _ in range(steps):
            dev.check(lib.rd_ctx_flush_l2(h))
            dev.check(lib.rd_ctx_event_record(h, 0))
            step()
            dev.check(lib.rd_ctx_event_record(h, 1))
            ms = ctypes.c_float()
            dev.check(lib.rd_ctx_event_elapsed(h, 0, 1, ctypes.byref(ms)))
            per.append(ms.value)
            total += ms.value
        return total, per

    for _ in range(args.warmup):
        step_device()
    dev.synchronize()
    launches0 = dev.kernel_launches
    barrier(pg)
    dev.synchronize()
    clocks = ClockSampler(local).__enter__()
    total_ms, per = timed(step_device, args.steps)
    dev.synchronize()
    launches = dev.kernel_launches - launches0
    barrier(pg)
    total_ms = max_over_ranks(pg, total_ms)
    # Per-kernel device times from extra steps with every launch bracketed by
    # events (outside the timed region: the events add work between launches).
    lib.rd_ctx_reset_kernel_timing(h)
    lib.rd_ctx_enable_kernel_timing(h, 1)
    timing_steps = min(args.steps, 10)
    timed(step_device, timing_steps)
    dev.synchronize()
    lib.rd_ctx_enable_kernel_timing(h, 0)
    families = {}
    for f in range(KERNEL_FAMILIES):
        name = ctypes.c_char_p()
        ms = ctypes.c_double()
        cnt = ctypes.c_uint64()
        lib.rd_ctx_kernel_timing(h, f, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(cnt))
        if ms.value > 0:
            families[name.value.decode()] = {"ms": ms.value, "launches": int(cnt.value)}
    # e2e through host buffers
    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    barrier(pg)
    e2e_ms, e2e_per = timed(step_e2e, args.steps)
    clocks.__exit__(None, None, None)  # sampled across both timed legs
    e2e_ms = max_over_ranks(pg, e2e_ms)

    ms_per_step = total_ms / args.steps
    value = world * args.steps / (total_ms / 1e3)
    e2e_value = world * args.steps / (e2e_ms / 1e3)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # Dominant HBM-bound kernel (largest device time among the bandwidth-bound families).
    kernels = {}
    for name, rec in families.items():
        b = family_bytes(name, N, n, H, tw)
        per_launch_ms = rec["ms"] / max(rec["launches"], 1)
        entry = {"total_ms": round(rec["ms"], 3), "launches": rec["launches"],
                 "ms_per_launch": round(per_launch_ms, 4)}
        if b is not None:
            gbs = b / (per_launch_ms / 1e3) / 1e9
            entry["algorithmic_gbs"] = round(gbs, 1)
            entry["hbm_frac"] = round(gbs / hbm_peak, 3)
        kernels[name] = entry
    step_kernel_ms = sum(r["ms"] for r in families.values()) / timing_steps
    # The dominant kernel is the family with the most device time in the timed region.
    dominant = max(families.items(), key=lambda kv: kv[1]["ms"])[0] if families else None
    roofline = None
    if dominant and family_bytes(dominant, N, n, H, tw) is not None:
        rec = families[dominant]
        per_launch_s = rec["ms"] / rec["launches"] / 1e3
        achieved = family_bytes(dominant, N, n, H, tw) / per_launch_s / 1e9
        bpp = MEASURED_TRAFFIC_BPP.get(dominant)
        roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": hbm_peak,
                    "unit": "GB/s", "frac": round(achieved / hbm_peak, 3),
                    "traffic": round(bpp[0] * N) if bpp else None,
                    "traffic_source": (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on "
                                       f"4096x3072 ({bpp[0]} B/px, {bpp[1]}), scaled to {N} px") if bpp else None,
                    "algorithmic_bytes": round(family_bytes(dominant, N, n, H, tw)),
                    "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                    else "fallback 6.8 TB/s"}
    fp32_roofline = None
    if "amaze" in families:
        rec = families["amaze"]
        per_launch_s = rec["ms"] / rec["launches"] / 1e3
        tops = AMAZE_FP32_OPS_PER_PX * N / per_launch_s / 1e12
        fp32_roofline = {"bound": "fp32", "kernel": "amaze", "achieved": round(tops, 2), "peak": round(FP32_PEAK_TOPS, 1),
                         "unit": "Top/s", "frac": round(tops / FP32_PEAK_TOPS, 3),
                         "ops_per_px": AMAZE_FP32_OPS_PER_PX,
                         "ops_source": "oracle census, profiles/amaze_fp32_census.md",
                         "peak_source": "nominal non-FMA FP32 rate at 2070 MHz (the kernel runs without FMA)"}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": f"full_24mp {W}x{H} RGGB 14-bit, {args.highlight} + {args.demosaic} + "
                               f"RL{args.iterations} + optics(poly5, PA vignetting, linear TCA) + area->{tw}x{th} "
                               f"+ WB/matrix + exposure/tone/HSL + sRGB8 + histogram",
                   "mp_per_s": round(value * N / 1e6, 1), "parallelism": f"replicas x{world}",
                   "l2": "flushed before every timed step (256 MB write outside the step events)"},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": mos_bytes,
                "d2h_bytes_per_step": 3 * n + 1024 * 8 + 6 * 8, "ms_per_step": round(e2e_ms / args.steps, 3)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "fp32_roofline": fp32_roofline,
        "kernels": kernels,
        "dominant_kernel": dominant,
        "kernel_ms_per_step": round(step_kernel_ms, 3),
        "rl_launch_shape": rl_shape_record(W, H, wl.capture.radius),
        "clocks": clocks.summary(),
    }
    lib.rd_host_free(h_mosaic)
    lib.rd_host_free(h_out)
    dev.check(lib.rd_device_free(h, ctypes.c_void_p(d_mosaic)))
    dev.close()
    if rank == 0 and not args.no_edit_latency:
        line["edit_latency"] = edit_latency(args)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_throughput(args)
    if rank == 0 and not args.no_export:
        line["export"] = export_output(args)
    if rank == 0 and args.export_stream:
        line["export_stream"] = export_stream(args, count=args.export_stream)
    # Last: the oracle's OpenMP threads stay busy for a while after a run and
    # would compete with the host threads of the latency measurements.
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, sample_rows=args.cpu_baseline_rows)
    return line


def edit_latency(args, images: int = 16, seconds: float = 2.0, rate: float = 200.0, develop_share: float = 0.1,
                 seed: int = 4) -> dict:
    """Preview edit latency, served vs plain, on one seeded Poisson trace.

    `images` 24 MP images are open; requests arrive at `rate` per second for
    `seconds`; a share are full re-develops (jittered capture amount), the rest
    preview edits of a resident base (jittered exposure, tone curve and HSL),
    with per-image increasing revisions. Served: the trace is submitted to the
    served loop (rd_server_*), latency = submit -> result with the sRGB8 image
    and histogram on the host. Plain: the same trace run in arrival order, one
    request at a time, through rd_develop/rd_spatial/rd_render on one context
    (each edit a synchronous render of its image's current base).
    """
    from rohditor_gb300 import (CaptureContract, Device, GpuPreviewProcessor, GpuSensorProcessor,
                                GpuSpatialProcessor)
    from rohditor_gb300.served import EDIT, PreviewServer
    from rohditor_gb300.workloads import full_24mp, hsl_bands, sixteen_knot_curve

    wl = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight,
                   width=args.width, height=args.height)
    dev = Device(0)
    lib = dev.lib
    mosaics = []
    for i in range(images):
        w = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight, seed=100 + i,
                      width=args.width, height=args.height)
        host = np.empty((w.height, w.width), dtype=np.uint16)
        d = w.synth_desc()
        dev.check(lib.rd_synth_mosaic(dev.handle, ctypes.byref(d),
                                      host.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))))
        mosaics.append(host)
    rng = np.random.default_rng(seed)
    trace = []
    t = 0.0
    revision = [0] * images
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        img = int(rng.integers(images))
        revision[img] += 1
        if rng.random() < develop_share:
            cap = CaptureContract(amount=float(rng.uniform(0.3, 0.7)), radius=wl.capture.radius,
                                  noise_protection=wl.capture.noise_protection, ceilings=wl.capture.ceilings,
                                  iterations=wl.capture.iterations)
            trace.append((t, 1, img, revision[img], cap))
        else:
            c = wl.color
            color = type(c)(wb_gains=c.wb_gains, camera_to_rec2020=c.camera_to_rec2020,
                            exposure_ev=float(0.5 + rng.uniform(-0.3, 0.3)), base_lut=c.base_lut,
                            tone_lut=sixteen_knot_curve(seed=int(rng.integers(1 << 30))),
                            hsl=hsl_bands(seed=int(rng.integers(1 << 30))))
            trace.append((t, 0, img, revision[img], color))

    def pct(v):
        v = np.asarray(v, dtype=np.float64)
        if v.size == 0:
            return {"p50_ms": None, "p99_ms": None, "n": 0}
        return {"p50_ms": round(float(np.percentile(v, 50)), 3), "p99_ms": round(float(np.percentile(v, 99)), 3),
                "mean_ms": round(float(v.mean()), 3), "n": int(v.size)}

    # Served.
    server = PreviewServer(0)
    for i in range(images):
        server.open(i, mosaics[i], wl.sensor, wl.capture, wl.optics, wl.target, wl.color.wb_gains,
                    wl.color.camera_to_rec2020)
    server.drain(120000)
    server.poll(4096)
    colors = [item[4].to_c() if item[1] == 0 else None for item in trace]
    t0 = time.perf_counter()
    for k, (ts, kind, img, rev, payload) in enumerate(trace):
        while time.perf_counter() - t0 < ts:
            time.sleep(0.0002)
        if kind == 0:
            server.submit_edit(img, rev, colors[k])
        else:
            server.submit_develop(img, rev, payload, wl.optics)
    server.drain(120000)
    res = server.poll(1 << 16)
    stats = server.stats()
    server.close()
    served_edits = [r["latency_ms"] for r in res if r["kind"] == EDIT and r["status"] == 0]
    served_dev = [r["latency_ms"] for r in res if r["kind"] != EDIT and r["status"] == 0]

    # Plain: one request at a time in arrival order.
    sensor_p, spatial_p, preview_p = GpuSensorProcessor(dev), GpuSpatialProcessor(dev), GpuPreviewProcessor(dev)
    bases = []
    for i in range(images):
        src = sensor_p.develop(mosaics[i], wl.sensor, wl.capture)
        bases.append(spatial_p.reduce_preview(src, wl.optics, wl.target, wl.color.wb_gains,
                                              wl.color.camera_to_rec2020))
        src.release()
    plain_edits, plain_dev = [], []
    t0 = time.perf_counter()
    for ts, kind, img, rev, payload in trace:
        while time.perf_counter() - t0 < ts:
            time.sleep(0.0002)
        if kind == 0:
            preview_p.render(bases[img], payload)
            plain_edits.append(1e3 * (time.perf_counter() - t0 - ts))
        else:
            src = sensor_p.develop(mosaics[img], wl.sensor, payload)
            base = spatial_p.reduce_preview(src, wl.optics, wl.target, wl.color.wb_gains, wl.color.camera_to_rec2020)
            src.release()
            bases[img].release()
            bases[img] = base
            plain_dev.append(1e3 * (time.perf_counter() - t0 - ts))
    for b in bases:
        b.release()
    dev.close()
    return {
        "trace": {"images": images, "image": f"{wl.width}x{wl.height}", "seconds": seconds, "rate_per_s": rate,
                  "develop_share": develop_share, "requests": len(trace), "seed": seed},
        "served": {"edit": pct(served_edits), "develop": pct(served_dev), "coalesced": stats["coalesced"],
                   "batches": stats["batches"], "batched_edits": stats["batched_edits"]},
        "plain": {"edit": pct(plain_edits), "develop": pct(plain_dev)},
    }


def batched_throughput(args, count: int = 24, lanes: int = 3) -> dict:
    """The uneven batch (rohditor_gb300.workloads.batched_uneven: 12-60 MP,
    random CFA phase, black, WB and matrices; Opposed + AMaZE + RL K=5 +
    optics + 2560-px preview, sRGB8 + histogram to the host) through
    rd_develop_batch with `lanes` concurrent lanes, and the same images one at
    a time (one lane). Host mosaics in, host outputs out, timed end to end."""
    from rohditor_gb300 import Device
    from rohditor_gb300.batch import BatchImage, PinnedBatch, develop_batch
    from rohditor_gb300.workloads import batched_uneven

    dev = Device(0)
    wls = batched_uneven(count)
    images = [BatchImage(w.mosaic(dev), w.sensor, w.capture, w.optics, w.target, w.color.wb_gains,
                         w.color.camera_to_rec2020, w.color) for w in wls]
    dev.close()
    pixels = sum(w.width * w.height for w in wls)
    # Warm-up over the whole batch: every image shape takes its first-develop
    # costs (launch-shape tuning, scratch and pool growth) outside the timing.
    develop_batch(images, lanes=lanes)
    _, _, wall = develop_batch(images, lanes=lanes)
    _, _, wall1 = develop_batch(images, lanes=1)
    # With the mosaics and outputs in pinned host memory (a decoder writing
    # into pinned buffers): one lane, concurrent lanes, and the batch as one
    # captured CUDA graph (rd_develop_batch_graph) with `chains` branches,
    # capture + instantiation timed apart.
    pinned = PinnedBatch(images)
    pinned.run(lanes=lanes)  # warm-up
    p1 = pinned.run(lanes=1)["wall_ms"]
    pl = pinned.run(lanes=lanes)["wall_ms"]
    graph = {}
    for chains in (lanes, 2 * lanes):
        g = pinned.run(lanes=chains, graph=True)
        graph[str(chains)] = {"launch_ms": round(g["launch_ms"], 1), "capture_ms": round(g["capture_ms"], 1),
                              "develops_per_s": round(count / (g["launch_ms"] / 1e3), 2),
                              "mp_per_s": round(pixels / 1e6 / (g["launch_ms"] / 1e3), 1),
                              "speedup_vs_one_lane": round(p1 / g["launch_ms"], 3)}
    pinned.close()
    pinned_runs = {"one_lane_wall_ms": round(p1, 1), "lanes_wall_ms": round(pl, 1),
                   "lanes_mp_per_s": round(pixels / 1e6 / (pl / 1e3), 1), "graph_chains": graph}
    return {"images": count, "megapixels": round(pixels / 1e6, 1), "lanes": lanes, "wall_ms": round(wall, 1),
            "develops_per_s": round(count / (wall / 1e3), 2), "mp_per_s": round(pixels / 1e6 / (wall / 1e3), 1),
            "one_lane_wall_ms": round(wall1, 1), "speedup_vs_one_lane": round(wall1 / wall, 3),
            "pinned_host": pinned_runs,
            "workload": "uneven batch: 12/24/45/60 MP, random CFA phase, Opposed + AMaZE + RL5 + optics + preview"}


def export_output(args, reps: int = 5) -> dict:
    """Full-resolution outputs of the 24 MP develop: one base at the mosaic's
    size (no area reduction), then rd_render_output_device into device buffers
    for each export format. Device time per launch of the output kernel, L2
    flushed before each; algorithmic bytes = 12 B/px planar f32 read + the
    format's bytes written."""
    from rohditor_gb300 import Device, OutputSpec
    from rohditor_gb300.workloads import full_24mp

    dev = Device(0)
    lib, h = dev.lib, dev.handle
    wl = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight,
                   width=args.width, height=args.height)
    W, H = wl.width, wl.height
    sensor, detail, optics, color = wl.sensor.to_c(), wl.capture.to_c(), wl.optics.to_c(), wl.color.to_c()
    wb = np.ascontiguousarray(wl.color.wb_gains, dtype=np.float32)
    cam = np.ascontiguousarray(wl.color.camera_to_rec2020, dtype=np.float32)
    d_mosaic = wl.mosaic_device(dev)
    src, base = ctypes.c_void_p(), ctypes.c_void_p()
    dev.check(lib.rd_develop_device(h, ctypes.c_void_p(d_mosaic), W, ctypes.byref(sensor), ctypes.byref(detail),
                                    None, ctypes.byref(src), None))
    dev.check(lib.rd_spatial(h, src, ctypes.byref(optics), W, H, wb.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                             cam.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(base), None))
    lib.rd_source_release(src)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    specs = {
        "extended_f16_p3_compress_h4": OutputSpec(format="extended_f16", primaries="display_p3",
                                                  policy="chroma_compress", headroom=4.0),
        "srgb8_clip": OutputSpec(format="srgb8"),
        "srgb16_compress_dither": OutputSpec(format="srgb16", policy="chroma_compress", dither="ordered8x8"),
        "extended_f32_srgb_clip_rotate90": OutputSpec(format="extended_f32", orientation="rotate90", headroom=2.0),
    }
    out = {}
    d_out, d_gamut = ctypes.c_void_p(), ctypes.c_void_p()
    dev.check(lib.rd_device_alloc(h, 12 * W * H, ctypes.byref(d_out)))
    dev.check(lib.rd_device_alloc(h, 64, ctypes.byref(d_gamut)))
    for name, spec in specs.items():
        oc = spec.to_c()
        bpp = {"srgb8": 3, "srgb16": 6, "extended_f32": 12, "extended_f16": 6}[spec.format]
        dev.check(lib.rd_render_output_device(h, base, ctypes.byref(color), ctypes.byref(oc), d_out, None, d_gamut,
                                              None))
        dev.synchronize()
        lib.rd_ctx_reset_kernel_timing(h)
        lib.rd_ctx_enable_kernel_timing(h, 1)
        for _ in range(reps):
            dev.check(lib.rd_ctx_flush_l2(h))
            dev.check(lib.rd_render_output_device(h, base, ctypes.byref(color), ctypes.byref(oc), d_out, None,
                                                  d_gamut, None))
        dev.synchronize()
        lib.rd_ctx_enable_kernel_timing(h, 0)
        ms, cnt = family_timing(lib, h, "display_output")
        per = ms / max(cnt, 1)
        gbs = (12 + bpp) * W * H / (per / 1e3) / 1e9
        gamut = np.zeros(5, dtype=np.uint64)
        dev.check(lib.rd_copy_to_host(h, gamut.ctypes.data_as(ctypes.c_void_p), d_gamut, 40))
        out[name] = {"ms": round(per, 4), "algorithmic_gbs": round(gbs, 1), "hbm_frac": round(gbs / hbm_peak, 3),
                     "out_bytes_per_px": bpp, "gamut": [int(v) for v in gamut]}
    dev.check(lib.rd_device_free(h, d_out))
    dev.check(lib.rd_device_free(h, d_gamut))
    lib.rd_base_release(base)
    dev.check(lib.rd_device_free(h, ctypes.c_void_p(d_mosaic)))
    dev.close()
    return {"image": f"{W}x{H}", "peak_gbs": hbm_peak, "outputs": out}


def export_stream(args, count: int = 24, window: int = 3, cap_gb: float = 60.0) -> dict:
    """The large-sensor export stream through the served loop: `count` 101.8 MP
    16-bit mosaics with hot pixels and specular blobs (workloads.large_export:
    Opposed + AMaZE + RL K = 20 + full optics) are opened in one rd_server with
    a `cap_gb` budget (each open develops and keeps the image's layers), then
    each is exported at full resolution as extended f16 (Display P3, chroma
    compression, headroom 4) plus sRGB8, into pinned host buffers reused by
    `window` exports in flight. Times are wall clock around the submissions
    and the polled results."""
    from rohditor_gb300 import Device, OutputSpec
    from rohditor_gb300 import _ffi
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hot_pixels, large_export

    wls = large_export(count)
    dev = Device(0)
    lib = dev.lib
    server = ctypes.c_void_p()
    dev.check(lib.rd_server_create(0, int(cap_gb * (1 << 30)), ctypes.byref(server)))
    W, H = wls[0].width, wls[0].height
    t0 = time.perf_counter()
    for k, wl in enumerate(wls):
        raw = hot_pixels(wl.mosaic(dev), seed=k)
        s, d, o = wl.sensor.to_c(), wl.capture.to_c(), wl.optics.to_c()
        wb = np.ascontiguousarray(wl.color.wb_gains, dtype=np.float32)
        cam = np.ascontiguousarray(CAMERA_TO_REC2020, dtype=np.float32)
        dev.check(lib.rd_server_open(server, k, raw.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), W,
                                     ctypes.byref(s), ctypes.byref(d), ctypes.byref(o), wl.target[0], wl.target[1],
                                     wb.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                     cam.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), None))
    dev.check(lib.rd_server_drain(server, 600000))
    buf = (_ffi.ServerResult * 256)()
    opened = [buf[i].status for i in range(lib.rd_server_poll(server, buf, 256, 0))]
    t1 = time.perf_counter()
    specs = [OutputSpec(format="extended_f16", primaries="display_p3", policy="chroma_compress", headroom=4.0),
             OutputSpec(format="srgb8")]
    sizes = [W * H * 6, W * H * 3]
    descs = (_ffi.OutputDesc * 2)(*[sp.to_c() for sp in specs])
    pool = []
    for _ in range(window):
        ptrs = []
        for n in sizes:
            p = ctypes.c_void_p()
            dev.check(lib.rd_host_alloc(n, ctypes.byref(p)))
            ptrs.append(p.value)
        pool.append(ptrs)
    in_flight, statuses, latencies = {}, [], []
    t2 = time.perf_counter()
    for k, wl in enumerate(wls):
        while not pool:
            n = lib.rd_server_poll(server, buf, 256, 1000)
            for i in range(n):
                if buf[i].kind == 2:
                    pool.append(in_flight.pop(buf[i].request_id))
                    statuses.append(buf[i].status)
                    latencies.append(buf[i].latency_ms)
        ptrs = pool.pop()
        dst = (ctypes.c_void_p * 2)(*ptrs)
        caps = (ctypes.c_size_t * 2)(*sizes)
        rid = ctypes.c_uint64()
        c = wl.color.to_c()
        dev.check(lib.rd_server_submit_export(server, k, 1, ctypes.byref(c), descs, 2, dst, caps, ctypes.byref(rid)))
        in_flight[rid.value] = ptrs
    while in_flight:
        n = lib.rd_server_poll(server, buf, 256, 1000)
        for i in range(n):
            if buf[i].kind == 2:
                pool.append(in_flight.pop(buf[i].request_id))
                statuses.append(buf[i].status)
                latencies.append(buf[i].latency_ms)
    t3 = time.perf_counter()
    st = _ffi.ServerStats()
    dev.check(lib.rd_server_get_stats(server, ctypes.byref(st)))
    lib.rd_server_destroy(server)
    for ptrs in pool:
        for p in ptrs:
            lib.rd_host_free(ctypes.c_void_p(p))
    dev.close()
    mp = W * H / 1e6
    return {"images": count, "image": f"{W}x{H} RGGB 16-bit, 0.5% hot pixels, specular blobs",
            "pipeline": "Opposed + AMaZE + RL20 + optics; export: extended f16 Display P3 chroma-compressed "
                        "headroom 4 + sRGB8, full resolution",
            "open_develop_s": round(t1 - t0, 2), "opens_ok": sum(1 for v in opened if v == 0),
            "export_s": round(t3 - t2, 3), "exports_ok": sum(1 for v in statuses if v == 0),
            "exports_per_s": round(count / (t3 - t2), 2), "export_mp_per_s": round(count * mp / (t3 - t2), 1),
            "export_latency_p50_ms": round(float(np.percentile(latencies, 50)), 1) if latencies else None,
            "peak_resident_gb": round(st.peak_resident_bytes / (1 << 30), 2), "cap_gb": cap_gb,
            "evictions": int(st.evictions)}


def cpu_develop_band(rows: int, args) -> tuple[float, float]:
    """Run the oracle pipeline on a `rows`-high band of the 24 MP workload; returns (seconds, fraction)."""
    from oracle import oracle as o
    from rohditor_gb300.workloads import full_24mp, preview_dimensions

    wl = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight)
    W, H = wl.width, wl.height
    rng = np.random.default_rng(5)
    # A band with the workload's statistics: smooth scene, ~5% clipped blobs, 14-bit levels.
    yy, xx = np.mgrid[0:rows, 0:W].astype(np.float32)
    scene = 0.35 + 0.2 * np.sin(xx / 97.0) * np.cos(yy / 61.0)
    blobs = ((xx % 900 - 450) ** 2 + (yy % 700 - 350) ** 2) < 110 ** 2
    scene[blobs] = 2.0
    raw = np.clip(512 + scene * 15871 + rng.normal(0, 20, scene.shape), 0, 16383).astype(np.uint16)
    odesc = o.sensor_desc(W, rows, W, (0, 0, W, rows), 0, [512.0], (1, 1), [16383.0])
    t0 = time.perf_counter()
    m, pattern = o.normalize(raw, odesc)
    if args.highlight == "opposed":
        m, _, _, _ = o.opposed(m, pattern, wl.sensor.detection_levels, wl.sensor.neutral_ceiling)
    else:
        m, _ = o.clip(m, pattern, wl.sensor.clip_levels)
    algo = {"bilinear": 0, "mhc": 1, "rcd": 2, "amaze": 3}[args.demosaic]
    rgb = o.demosaic(m, pattern, wl.sensor.demosaic_balance, algo)
    cap = wl.capture
    rgb = o.capture(rgb, cap.amount, cap.radius, cap.noise_protection, cap.ceilings, cap.iterations)
    plan = o.optics_plan(W, rows, 2, (-0.02, 0.005, 0.0), 1, (1.0003, 0, 0), (0.9997, 0, 0))
    plan.vignetting_model = 1
    for k, v in enumerate(wl.optics.vignetting_k):
        plan.vignetting[k] = v
    rgb = o.optics_apply(plan, rgb)
    tw, th = preview_dimensions(W, rows, 2560)
    base = o.camera_matrix(o.white_balance(o.area_reduce(rgb, (tw, th)), wl.color.wb_gains),
                           wl.color.camera_to_rec2020)
    c = wl.color
    x = o.adjust(base, c.exposure_ev, c.base_lut, c.tone_lut, c.saturation, c.vibrance, c.hsl, c.grading)
    o.histogram(o.display_srgb8(x))
    return time.perf_counter() - t0, rows / H


def cpu_baseline(args, sample_rows: int) -> dict:
    secs, frac = cpu_develop_band(sample_rows, args)
    cores = os.cpu_count() or 1
    return {"value": round(frac / secs, 4), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle (C++ restatement of the reference CPU pipeline, OpenMP on {cores} threads) on a "
                      f"6048x{sample_rows} band of the 24 MP workload ({frac:.3f} of a develop) in {secs:.1f} s; "
                      f"value = develop-fraction / seconds"}


def run_reference(args, world, rank, pg):
    if rank != 0:
        return None
    rows = args.cpu_rows
    times = []
    for i in range(args.warmup + args.steps):
        secs, frac = cpu_develop_band(rows, args)
        if i >= args.warmup:
            times.append(secs)
    total = sum(times)
    value = args.steps * frac / total
    cores = os.cpu_count() or 1
    cpu = {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"6048x{rows} band ({frac:.3f} of a 24 MP develop) per step through the oracle"}
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps / frac, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": f"full_24mp 6048x4024, {args.highlight} + {args.demosaic} + RL{args.iterations} + "
                               f"optics + area->2560x1703 + colour + sRGB8 + histogram (CPU restatement; the Rust "
                               f"reference cannot be built on this image)"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--highlight", default="opposed", choices=["opposed", "clip"])
    p.add_argument("--demosaic", default="amaze", choices=["amaze", "rcd", "mhc"])
    p.add_argument("--iterations", type=int, default=10)
    p.add_argument("--cpu-rows", type=int, default=256)
    p.add_argument("--width", type=int, default=6048, help="mosaic width (smaller cases for profiling)")
    p.add_argument("--height", type=int, default=4024)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-edit-latency", action="store_true", help="skip the served-vs-plain edit latency trace")
    p.add_argument("--no-batched", action="store_true", help="skip the uneven batched-develop measurement")
    p.add_argument("--no-export", action="store_true", help="skip the full-resolution output measurement")
    p.add_argument("--export-stream", type=int, default=0, metavar="N",
                   help="also run the large-sensor export stream through the served loop with N images")
    p.add_argument("--cpu-baseline-rows", type=int, default=2048,
                   help="band height of the CPU baseline sample (2048 rows = half a 24 MP develop)")
    args = p.parse_args()
    world, rank, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, world, rank, pg)
    else:
        line = run_ours(args, world, rank, local, pg)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
