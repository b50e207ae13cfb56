"""Benchmark: full-sensor 24 MP develops per second on one GB300.

Headline workload (the reference's full-sensor configuration, defined in
workload_spec.full_24mp): 6048x4024 RGGB u16 14-bit synthetic mosaic, ~5%
clipped in Gaussian blobs; Opposed highlight; AMaZE; masked RL capture
sharpening, 10 iterations, sigma 0.7; optics (Poly5 distortion -0.02/0.005,
PA vignetting, linear TCA 1.0003/0.9997); exact area reduction to 2560x1703;
WB + camera matrix; exposure +0.5 EV, 16-knot tone curve, 8-band HSL; sRGB
8-bit + histogram.

A step is one complete develop of one mosaic. `value` is measured with the
mosaic already resident in HBM (rd_develop_device -> rd_spatial ->
rd_render_device); `e2e` goes through the host-buffer C ABI (rd_develop from
pinned host memory -> rd_spatial -> rd_render into host memory), copies
included. L2 is flushed before every timed step (outside the step's events).

After the headline, rank 0 measures the other configurations of the
reference workload set, each under its own key: the 3008x2008 Clip + AMaZE
full-resolution render and the 24 MP develop with RCD and with MHC
(`configs`), the 48-image uneven batch (`batched`), the served trace over
16 mixed-size images under a 120 GB budget (`edit_latency`), the
full-resolution output formats with their PNG and JPEG files (`export`,
`export.png`; the PNG leg beside the oracle's filter selection + zlib level
6 on one core) and the 102 MP export stream
(`export_stream`); then the CPU baseline, the oracle developing the very
same mosaic on the host cores, whose outputs also give the per-stage parity
of the GPU develop (`parity`).

Multi-GPU: images are independent, so N GPUs run N replicas; value = N x
per-GPU develops/s from the max step time over ranks. `--gpus N` without a
launcher starts N ranks itself.

`--impl reference` times the reference algorithm on the host cores: the
reference is Rust and cannot be built here, so its CPU restatement (the
oracle) develops the whole seeded mosaic each step. It loads no part of the
GPU library.
"""

from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import shutil
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import workload_spec as spec  # noqa: E402

METRIC = "24MP develops/s"
UNIT = "develops/s"
KERNEL_FAMILIES = 16  # RD_KERNEL_FAMILIES of include/rd_gpu.h

# Algorithmic FP32 operations per output pixel of AMaZE, counted on the bench
# mosaic by the oracle's counting-float build (oracle/flops/census.py), and the
# non-FMA FP32 issue rate at the maximum SM clock (152 SMs x 128 lanes x 2.07
# GHz; the kernel is built without FMA contraction). No FP32 peak is measured
# for this pool, so the nominal rate is the denominator.
AMAZE_FP32_OPS_PER_PX = 478.18
FP32_PEAK_TOPS = 152 * 128 * 2.07e9 / 1e12


# ------------------------------------------------------------------ ranks
def relaunch_with_ranks(gpus: int) -> int:
    """`--gpus N` without a launcher: run this command under torch.distributed.run with N ranks."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
           "--master-addr", "127.0.0.1", "--master-port", os.environ.get("BENCH_MASTER_PORT", "29531")]
    return subprocess.call(cmd + [os.path.abspath(__file__)] + sys.argv[1:])


def dist_setup(backend: str = "gloo"):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend, init_method="env://")
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


def replica_throughput(pg, world: int, steps: int, local_ms: float) -> tuple[float, float]:
    """Whole-job units/s of `world` replicas that each ran `steps` units in `local_ms`:
    world x steps over the slowest rank's time. Returns (units/s, slowest ms)."""
    slowest = max_over_ranks(pg, local_ms)
    return world * steps / (slowest / 1e3), slowest


# ------------------------------------------------------------------ clocks
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


# ------------------------------------------------------------------ rooflines
def load_peaks() -> tuple[float, str]:
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s"


def load_traffic() -> dict:
    """DRAM bytes per pixel of one launch per kernel family, from the ncu captures in profiles/."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json")))["kernels"]
    except (OSError, ValueError, KeyError):
        return {}


def family_bytes(name: str, N: int, n: int) -> float | None:
    """Algorithmic bytes of one launch of a kernel family (N input pixels, n preview pixels)."""
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
        "opposed": 6.0 * N,         # u16 mosaic in, normalized and reconstructed f32 mosaic out
        "mhc_bilinear": 14.0 * N,
        "rcd": 14.0 * N,
    }
    return table.get(name)


FP32_BOUND = ("amaze", "rcd")


def family_timing(lib, h, family: str) -> tuple[float, int]:
    """Total ms and launch count of one kernel family since the last reset."""
    nm, ms, cnt = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_uint64()
    for f in range(KERNEL_FAMILIES):
        lib.rd_ctx_kernel_timing(h, f, ctypes.byref(nm), ctypes.byref(ms), ctypes.byref(cnt))
        if nm.value and nm.value.decode() == family:
            return ms.value, int(cnt.value)
    raise KeyError(family)


def settle_launch_shapes(b, limit: int = 16) -> int:
    """Untimed develops until the launch shapes tuned across calls are settled for this workload's
    sizes (they settle within a few develops of a shape), so that no tuning run falls inside a timed
    region; returns how many were needed (at most `limit`)."""
    from rohditor_gb300 import launch_shape

    def pending() -> bool:
        if launch_shape("color", b.tw, b.th) is None:
            return True
        if b.wl.optics is not None and launch_shape("optics", b.W, b.H) is None:
            return True
        cap = b.wl.capture
        return cap is not None and launch_shape("rl_mask", b.W, b.H, cap.radius) is None

    steps = 0
    while steps < limit and pending():
        b.step_device()
        steps += 1
    return steps


def rl_shape_record(W: int, H: int, radius: float, tw: int, th: int) -> dict | None:
    """Launch shapes the warm-up develops picked by timing, beside the heuristics' defaults: row
    segments per strip of the RL iteration and of the RL guide / mask kernel, CTAs per SM of the
    colour kernel, rows of the optics gather's tiles."""
    from rohditor_gb300 import launch_shape, rl_launch_shape

    out = {}
    s = rl_launch_shape(W, H, radius)
    if s is not None:
        out["rl_iteration"] = {"segments": s.segments, "default_segments": s.default_segments,
                               "tuned_ms": round(s.best_ms, 4), "default_ms": round(s.default_ms, 4)}
    for stage, (w, h) in (("rl_mask", (W, H)), ("color", (tw, th)), ("optics", (W, H))):
        t = launch_shape(stage, w, h, radius)
        if t is not None:
            out[stage] = {"value": t.segments, "default": t.default_segments, "tuned_ms": round(t.best_ms, 4),
                          "default_ms": round(t.default_ms, 4)}
    return out or None


# ------------------------------------------------------------------ one workload on the device
class DevelopBench:
    """One workload's develop -> spatial -> render on a device context, resident or end to end."""

    def __init__(self, dev, wl):
        self.dev, self.lib, self.h, self.wl = dev, dev.lib, dev.handle, wl
        self.W, self.H = wl.width, wl.height
        self.tw, self.th = wl.target
        self.N, self.n = self.W * self.H, self.tw * self.th
        self.sensor = wl.sensor.to_c()
        self.detail = wl.capture.to_c() if wl.capture is not None else None
        self.optics = wl.optics.to_c() if wl.optics is not None else None
        self.color = wl.color.to_c()
        self.wb = np.ascontiguousarray(wl.color.wb_gains, dtype=np.float32)
        self.cam = np.ascontiguousarray(wl.color.camera_to_rec2020, dtype=np.float32)
        self.d_mosaic = wl.mosaic_device(dev)
        self.mos_bytes = 2 * self.N
        lib = self.lib
        self.h_mosaic = ctypes.c_void_p()
        dev.check(lib.rd_host_alloc(self.mos_bytes, ctypes.byref(self.h_mosaic)))
        dev.check(lib.rd_copy_to_host(self.h, self.h_mosaic, ctypes.c_void_p(self.d_mosaic), self.mos_bytes))
        self.h_out = ctypes.c_void_p()
        dev.check(lib.rd_host_alloc(3 * self.n, ctypes.byref(self.h_out)))
        self.hist = np.zeros(1024, dtype=np.uint64)
        self.clipped = np.zeros(6, dtype=np.uint64)
        self.d2h_bytes = 3 * self.n + 1024 * 8 + 6 * 8

    def _ptrs(self):
        d = ctypes.byref(self.detail) if self.detail is not None else None
        o = ctypes.byref(self.optics) if self.optics is not None else None
        return d, o, self.wb.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), \
            self.cam.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def step_device(self):
        lib, h, dev = self.lib, self.h, self.dev
        d, o, wbp, camp = self._ptrs()
        src, base = ctypes.c_void_p(), ctypes.c_void_p()
        dev.check(lib.rd_develop_device(h, ctypes.c_void_p(self.d_mosaic), self.W, ctypes.byref(self.sensor), d,
                                        None, ctypes.byref(src), None))
        dev.check(lib.rd_spatial(h, src, o, self.tw, self.th, wbp, camp, ctypes.byref(base), None))
        dev.check(lib.rd_render_device(h, base, ctypes.byref(self.color), None))
        lib.rd_source_release(src)
        lib.rd_base_release(base)

    def step_e2e(self, keep: bool = False):
        lib, h, dev = self.lib, self.h, self.dev
        d, o, wbp, camp = self._ptrs()
        src, base = ctypes.c_void_p(), ctypes.c_void_p()
        dev.check(lib.rd_develop(h, ctypes.cast(self.h_mosaic, ctypes.POINTER(ctypes.c_uint16)), self.W,
                                 ctypes.byref(self.sensor), d, None, ctypes.byref(src), None))
        dev.check(lib.rd_spatial(h, src, o, self.tw, self.th, wbp, camp, ctypes.byref(base), None))
        dev.check(lib.rd_render(h, base, ctypes.byref(self.color), ctypes.cast(self.h_out, ctypes.POINTER(ctypes.c_uint8)),
                                self.hist.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                self.clipped.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None))
        kept = None
        if keep:
            source = np.empty((self.H, 3 * self.W), dtype=np.float32)
            dev.check(lib.rd_source_download(h, src, source.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
            b = np.empty((self.th, 3 * self.tw), dtype=np.float32)
            dev.check(lib.rd_base_download(h, base, b.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
            srgb = np.empty((self.th, 3 * self.tw), dtype=np.uint8)
            ctypes.memmove(srgb.ctypes.data, self.h_out, srgb.nbytes)
            # The normalized, highlight-processed mosaic of the same input (rd_stage_highlight).
            highlighted = np.empty((self.H, self.W), dtype=np.float32)
            stats = np.zeros(9, dtype=np.uint64)
            dev.check(lib.rd_stage_highlight(h, ctypes.cast(self.h_mosaic, ctypes.POINTER(ctypes.c_uint16)), self.W,
                                             ctypes.byref(self.sensor),
                                             highlighted.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                             stats.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
            kept = {"source": source, "base": b, "srgb8": srgb, "hist": self.hist.copy(), "highlighted": highlighted,
                    "highlight_stats": stats}
        lib.rd_source_release(src)
        lib.rd_base_release(base)
        return kept

    def timed(self, step, steps: int) -> tuple[float, list[float]]:
        lib, h, dev = self.lib, self.h, self.dev
        total, per = 0.0, []
        # No garbage-collector pause may stall the host between the launches of a step.
        gc.collect()
        gc.disable()
        try:
            for _ in range(steps):
                dev.check(lib.rd_ctx_flush_l2(h))
                dev.check(lib.rd_ctx_event_record(h, 0))
                step()
                dev.check(lib.rd_ctx_event_record(h, 1))
                ms = ctypes.c_float()
                dev.check(lib.rd_ctx_event_elapsed(h, 0, 1, ctypes.byref(ms)))
                per.append(ms.value)
                total += ms.value
        finally:
            gc.enable()
        return total, per

    def kernel_table(self, steps: int) -> tuple[dict, dict, float]:
        """Per-kernel device times from `steps` extra steps with every launch bracketed by events
        (outside any timed region: the events add work between launches)."""
        lib, h = self.lib, self.h
        lib.rd_ctx_reset_kernel_timing(h)
        lib.rd_ctx_enable_kernel_timing(h, 1)
        self.timed(self.step_device, steps)
        self.dev.synchronize()
        lib.rd_ctx_enable_kernel_timing(h, 0)
        families = {}
        for f in range(KERNEL_FAMILIES):
            name, ms, cnt = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_uint64()
            lib.rd_ctx_kernel_timing(h, f, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(cnt))
            if ms.value > 0:
                families[name.value.decode()] = {"ms": ms.value, "launches": int(cnt.value)}
        hbm_peak, _ = load_peaks()
        kernels = {}
        for name, rec in families.items():
            b = family_bytes(name, self.N, self.n)
            per_launch_ms = rec["ms"] / max(rec["launches"], 1)
            entry = {"total_ms_per_step": round(rec["ms"] / steps, 4), "launches_per_step": rec["launches"] / steps,
                     "ms_per_launch": round(per_launch_ms, 4)}
            if b is not None:
                gbs = b / (per_launch_ms / 1e3) / 1e9
                entry["algorithmic_gbs"] = round(gbs, 1)
                entry["hbm_frac"] = round(gbs / hbm_peak, 3)
            if name == "amaze":
                tops = AMAZE_FP32_OPS_PER_PX * self.N / (per_launch_ms / 1e3) / 1e12
                entry["fp32_tops"] = round(tops, 2)
                entry["fp32_frac"] = round(tops / FP32_PEAK_TOPS, 3)
            kernels[name] = entry
        kernel_ms = sum(r["ms"] for r in families.values()) / steps
        return families, kernels, kernel_ms

    def close(self):
        self.lib.rd_host_free(self.h_mosaic)
        self.lib.rd_host_free(self.h_out)
        self.dev.check(self.lib.rd_device_free(self.h, ctypes.c_void_p(self.d_mosaic)))


def rooflines(families: dict, N: int, n: int) -> tuple[dict | None, dict | None]:
    """(roofline of the dominant kernel, HBM roofline of the dominant bandwidth-bound kernel)."""
    hbm_peak, peak_src = load_peaks()
    traffic = load_traffic()

    def hbm_line(name):
        rec = families[name]
        per_launch_s = rec["ms"] / rec["launches"] / 1e3
        b = family_bytes(name, N, n)
        achieved = b / per_launch_s / 1e9
        t = traffic.get(name)
        return {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 3), "traffic": round(t["bytes_per_px"] * N) if t else None,
                "traffic_source": (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the {t['case']} "
                                   f"frame, cold L2 ({t['bytes_per_px']} B/px, profiles/{t['summary']}), times {N} px")
                if t else None,
                "algorithmic_bytes": round(b), "peak_source": peak_src}

    if not families:
        return None, None
    dominant = max(families.items(), key=lambda kv: kv[1]["ms"])[0]
    hbm_kernels = [k for k in families if k not in FP32_BOUND and family_bytes(k, N, n) is not None]
    hbm_dominant = max(hbm_kernels, key=lambda k: families[k]["ms"]) if hbm_kernels else None
    hbm = hbm_line(hbm_dominant) if hbm_dominant else None
    if dominant == "amaze":
        rec = families["amaze"]
        per_launch_s = rec["ms"] / rec["launches"] / 1e3
        tops = AMAZE_FP32_OPS_PER_PX * N / per_launch_s / 1e12
        t = traffic.get("amaze")
        primary = {"bound": "fp32", "kernel": "amaze", "achieved": round(tops, 2), "peak": round(FP32_PEAK_TOPS, 1),
                   "unit": "TFLOP/s", "frac": round(tops / FP32_PEAK_TOPS, 3),
                   "traffic": round(t["bytes_per_px"] * N) if t else None,
                   "algorithmic_bytes": round(family_bytes("amaze", N, n)),
                   "hbm_frac": round(family_bytes("amaze", N, n) / per_launch_s / 1e9 / hbm_peak, 4),
                   "ops_per_px": AMAZE_FP32_OPS_PER_PX,
                   "ops_source": "FP32 operations per pixel counted by the oracle's counting-float AMaZE build",
                   "peak_source": "nominal non-FMA FP32 rate at 2070 MHz (no FP32 peak is measured; the kernel "
                                  "runs without FMA contraction)"}
        return primary, hbm
    if dominant in hbm_kernels:
        return hbm_line(dominant), hbm
    return None, hbm


# ------------------------------------------------------------------ the GPU arm
def run_ours(args, world, rank, local, pg):
    from rohditor_gb300 import Device
    from rohditor_gb300.workloads import full_24mp

    dev = Device(local)
    wl = full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight,
                   width=args.width, height=args.height)
    b = DevelopBench(dev, wl)
    for _ in range(args.warmup):
        b.step_device()
    tuning_steps = settle_launch_shapes(b)
    dev.synchronize()
    launches0 = dev.kernel_launches
    barrier(pg)
    dev.synchronize()
    clocks = ClockSampler(local).__enter__()
    total_ms, step_ms = b.timed(b.step_device, args.steps)
    dev.synchronize()
    launches = dev.kernel_launches - launches0
    barrier(pg)
    value, total_ms = replica_throughput(pg, world, args.steps, total_ms)
    timing_steps = min(args.steps, 10)
    families, kernels, kernel_ms = b.kernel_table(timing_steps)
    # e2e through host buffers
    for _ in range(max(1, args.warmup // 2)):
        b.step_e2e()
    barrier(pg)
    e2e_local, _ = b.timed(b.step_e2e, args.steps)
    clocks.__exit__(None, None, None)  # sampled across both timed legs
    e2e_value, e2e_ms = replica_throughput(pg, world, args.steps, e2e_local)
    kept = b.step_e2e(keep=True) if rank == 0 and not args.no_cpu_baseline else None
    roofline, hbm_roofline = rooflines(families, b.N, b.n)
    dv = wl.spec
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": dv.describe(), "mp_per_s": round(value * b.N / 1e6, 1),
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed before every timed step (256 MB write outside the step events)"},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": b.mos_bytes,
                "d2h_bytes_per_step": b.d2h_bytes, "ms_per_step": round(e2e_ms / args.steps, 3)},
        "gpu_launches": int(launches),
        "step_ms": {"min": round(min(step_ms), 3), "median": round(statistics.median(step_ms), 3),
                    "max": round(max(step_ms), 3), "max_at": int(max(range(len(step_ms)), key=step_ms.__getitem__))},
        "roofline": roofline,
        "hbm_roofline": hbm_roofline,
        "kernels": kernels,
        "kernel_ms_per_step": round(kernel_ms, 3),
        "launch_shapes": rl_shape_record(b.W, b.H, wl.capture.radius, b.tw, b.th),
        "tuning_steps": tuning_steps,
        "clocks": clocks.summary(),
    }
    b.close()
    dev.close()
    if rank == 0 and not args.no_configs:
        line["configs"] = other_configs(args)
    if rank == 0 and not args.no_edit_latency:
        line["edit_latency"] = edit_latency(args)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_throughput(args, count=args.batch_images)
    if rank == 0 and not args.no_export:
        line["export"] = export_output(args)
    if rank == 0 and args.export_stream:
        line["export_stream"] = export_stream(args, count=args.export_stream)
    # Last: the oracle's OpenMP threads stay busy for a while after a run and
    # would compete with the host threads of the latency measurements.
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"], line["parity"] = cpu_baseline(dv, kept, seconds=args.cpu_baseline_seconds)
    return line


def other_configs(args, steps: int = 20) -> dict:
    """The 3008x2008 Clip + AMaZE full-resolution render and the 24 MP develop with RCD and with
    MHC: device-resident develops/s, end to end through host buffers, and per-kernel tables."""
    from rohditor_gb300 import Device
    from rohditor_gb300.workloads import full_24mp, plain_3mp

    out = {}
    cases = {"plain_3mp_clip_amaze": plain_3mp(),
             "full_24mp_rcd": full_24mp(demosaic="rcd", iterations=args.iterations),
             "full_24mp_mhc": full_24mp(demosaic="mhc", iterations=args.iterations)}
    dev = Device(0)
    for name, wl in cases.items():
        b = DevelopBench(dev, wl)
        for _ in range(3):
            b.step_device()
        settled = settle_launch_shapes(b)
        dev.synchronize()
        total, _ = b.timed(b.step_device, steps)
        _, kernels, kernel_ms = b.kernel_table(min(steps, 5))
        b.step_e2e()
        e2e, _ = b.timed(b.step_e2e, steps)
        out[name] = {"workload": wl.spec.describe(), "develops_per_s": round(steps / (total / 1e3), 2),
                     "ms_per_develop": round(total / steps, 3), "mp_per_s": round(steps * b.N / 1e6 / (total / 1e3), 1),
                     "e2e_develops_per_s": round(steps / (e2e / 1e3), 2), "kernel_ms_per_develop": round(kernel_ms, 3),
                     "kernels": kernels, "tuning_steps": settled}
        b.close()
    dev.close()
    return out


def edit_latency(args, images: int = 16, seconds: float = 2.0, rate: float = 200.0, develop_share: float = 0.1,
                 seed: int = 4, budget_gb: float = 120.0) -> dict:
    """Preview edit latency, served vs plain, on one seeded Poisson trace.

    `images` open images of the uneven batch's mixed sizes (12-60 MP, random
    CFA phase, Opposed + AMaZE + RL K=5 + optics, 2560-px preview bases);
    requests arrive at `rate` per second for `seconds`; a share are full
    re-develops (jittered capture amount), the rest preview edits of a
    resident base (jittered exposure, tone curve, HSL and grading), with
    per-image increasing revisions. Served: the trace is submitted to the
    served loop (rd_server_*) under a `budget_gb` admission budget, latency =
    submit -> result with the sRGB8 image and histogram on the host. Plain:
    the same trace run in arrival order, one request at a time, through
    rd_develop/rd_spatial/rd_render on one context (each edit a synchronous
    render of its image's current base).
    """
    from rohditor_gb300 import (CaptureContract, Device, GpuPreviewProcessor, GpuSensorProcessor,
                                GpuSpatialProcessor)
    from rohditor_gb300.served import EDIT, PreviewServer
    from rohditor_gb300.workloads import batched_uneven, hsl_bands, sixteen_knot_curve

    wls = batched_uneven(images, seed=11)
    dev = Device(0)
    mosaics = [w.mosaic(dev) for w in wls]
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
        wl = wls[img]
        if rng.random() < develop_share:
            cap = CaptureContract(amount=float(rng.uniform(0.3, 0.7)), radius=wl.capture.radius,
                                  noise_protection=wl.capture.noise_protection, ceilings=wl.capture.ceilings,
                                  iterations=wl.capture.iterations)
            trace.append((t, 1, img, revision[img], cap))
        else:
            c = wl.color
            grading = rng.uniform(-0.2, 0.2, size=(3, 3)).astype(np.float32)
            color = type(c)(wb_gains=c.wb_gains, camera_to_rec2020=c.camera_to_rec2020,
                            exposure_ev=float(c.exposure_ev + rng.uniform(-0.3, 0.3)), base_lut=c.base_lut,
                            tone_lut=sixteen_knot_curve(seed=int(rng.integers(1 << 30))),
                            hsl=hsl_bands(seed=int(rng.integers(1 << 30))), grading=grading)
            trace.append((t, 0, img, revision[img], color))

    def pct(v):
        v = np.asarray(v, dtype=np.float64)
        if v.size == 0:
            return {"p50_ms": None, "p99_ms": None, "n": 0}
        return {"p50_ms": round(float(np.percentile(v, 50)), 3), "p99_ms": round(float(np.percentile(v, 99)), 3),
                "mean_ms": round(float(v.mean()), 3), "n": int(v.size)}

    # Served.
    server = PreviewServer(0, budget_bytes=int(budget_gb * (1 << 30)))
    for i, wl in enumerate(wls):
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
            server.submit_develop(img, rev, payload, wls[img].optics)
    server.drain(120000)
    t_served = time.perf_counter() - t0
    res = server.poll(1 << 16)
    stats = server.stats()
    server.close()
    served_edits = [r["latency_ms"] for r in res if r["kind"] == EDIT and r["status"] == 0]
    served_dev = [r["latency_ms"] for r in res if r["kind"] != EDIT and r["status"] == 0]

    # Plain: one request at a time in arrival order.
    sensor_p, spatial_p, preview_p = GpuSensorProcessor(dev), GpuSpatialProcessor(dev), GpuPreviewProcessor(dev)
    bases = []
    for i, wl in enumerate(wls):
        src = sensor_p.develop(mosaics[i], wl.sensor, wl.capture)
        bases.append(spatial_p.reduce_preview(src, wl.optics, wl.target, wl.color.wb_gains,
                                              wl.color.camera_to_rec2020))
        src.release()
    plain_edits, plain_dev = [], []
    t0 = time.perf_counter()
    for ts, kind, img, rev, payload in trace:
        while time.perf_counter() - t0 < ts:
            time.sleep(0.0002)
        wl = wls[img]
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
    t_plain = time.perf_counter() - t0
    for b in bases:
        b.release()
    dev.close()
    sizes = sorted({f"{w.width}x{w.height}" for w in wls})
    done = len(served_edits) + len(served_dev)
    return {
        "trace": {"images": images, "sizes": sizes, "seconds": seconds, "rate_per_s": rate,
                  "develop_share": develop_share, "requests": len(trace), "seed": seed, "budget_gb": budget_gb},
        "served": {"edit": pct(served_edits), "develop": pct(served_dev), "coalesced": stats["coalesced"],
                   "batches": stats["batches"], "batched_edits": stats["batched_edits"],
                   "completed_per_s": round(done / t_served, 1), "evictions": stats.get("evictions")},
        "plain": {"edit": pct(plain_edits), "develop": pct(plain_dev),
                  "completed_per_s": round((len(plain_edits) + len(plain_dev)) / t_plain, 1)},
    }


def batched_throughput(args, count: int = 48, lanes: int = 3) -> dict:
    """The uneven batch (workload_spec.batched_uneven: 12-60 MP, random CFA
    phase, black, WB and matrices; Opposed + AMaZE + RL K=5 + optics + 2560-px
    preview, sRGB8 + histogram to the host) through rd_develop_batch with
    `lanes` concurrent lanes, the same images one at a time (one lane), and the
    batch as one captured CUDA graph, and stage by stage with one AMaZE launch
    over the tiles of all images (rd_develop_batch_flat). Host mosaics in, host
    outputs out, timed end to end."""
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
    # Stage by stage, with one AMaZE launch over the tiles of all images.
    develop_batch(images, lanes=lanes, flat=True)
    _, _, wall_flat = develop_batch(images, lanes=lanes, flat=True)
    # With the mosaics and outputs in pinned host memory (a decoder writing
    # into pinned buffers): one lane, concurrent lanes, and the batch as one
    # captured CUDA graph (rd_develop_batch_graph) with `chains` branches,
    # capture + instantiation timed apart.
    pinned = PinnedBatch(images)
    pinned.run(lanes=lanes)  # warm-up
    p1 = pinned.run(lanes=1)["wall_ms"]
    pl = pinned.run(lanes=lanes)["wall_ms"]
    pf = pinned.run(lanes=lanes, flat=True)["wall_ms"]
    graph = {}
    for chains in (lanes, 2 * lanes):
        g = pinned.run(lanes=chains, graph=True)
        graph[str(chains)] = {"launch_ms": round(g["launch_ms"], 1), "capture_ms": round(g["capture_ms"], 1),
                              "develops_per_s": round(count / (g["launch_ms"] / 1e3), 2),
                              "mp_per_s": round(pixels / 1e6 / (g["launch_ms"] / 1e3), 1),
                              "speedup_vs_one_lane": round(p1 / g["launch_ms"], 3)}
    # The stage-by-stage batch as one captured graph (rd_develop_batch_flat_graph).
    pinned.run(lanes=lanes, graph=True, flat=True)  # warm-up
    fg = pinned.run(lanes=lanes, graph=True, flat=True)
    flat_graph = {"launch_ms": round(fg["launch_ms"], 1), "capture_ms": round(fg["capture_ms"], 1),
                  "develops_per_s": round(count / (fg["launch_ms"] / 1e3), 2),
                  "mp_per_s": round(pixels / 1e6 / (fg["launch_ms"] / 1e3), 1),
                  "speedup_vs_one_lane": round(p1 / fg["launch_ms"], 3)}
    pinned.close()
    pinned_runs = {"one_lane_wall_ms": round(p1, 1), "lanes_wall_ms": round(pl, 1),
                   "lanes_mp_per_s": round(pixels / 1e6 / (pl / 1e3), 1), "flat_wall_ms": round(pf, 1),
                   "flat_mp_per_s": round(pixels / 1e6 / (pf / 1e3), 1),
                   "flat_speedup_vs_one_lane": round(p1 / pf, 3), "graph_chains": graph, "flat_graph": flat_graph}
    return {"images": count, "megapixels": round(pixels / 1e6, 1), "lanes": lanes, "wall_ms": round(wall, 1),
            "develops_per_s": round(count / (wall / 1e3), 2), "mp_per_s": round(pixels / 1e6 / (wall / 1e3), 1),
            "one_lane_wall_ms": round(wall1, 1), "speedup_vs_one_lane": round(wall1 / wall, 3),
            "flat": {"wall_ms": round(wall_flat, 1), "develops_per_s": round(count / (wall_flat / 1e3), 2),
                     "mp_per_s": round(pixels / 1e6 / (wall_flat / 1e3), 1),
                     "speedup_vs_one_lane": round(wall1 / wall_flat, 3)},
            "pinned_host": pinned_runs,
            "workload": f"uneven batch of {count}: 12/24/45/60 MP, random CFA phase, Opposed + AMaZE + RL5 + optics "
                        f"+ preview"}


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
    hbm_peak, _ = load_peaks()
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
    for name, sp in specs.items():
        oc = sp.to_c()
        bpp = {"srgb8": 3, "srgb16": 6, "extended_f32": 12, "extended_f16": 6}[sp.format]
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
    png = png_files(dev, base, color, specs, d_out, d_gamut, W, H, reps)
    dev.check(lib.rd_device_free(h, d_out))
    dev.check(lib.rd_device_free(h, d_gamut))
    lib.rd_base_release(base)
    dev.check(lib.rd_device_free(h, ctypes.c_void_p(d_mosaic)))
    dev.close()
    return {"image": f"{W}x{H}", "peak_gbs": hbm_peak, "outputs": out, "png": png}


def png_files(dev, base, color, specs, d_out, d_gamut, W: int, H: int, reps: int) -> dict:
    """PNG files of the 8-bit and 16-bit outputs (export::encode's PNG arms).
    Resident: rd_encode_png_device from the output rows in HBM to a file in
    HBM, device time of the encoder's four kernels per file, L2 flushed before
    each. End to end: rd_encode_png from host rows to host bytes (wall clock,
    upload and readback included). CPU: the oracle's filter selection plus
    zlib level 6 on one core over the same 8-bit rows (one pass)."""
    from rohditor_gb300 import PngEncoder

    lib, h = dev.lib, dev.handle
    enc = PngEncoder(dev)
    result = {}
    for name, depth in (("srgb8_clip", 8), ("srgb16_compress_dither", 16)):
        oc = specs[name].to_c()
        dev.check(lib.rd_render_output_device(h, base, ctypes.byref(color), ctypes.byref(oc), d_out, None, d_gamut,
                                              None))
        cap = int(lib.rd_png_bound(W, H, depth, 0, 0))
        d_png, d_size = ctypes.c_void_p(), ctypes.c_void_p()
        dev.check(lib.rd_device_alloc(h, cap, ctypes.byref(d_png)))
        dev.check(lib.rd_device_alloc(h, 16, ctypes.byref(d_size)))

        def encode():
            dev.check(lib.rd_encode_png_device(h, d_out, W, H, 3 * W, depth, None, 0, None, 0, d_png, cap, d_size))

        encode()
        dev.synchronize()
        lib.rd_ctx_reset_kernel_timing(h)
        lib.rd_ctx_enable_kernel_timing(h, 1)
        for _ in range(reps):
            dev.check(lib.rd_ctx_flush_l2(h))
            encode()
        dev.synchronize()
        lib.rd_ctx_enable_kernel_timing(h, 0)
        ms, launches = family_timing(lib, h, "file_encode")
        per = ms / reps
        size = np.zeros(1, dtype=np.uint64)
        dev.check(lib.rd_copy_to_host(h, size.ctypes.data_as(ctypes.c_void_p), d_size, 8))
        dtype = np.uint8 if depth == 8 else np.uint16
        rows = np.empty((H, W, 3), dtype=dtype)
        dev.check(lib.rd_copy_to_host(h, rows.ctypes.data_as(ctypes.c_void_p), d_out, rows.nbytes))
        enc.encode(rows)
        t0 = time.perf_counter()
        for _ in range(reps):
            data = enc.encode(rows)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
        entry = {"ms": round(per, 4), "launches_per_file": launches // max(reps, 1),
                 "mp_per_s": round(W * H / (per / 1e3) / 1e6, 1),
                 "input_gbs": round(rows.nbytes / (per / 1e3) / 1e9, 1),
                 "file_bytes": int(size[0]), "ratio": round(int(size[0]) / rows.nbytes, 4),
                 "e2e_ms": round(e2e_ms, 3), "e2e_h2d_bytes": rows.nbytes, "e2e_d2h_bytes": len(data)}
        if depth == 8:
            import zlib

            from oracle import oracle as orc

            t0 = time.perf_counter()
            z = zlib.compress(orc.png_filter(rows), 6)
            entry["cpu_baseline"] = {"ms": round((time.perf_counter() - t0) * 1e3, 1), "cores": 1, "kind": "port",
                                     "sample": "the whole 8-bit frame once: oracle filter selection + zlib level 6",
                                     "idat_bytes": len(z)}
        result[name] = entry
        dev.check(lib.rd_device_free(h, d_png))
        dev.check(lib.rd_device_free(h, d_size))
        if depth == 8:
            result["jpeg_q90"] = jpeg_file(dev, d_out, rows, W, H, reps)
    return result


def jpeg_file(dev, d_out, rows, W: int, H: int, reps: int, quality: int = 90) -> dict:
    """JPEG file of the 8-bit output (export::encode's JPEG arm): rd_encode_jpeg_device
    from the rows in HBM, the encoder's kernel time per file (L2 flushed before
    each) and its wall time (it reads the symbol counts back once to build the
    Huffman tables); end to end through rd_encode_jpeg from host rows."""
    from rohditor_gb300 import JpegEncoder

    lib, h = dev.lib, dev.handle
    cap = int(lib.rd_jpeg_bound(W, H, 0, 0))
    d_file, d_size = ctypes.c_void_p(), ctypes.c_void_p()
    dev.check(lib.rd_device_alloc(h, cap, ctypes.byref(d_file)))
    dev.check(lib.rd_device_alloc(h, 16, ctypes.byref(d_size)))

    def encode():
        dev.check(lib.rd_encode_jpeg_device(h, d_out, W, H, 3 * W, quality, None, 0, None, 0, d_file, cap, d_size))

    encode()
    dev.synchronize()
    lib.rd_ctx_reset_kernel_timing(h)
    lib.rd_ctx_enable_kernel_timing(h, 1)
    wall = 0.0
    for _ in range(reps):
        dev.check(lib.rd_ctx_flush_l2(h))
        dev.synchronize()
        t0 = time.perf_counter()
        encode()
        dev.synchronize()
        wall += time.perf_counter() - t0
    lib.rd_ctx_enable_kernel_timing(h, 0)
    ms, launches = family_timing(lib, h, "file_encode")
    size = np.zeros(1, dtype=np.uint64)
    dev.check(lib.rd_copy_to_host(h, size.ctypes.data_as(ctypes.c_void_p), d_size, 8))
    enc = JpegEncoder(dev)
    enc.encode(rows, quality)
    t0 = time.perf_counter()
    for _ in range(reps):
        data = enc.encode(rows, quality)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    dev.check(lib.rd_device_free(h, d_file))
    dev.check(lib.rd_device_free(h, d_size))
    per = ms / reps
    return {"quality": quality, "kernel_ms": round(per, 4), "wall_ms": round(wall * 1e3 / reps, 4),
            "launches_per_file": launches // max(reps, 1), "mp_per_s": round(W * H / (per / 1e3) / 1e6, 1),
            "file_bytes": int(size[0]), "bits_per_px": round(8.0 * int(size[0]) / (W * H), 3),
            "e2e_ms": round(e2e_ms, 3), "e2e_h2d_bytes": rows.nbytes, "e2e_d2h_bytes": len(data)}


def export_stream(args, count: int = 24, window: int = 3, cap_gb: float = 60.0) -> dict:
    """The large-sensor export stream through the served loop: `count` 101.8 MP
    16-bit mosaics with hot pixels and specular blobs (workload_spec.large_export:
    Opposed + AMaZE + RL K = 20 + full optics) are opened in one rd_server with
    a `cap_gb` budget (each open develops and keeps the image's layers), then
    each is exported at full resolution as extended f16 (Display P3, chroma
    compression, headroom 4) plus sRGB8, into pinned host buffers reused by
    `window` exports in flight. Times are wall clock around the submissions
    and the polled results."""
    from rohditor_gb300 import Device, OutputSpec
    from rohditor_gb300 import _ffi
    from rohditor_gb300.workloads import large_export

    wls = large_export(count)
    dev = Device(0)
    lib = dev.lib
    server = ctypes.c_void_p()
    dev.check(lib.rd_server_create(0, int(cap_gb * (1 << 30)), ctypes.byref(server)))
    W, H = wls[0].width, wls[0].height
    raws = [wl.mosaic(dev) for wl in wls]
    t0 = time.perf_counter()
    for k, wl in enumerate(wls):
        raw = raws[k]
        s, d, o = wl.sensor.to_c(), wl.capture.to_c(), wl.optics.to_c()
        wb = np.ascontiguousarray(wl.color.wb_gains, dtype=np.float32)
        cam = np.ascontiguousarray(wl.color.camera_to_rec2020, dtype=np.float32)
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
            "develops_per_s": round(count / (t1 - t0), 2),
            "export_s": round(t3 - t2, 3), "exports_ok": sum(1 for v in statuses if v == 0),
            "exports_per_s": round(count / (t3 - t2), 2), "export_mp_per_s": round(count * mp / (t3 - t2), 1),
            "export_latency_p50_ms": round(float(np.percentile(latencies, 50)), 1) if latencies else None,
            "peak_resident_gb": round(st.peak_resident_bytes / (1 << 30), 2), "cap_gb": cap_gb,
            "evictions": int(st.evictions)}


# ------------------------------------------------------------------ the CPU side
def probe_cargo() -> str:
    """The reference's own bench needs cargo; record whether this host has it."""
    path = shutil.which("cargo")
    if not path:
        return "cargo absent on this host (the Rust reference and its pipeline_stages bench cannot be built)"
    try:
        return subprocess.run([path, "--version"], capture_output=True, text=True, timeout=20).stdout.strip()
    except (OSError, subprocess.TimeoutExpired) as e:
        return f"cargo present but failed: {e}"


def native_libraries() -> list[str]:
    """Shared libraries of this repository mapped into this process."""
    found = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1] if line.strip() else ""
            if path.startswith(ROOT) and path.endswith(".so"):
                found.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(found)


def oracle_develops(dv, raw, steps: int, warmup: int = 1) -> tuple[list[float], dict, dict]:
    """`warmup` + `steps` whole develops of `raw` through the oracle; returns the per-step seconds,
    the median per-stage ms (StageTimings names) and the last develop's outputs."""
    from oracle import develop as od
    from oracle import oracle as o

    luts = {"base": o.standard_base_lut()}
    secs, stages, res = [], {}, None
    for i in range(warmup + steps):
        t = time.perf_counter()
        res = od.develop(dv, raw, luts)
        dt = time.perf_counter() - t
        if i >= warmup:
            secs.append(dt)
            for k, v in res["timings"].items():
                stages.setdefault(k, []).append(v)
    return secs, {k: round(statistics.median(v), 1) for k, v in stages.items()}, res


def parity_summary(dv, gpu: dict, ref: dict) -> dict:
    """Per-stage agreement of one GPU develop with the oracle on the same mosaic, each stage fed
    the GPU's own output of the stage before (the tolerances of the tests), and the chained
    spread (the oracle fed only its own outputs)."""
    from oracle import develop as od
    from oracle import oracle as o

    def same(a, b):
        return bool(a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32)))

    out = {}
    dh = np.abs(gpu["highlighted"] - ref["highlighted"])
    out["highlight"] = {"stats_exact": bool(np.array_equal(gpu["highlight_stats"], ref["highlight_stats"])),
                        "max_abs": float(dh.max()), "samples_differing": int((dh > 0).sum()), "bound": 1e-4,
                        "ok": float(dh.max()) <= 1e-4}
    cap = dv.capture
    pattern = spec.CFA_CODES[dv.scene.cfa]
    rgb = o.demosaic(gpu["highlighted"], pattern, dv.scene.as_shot, od.DEMOSAIC_CODES[dv.demosaic])
    rgb = o.capture(rgb, cap.amount, cap.radius, cap.noise_protection,
                    od.capture_ceilings(dv.highlight, dv.highlight_threshold, dv.wb_gains), cap.iterations)
    out["demosaic_capture"] = {"bit_exact": same(gpu["source"], rgb), "max_abs": float(np.max(np.abs(gpu["source"] - rgb)))}
    base = o.optics_apply(od.optics_desc(dv), gpu["source"])
    base = o.camera_matrix(o.white_balance(o.area_reduce(base, dv.target), dv.wb_gains), dv.camera_to_rec2020)
    out["spatial"] = {"bit_exact": same(gpu["base"], base), "max_abs": float(np.max(np.abs(gpu["base"] - base)))}
    light = o.light_tone_lut(*dv.light) if any(v != 0.0 for v in dv.light) else None
    x = o.adjust(gpu["base"], dv.exposure_ev, o.standard_base_lut() if dv.base_rendering else None, dv.tone_lut, 1.0,
                 0.0, dv.hsl, None, light_lut=light)
    d8 = np.abs(gpu["srgb8"].astype(np.int16) - o.display_srgb8(x).astype(np.int16))
    out["colour_srgb8"] = {"max_lsb": int(d8.max()), "frac_differing": float((d8 > 0).mean()),
                           "ok": int(d8.max()) <= 1 and float((d8 > 0).mean()) <= 1e-3}
    own_hist, _ = o.histogram(gpu["srgb8"])
    out["histogram_of_own_output"] = {"exact": bool(np.array_equal(gpu["hist"], own_hist))}
    dc = np.abs(gpu["source"] - ref["source"])
    out["chained_developed_rgb"] = {
        "max_abs": float(dc.max()),
        "frac_outside_2e-5(1+|x|)": float((dc > 2e-5 * (1.0 + np.abs(ref["source"]))).mean()),
        "note": "oracle fed only its own outputs: last-bit Opposed differences move some AMaZE decisions"}
    return out


def cpu_baseline(dv, kept: dict | None, seconds: float = 10.0) -> tuple[dict, dict | None]:
    """The oracle developing the same seeded mosaic (generated by the oracle's own generator) on all
    host cores, repeated for about `seconds`; with the GPU's outputs of that mosaic, the parity."""
    from oracle import develop as od

    raw = od.mosaic(dv)
    # One develop to learn the time, then as many as fit in `seconds` (at least 2).
    first, _, _ = oracle_develops(dv, raw, steps=1, warmup=0)
    reps = max(2, int(seconds / max(first[0], 1e-3)))
    secs, stages, res = oracle_develops(dv, raw, steps=reps, warmup=0)
    cores = os.cpu_count() or 1
    cpu = {"value": round(len(secs) / sum(secs), 4), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{len(secs)} whole develops of the same seeded {dv.scene.width}x{dv.scene.height} mosaic through "
                     f"the oracle (C++ restatement of the reference CPU pipeline, OpenMP on {cores} threads), "
                     f"{sum(secs):.1f} s", "stage_ms": stages, "cargo": probe_cargo()}
    parity = parity_summary(dv, kept, res) if kept is not None else None
    return cpu, parity


def run_reference(args, world, rank, pg):
    """The reference algorithm on the host cores: the oracle develops the whole headline mosaic each step."""
    if rank != 0:
        return None
    from oracle import develop as od

    dv = spec.full_24mp(demosaic=args.demosaic, iterations=args.iterations, highlight=args.highlight,
                        width=args.width, height=args.height)
    raw = od.mosaic(dv)
    secs, stages, _ = oracle_develops(dv, raw, steps=args.steps, warmup=args.warmup)
    total = sum(secs)
    value = args.steps / total
    cores = os.cpu_count() or 1
    cpu = {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"whole {dv.scene.width}x{dv.scene.height} develop of the same seeded mosaic per step through the "
                     f"oracle (the Rust reference cannot be built: {probe_cargo()})"}
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": dv.describe(), "mp_per_s": round(value * dv.scene.width * dv.scene.height / 1e6, 2),
                   "parallelism": "host cores (OpenMP), rank 0 only"},
        "cpu_baseline": cpu,
        "stage_ms": stages,
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_so_loaded": native_libraries(),
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
    p.add_argument("--width", type=int, default=6048, help="mosaic width (smaller cases for profiling)")
    p.add_argument("--height", type=int, default=4024)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the 3 MP, RCD and MHC configurations")
    p.add_argument("--no-edit-latency", action="store_true", help="skip the served-vs-plain edit latency trace")
    p.add_argument("--no-batched", action="store_true", help="skip the uneven batched-develop measurement")
    p.add_argument("--no-export", action="store_true", help="skip the full-resolution output measurement")
    p.add_argument("--batch-images", type=int, default=48, help="images in the uneven batch")
    p.add_argument("--export-stream", type=int, default=24, metavar="N",
                   help="images in the large-sensor export stream through the served loop (0 skips it)")
    p.add_argument("--cpu-baseline-seconds", type=float, default=10.0,
                   help="about how long the CPU baseline develops the mosaic")
    args = p.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_with_ranks(args.gpus))
    world, rank, local, pg = dist_setup()
    if world != args.gpus:
        print(f"bench: --gpus {args.gpus} but {world} ranks were launched", file=sys.stderr)
        sys.exit(2)
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
