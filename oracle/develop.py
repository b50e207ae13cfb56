"""One complete develop through the CPU oracle, for the benchmark's CPU arm and the tests.

Test and benchmark infrastructure: nothing in the GPU library imports this.
It resolves a `workload_spec.Develop` with the oracle's own restatements of
the reference's host rules and runs every stage of the reference's CPU
pipeline in its order (crates/core/src/pipeline/orchestration.rs, the
stages of crates/core/src/cpu/stages.rs), timing each stage under the field
names of `StageTimings` (orchestration.rs:101-124):

  normalization          NormalizationContract::normalize      sensor.rs:221-277
  highlight_processing   Clip / Opposed                        crates/highlight
  demosaic               AMaZE / RCD / MHC / bilinear          crates/demosaic
  capture_sharpening     masked Richardson-Lucy                sharpening.rs:87-389
  optics                 vignetting + distortion/TCA remap     crates/optics
  resampling             exact area reduction                  resample.rs:45-113
  color_conversion       WB + camera matrix                    stages.rs:250-308
  adjustments            the global adjustment chain           stages.rs:380-528
  output_conversion      sRGB8 + histogram                     stages.rs:1028-1094, histogram.rs

The mosaic comes from the oracle's restatement of the seeded generator, equal
bit for bit to the library's.
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

import workload_spec as spec  # noqa: E402

from . import oracle as o  # noqa: E402

DETECTION_SAFETY_MARGIN = np.float32(0.987)  # crates/highlight/src/lib.rs:27
DEMOSAIC_CODES = {"bilinear": 0, "mhc": 1, "rcd": 2, "amaze": 3}
DISTORTION_CODES = {"none": 0, "poly3": 1, "poly5": 2, "ptlens": 3}
TCA_CODES = {"none": 0, "linear": 1, "poly3": 2}


def clip_levels(threshold, gains):
    """HighlightExecution::Clip (sensor.rs:413-421): threshold * margin * min(gains) / gain, in f32."""
    g = [np.float32(x) for x in gains]
    common = np.float32(np.float32(np.float32(threshold) * DETECTION_SAFETY_MARGIN) * min(g))
    return tuple(np.float32(common / x) for x in g)


def opposed_levels(threshold, as_shot):
    """HighlightExecution::Opposed (sensor.rs:422-434) and neutral_ceiling (:443-455)."""
    level = np.float32(np.float32(threshold) * DETECTION_SAFETY_MARGIN)
    g = [np.float32(x) for x in as_shot]
    common = np.float32(level * min(g))
    return (level,) * 3, tuple(np.float32(common / x) for x in g)


def capture_ceilings(highlight, threshold, gains):
    """ceilings (crates/core/src/pipeline/detail.rs:323-337)."""
    if highlight == "clip":
        g = [np.float32(x) for x in gains]
        common = np.float32(np.float32(threshold) * min(g))
        return tuple(np.float32(common / x) for x in g)
    if highlight == "opposed":
        return (np.float32(threshold),) * 3
    return (np.float32(1.0),) * 3


def mosaic(dv: spec.Develop) -> np.ndarray:
    s = dv.scene
    return o.synth_mosaic(s.width, s.height, spec.CFA_CODES[s.cfa], s.bits, s.black, s.white, s.clip_fraction,
                          s.channel_gains(), s.seed, s.blobs, s.hot_pixel_fraction)


def optics_desc(dv: spec.Develop):
    ln, s = dv.lens, dv.scene
    d = o.optics_plan(s.width, s.height, DISTORTION_CODES[ln.distortion], ln.distortion_k, TCA_CODES[ln.tca],
                      ln.tca_red, ln.tca_blue, ln.crop_factor, ln.real_focal)
    if ln.vignetting_k is not None:
        d.vignetting_model = 1
        for k, v in enumerate(ln.vignetting_k):
            d.vignetting[k] = v
    return d


class Timer:
    def __init__(self):
        self.ms = {}
        self._t = time.perf_counter()

    def lap(self, name):
        t = time.perf_counter()
        self.ms[name] = self.ms.get(name, 0.0) + 1e3 * (t - self._t)
        self._t = t


def develop(dv: spec.Develop, raw: np.ndarray, luts: dict | None = None) -> dict:
    """Develop `raw` (the scene's u16 mosaic) through the oracle.

    Returns the camera-RGB source, the Rec.2020 preview base, the adjusted
    image, the sRGB8 output, the histogram and clip counts, and the per-stage
    wall times in ms (`timings`, StageTimings names, plus `total`).
    `luts` may carry prebuilt 'base' / 'light' tables (built otherwise).
    """
    s = dv.scene
    luts = luts if luts is not None else {}
    start = time.perf_counter()
    clock = Timer()
    desc = o.sensor_desc(s.width, s.height, s.width, (0, 0, s.width, s.height), spec.CFA_CODES[s.cfa], [s.black],
                         (1, 1), [s.white])
    m, pattern = o.normalize(raw, desc)
    clock.lap("normalization")
    stats = None
    if dv.highlight == "opposed":
        det, ceiling = opposed_levels(dv.highlight_threshold, s.as_shot)
        m, stats, _, _ = o.opposed(m, pattern, det, ceiling)
    elif dv.highlight == "clip":
        m, stats = o.clip(m, pattern, clip_levels(dv.highlight_threshold, dv.wb_gains))
    highlighted = m
    clock.lap("highlight_processing")
    rgb = o.demosaic(m, pattern, s.as_shot, DEMOSAIC_CODES[dv.demosaic])
    clock.lap("demosaic")
    if dv.capture is not None:
        c = dv.capture
        rgb = o.capture(rgb, c.amount, c.radius, c.noise_protection,
                        capture_ceilings(dv.highlight, dv.highlight_threshold, dv.wb_gains), c.iterations)
    clock.lap("capture_sharpening")
    source = rgb
    if dv.lens is not None:
        rgb = o.optics_apply(optics_desc(dv), rgb)
    clock.lap("optics")
    if tuple(dv.target) != (s.width, s.height):
        rgb = o.area_reduce(rgb, dv.target)
    clock.lap("resampling")
    base = o.camera_matrix(o.white_balance(rgb, dv.wb_gains), dv.camera_to_rec2020)
    clock.lap("color_conversion")
    base_lut = luts.get("base")
    if base_lut is None and dv.base_rendering:
        base_lut = o.standard_base_lut()
    light = luts.get("light")
    if light is None and any(v != 0.0 for v in dv.light):
        light = o.light_tone_lut(*dv.light)
    x = o.adjust(base, dv.exposure_ev, base_lut, dv.tone_lut, 1.0, 0.0, dv.hsl, None, light_lut=light)
    clock.lap("adjustments")
    srgb8 = o.display_srgb8(x)
    hist, clipped = o.histogram(srgb8)
    clock.lap("output_conversion")
    timings = dict(clock.ms)
    timings["total"] = 1e3 * (time.perf_counter() - start)
    return {"highlighted": highlighted, "source": source, "base": base, "adjusted": x, "srgb8": srgb8, "hist": hist, "clipped": clipped,
            "highlight_stats": stats, "timings": timings}
