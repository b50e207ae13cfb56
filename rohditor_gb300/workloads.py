"""Synthetic workloads of the sensor-development benchmarks.

Each workload is a seeded synthetic scene plus the resolved contracts the
pipeline consumes. Shapes, bit depths, levels and edit settings follow the
benchmark configurations of the reference workloads:

  plain_3mp   3008x2008 RGGB 14-bit (black 512, white 16383), ~2% clipped,
              Clip + AMaZE, WB (2.0, 1.0, 1.6), fixed camera matrix, no
              sharpening or optics, full-resolution sRGB8 + histogram.
  full_24mp   6048x4024 RGGB 14-bit, ~5% clipped in Gaussian blobs, Opposed,
              AMaZE (or RCD / MHC), 10-iteration RL (sigma 0.7), Poly5
              distortion (-0.02, 0.005), PA vignetting, linear TCA
              1.0003 / 0.9997, area reduction to a 2560 px long edge, WB +
              matrix, exposure +0.5 EV, 16-knot tone curve, 8-band HSL.

Scenes come from the library's counter-based generator, so a mosaic is a
pure function of (shape, seed) on every machine.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _ffi
from .processor import (CaptureContract, ColorContract, Device, OpticsExecution, SensorDescription, clip_levels,
                        opposed_levels, standard_base_lut)

# A fixed camera -> linear Rec.2020 matrix (rows sum to 1: neutral stays neutral).
CAMERA_TO_REC2020 = (1.62, -0.47, -0.15, -0.19, 1.44, -0.25, 0.02, -0.38, 1.36)


def preview_dimensions(width: int, height: int, max_long_edge: int) -> tuple[int, int]:
    """preview_dimensions (crates/core/src/cpu/stages.rs:112-148)."""
    long_edge = max(width, height)
    if long_edge <= max_long_edge:
        return width, height

    def scale(d: int) -> int:
        return min(max((d * max_long_edge + long_edge // 2) // long_edge, 2), d)

    return scale(width), scale(height)


def monotone_curve_lut(knots: np.ndarray, size: int = 4096) -> np.ndarray:
    """Tone-curve LUT over linear 0..1 from knots via monotone cubic (Fritsch-Carlson) interpolation."""
    x = knots[:, 0].astype(np.float64)
    y = knots[:, 1].astype(np.float64)
    h = np.diff(x)
    delta = np.diff(y) / h
    m = np.zeros_like(y)
    m[0], m[-1] = delta[0], delta[-1]
    for k in range(1, len(x) - 1):
        if delta[k - 1] * delta[k] <= 0:
            m[k] = 0.0
        else:
            w1, w2 = 2 * h[k] + h[k - 1], h[k] + 2 * h[k - 1]
            m[k] = (w1 + w2) / (w1 / delta[k - 1] + w2 / delta[k])
    t = np.linspace(0.0, 1.0, size)
    idx = np.clip(np.searchsorted(x, t, side="right") - 1, 0, len(x) - 2)
    s = (t - x[idx]) / h[idx]
    h00, h10 = 2 * s**3 - 3 * s**2 + 1, s**3 - 2 * s**2 + s
    h01, h11 = -2 * s**3 + 3 * s**2, s**3 - s**2
    v = h00 * y[idx] + h10 * h[idx] * m[idx] + h01 * y[idx + 1] + h11 * h[idx] * m[idx + 1]
    return np.clip(v, 0.0, 1.0).astype(np.float32)


def sixteen_knot_curve(seed: int = 7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, 16)
    base = x ** 0.9
    bump = 0.04 * np.sin(np.pi * x) * rng.uniform(0.5, 1.0)
    y = np.clip(base + bump, 0.0, 1.0)
    y = np.maximum.accumulate(y)
    y[0], y[-1] = 0.0, 1.0
    return monotone_curve_lut(np.stack([x, y], axis=1))


def hsl_bands(seed: int = 11) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.3, 0.3, size=(8, 3)).astype(np.float32)


@dataclass
class Workload:
    name: str
    width: int
    height: int
    cfa: str
    bits: int
    black: float
    white: float
    clip_fraction: float
    blobs: bool
    as_shot: tuple[float, float, float]
    sensor: SensorDescription
    capture: CaptureContract | None
    optics: OpticsExecution | None
    target: tuple[int, int]
    color: ColorContract
    seed: int

    def synth_desc(self) -> _ffi.SynthDesc:
        d = _ffi.SynthDesc()
        d.width, d.height, d.cfa, d.bits = self.width, self.height, _ffi.CFA[self.cfa], self.bits
        d.black, d.white, d.clip_fraction = self.black, self.white, self.clip_fraction
        # The sensor's channel response is the inverse of its as-shot WB.
        for c in range(3):
            d.gains[c] = min(self.as_shot) / self.as_shot[c]
        d.seed = self.seed
        d.highlight_blobs = 1 if self.blobs else 0
        return d

    def mosaic(self, device: Device) -> np.ndarray:
        """The seeded u16 mosaic [height][width], generated on the device."""
        out = np.empty((self.height, self.width), dtype=np.uint16)
        d = self.synth_desc()
        device.check(device.lib.rd_synth_mosaic(device.handle, ctypes.byref(d),
                                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))))
        return out

    def mosaic_device(self, device: Device) -> int:
        """Generate the mosaic straight into device memory; returns the device pointer."""
        ptr = ctypes.c_void_p()
        device.check(device.lib.rd_device_alloc(device.handle, 2 * self.width * self.height, ctypes.byref(ptr)))
        d = self.synth_desc()
        device.check(device.lib.rd_synth_mosaic_device(device.handle, ctypes.byref(d), ptr))
        return ptr.value


def plain_3mp(seed: int = 1) -> Workload:
    wb = (2.0, 1.0, 1.6)
    sensor = SensorDescription(
        sensor_width=3008, sensor_height=2008, cfa="RGGB", black=(512.0,), white=(16383.0,),
        highlight="clip", clip_levels=clip_levels(1.0, wb), demosaic="amaze", demosaic_balance=wb)
    color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, base_lut=standard_base_lut())
    return Workload("plain_3mp", 3008, 2008, "RGGB", 14, 512.0, 16383.0, 0.02, False, wb, sensor, None, None,
                    (3008, 2008), color, seed)


def full_24mp(demosaic: str = "amaze", iterations: int = 10, seed: int = 2, highlight: str = "opposed",
              width: int = 6048, height: int = 4024) -> Workload:
    wb = (2.0, 1.0, 1.6)
    if highlight == "opposed":
        det, ceiling = opposed_levels(1.0, wb)
        sensor = SensorDescription(
            sensor_width=width, sensor_height=height, cfa="RGGB", black=(512.0,), white=(16383.0,),
            highlight="opposed", detection_levels=det, neutral_ceiling=ceiling, demosaic=demosaic,
            demosaic_balance=wb)
        ceilings = (1.0, 1.0, 1.0)  # detail.rs:323-337, Opposed: [detection_threshold; 3]
    else:
        sensor = SensorDescription(
            sensor_width=width, sensor_height=height, cfa="RGGB", black=(512.0,), white=(16383.0,),
            highlight="clip", clip_levels=clip_levels(1.0, wb), demosaic=demosaic, demosaic_balance=wb)
        ceilings = clip_levels(1.0, wb)
    capture = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=ceilings,
                              iterations=iterations)
    rng = np.random.default_rng(seed)
    vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
    optics = OpticsExecution(width=width, height=height, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0),
                             tca="linear", tca_red=(1.0003, 0.0, 0.0), tca_blue=(0.9997, 0.0, 0.0),
                             vignetting_k=vig, crop_factor=1.0, real_focal=35.0)
    target = preview_dimensions(width, height, 2560)
    color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.5,
                          base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(), hsl=hsl_bands())
    return Workload("full_24mp", width, height, "RGGB", 14, 512.0, 16383.0, 0.05, True, wb, sensor, capture, optics,
                    target, color, seed)


# Sizes and bit depths of the uneven batch (12-, 24-, 45- and 60-megapixel sensors).
BATCH_SENSORS = ((4000, 3000, 12), (6048, 4024, 14), (8256, 5504, 14), (9504, 6336, 14))


def batched_uneven(count: int = 48, seed: int = 3, iterations: int = 5) -> list[Workload]:
    """The uneven batch: sizes drawn from BATCH_SENSORS, random CFA phase,
    black U(256, 1024), per-image as-shot WB and camera matrix from seeded
    ranges; Opposed + AMaZE + RL (K iterations) + optics + 2560-px preview."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        width, height, bits = BATCH_SENSORS[int(rng.integers(len(BATCH_SENSORS)))]
        cfa = ("RGGB", "BGGR", "GRBG", "GBRG")[int(rng.integers(4))]
        white = float((1 << bits) - 1)
        black = float(rng.uniform(256.0, 1024.0)) if bits == 14 else float(rng.uniform(64.0, 256.0))
        wb = (float(rng.uniform(1.6, 2.4)), 1.0, float(rng.uniform(1.3, 2.0)))
        cam = tuple(float(v) for v in (np.asarray(CAMERA_TO_REC2020) * rng.uniform(0.95, 1.05, 9)))
        det, ceiling = opposed_levels(1.0, wb)
        sensor = SensorDescription(sensor_width=width, sensor_height=height, cfa=cfa, black=(black,), white=(white,),
                                   highlight="opposed", detection_levels=det, neutral_ceiling=ceiling,
                                   demosaic="amaze", demosaic_balance=wb)
        capture = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=(1.0, 1.0, 1.0),
                                  iterations=iterations)
        vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
        optics = OpticsExecution(width=width, height=height, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0),
                                 tca="linear", tca_red=(1.0003, 0.0, 0.0), tca_blue=(0.9997, 0.0, 0.0),
                                 vignetting_k=vig, crop_factor=1.0, real_focal=35.0)
        color = ColorContract(wb_gains=wb, camera_to_rec2020=cam, exposure_ev=float(rng.uniform(-0.5, 0.8)),
                              base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=int(rng.integers(1 << 30))),
                              hsl=hsl_bands(seed=int(rng.integers(1 << 30))))
        out.append(Workload(f"batch_{k}", width, height, cfa, bits, black, white, 0.05, True, wb, sensor, capture,
                            optics, preview_dimensions(width, height, 2560), color, seed * 1000 + k))
    return out


def large_export(count: int = 24, seed: int = 5, iterations: int = 20) -> list[Workload]:
    """The large-sensor export stream: 11648x8736 (101.8 MP) RGGB 16-bit
    mosaics (white 65535) with saturated specular blobs; Opposed + AMaZE + RL
    (K iterations) + full optics; a 2560-px preview while open. Hot pixels
    (0.5% of samples at white) are added to the host mosaic by `hot_pixels`."""
    out = []
    width, height, bits = 11648, 8736, 16
    for k in range(count):
        rng = np.random.default_rng(seed * 1000 + k)
        wb = (float(rng.uniform(1.7, 2.3)), 1.0, float(rng.uniform(1.4, 1.9)))
        det, ceiling = opposed_levels(1.0, wb)
        sensor = SensorDescription(sensor_width=width, sensor_height=height, cfa="RGGB", black=(1024.0,),
                                   white=(65535.0,), highlight="opposed", detection_levels=det,
                                   neutral_ceiling=ceiling, demosaic="amaze", demosaic_balance=wb)
        capture = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=(1.0, 1.0, 1.0),
                                  iterations=iterations)
        vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
        optics = OpticsExecution(width=width, height=height, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0),
                                 tca="linear", tca_red=(1.0003, 0.0, 0.0), tca_blue=(0.9997, 0.0, 0.0),
                                 vignetting_k=vig, crop_factor=1.0, real_focal=35.0)
        color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.3,
                              base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=k),
                              hsl=hsl_bands(seed=k))
        out.append(Workload(f"export_{k}", width, height, "RGGB", bits, 1024.0, 65535.0, 0.05, True, wb, sensor,
                            capture, optics, preview_dimensions(width, height, 2560), color, seed * 1000 + k))
    return out


def hot_pixels(mosaic: np.ndarray, fraction: float = 0.005, seed: int = 0, white: int = 65535) -> np.ndarray:
    """Stuck-at-white samples at a seeded `fraction` of positions (in place)."""
    rng = np.random.default_rng(seed)
    n = int(mosaic.size * fraction)
    flat = mosaic.reshape(-1)
    flat[rng.choice(mosaic.size, size=n, replace=False)] = white
    return mosaic
