"""The benchmark workloads as this library's contracts.

The parameters live in the implementation-neutral `workload_spec` module at
the repository root (shared with the CPU oracle's benchmark arm); this
module resolves them into the processor contracts (level ceilings, optics
plan, base rendering LUT) with the library's own host code, and generates
the seeded mosaic on the device.
"""

from __future__ import annotations

import ctypes
import os
import sys
from dataclasses import dataclass

import numpy as np

from . import _ffi
from .processor import (CaptureContract, ColorContract, Device, OpticsExecution, SensorDescription, capture_ceilings,
                        clip_levels, light_tone_lut, opposed_levels, standard_base_lut)

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

import workload_spec as spec  # noqa: E402
from workload_spec import (BATCH_SENSORS, CAMERA_TO_REC2020, hsl_bands, monotone_curve_lut,  # noqa: E402,F401
                           preview_dimensions, sixteen_knot_curve)


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
    spec: spec.Develop | None = None
    hot_pixel_fraction: float = 0.0

    def synth_desc(self) -> _ffi.SynthDesc:
        d = _ffi.SynthDesc()
        d.width, d.height, d.cfa, d.bits = self.width, self.height, _ffi.CFA[self.cfa], self.bits
        d.black, d.white, d.clip_fraction = self.black, self.white, self.clip_fraction
        # The sensor's channel response is the inverse of its as-shot WB.
        for c in range(3):
            d.gains[c] = min(self.as_shot) / self.as_shot[c]
        d.seed = self.seed
        d.highlight_blobs = 1 if self.blobs else 0
        d.hot_pixel_fraction = self.hot_pixel_fraction
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


def from_spec(dv: spec.Develop) -> Workload:
    """Resolve a workload description into this library's contracts."""
    s = dv.scene
    if dv.highlight == "opposed":
        det, ceiling = opposed_levels(dv.highlight_threshold, s.as_shot)
        sensor = SensorDescription(sensor_width=s.width, sensor_height=s.height, cfa=s.cfa, black=(s.black,),
                                   white=(s.white,), highlight="opposed", detection_levels=det,
                                   neutral_ceiling=ceiling, demosaic=dv.demosaic, demosaic_balance=s.as_shot)
    else:
        levels = clip_levels(dv.highlight_threshold, dv.wb_gains)
        sensor = SensorDescription(sensor_width=s.width, sensor_height=s.height, cfa=s.cfa, black=(s.black,),
                                   white=(s.white,), highlight="clip", clip_levels=levels, demosaic=dv.demosaic,
                                   demosaic_balance=s.as_shot)
    capture = None
    if dv.capture is not None:
        c = dv.capture
        capture = CaptureContract(amount=c.amount, radius=c.radius, noise_protection=c.noise_protection,
                                  ceilings=capture_ceilings(dv.highlight, dv.highlight_threshold, dv.wb_gains),
                                  iterations=c.iterations)
    optics = None
    if dv.lens is not None:
        ln = dv.lens
        optics = OpticsExecution(width=s.width, height=s.height, distortion=ln.distortion,
                                 distortion_k=ln.distortion_k, tca=ln.tca, tca_red=ln.tca_red, tca_blue=ln.tca_blue,
                                 vignetting_k=ln.vignetting_k, crop_factor=ln.crop_factor, real_focal=ln.real_focal)
    color = ColorContract(wb_gains=dv.wb_gains, camera_to_rec2020=dv.camera_to_rec2020, exposure_ev=dv.exposure_ev,
                          base_lut=standard_base_lut() if dv.base_rendering else None,
                          light_tone_lut=light_tone_lut(*dv.light), tone_lut=dv.tone_lut, hsl=dv.hsl)
    return Workload(dv.name, s.width, s.height, s.cfa, s.bits, s.black, s.white, s.clip_fraction, s.blobs, s.as_shot,
                    sensor, capture, optics, dv.target, color, s.seed, dv, s.hot_pixel_fraction)


def plain_3mp(seed: int = 1) -> Workload:
    return from_spec(spec.plain_3mp(seed))


def full_24mp(demosaic: str = "amaze", iterations: int = 10, seed: int = 2, highlight: str = "opposed",
              width: int = 6048, height: int = 4024) -> Workload:
    return from_spec(spec.full_24mp(demosaic, iterations, seed, highlight, width, height))


def batched_uneven(count: int = 48, seed: int = 3, iterations: int = 5) -> list[Workload]:
    return [from_spec(d) for d in spec.batched_uneven(count, seed, iterations)]


def large_export(count: int = 24, seed: int = 5, iterations: int = 20) -> list[Workload]:
    return [from_spec(d) for d in spec.large_export(count, seed, iterations)]
