"""Host-side mirror of the reference's `rohditor-gpu` processor interface.

The classes keep the reference's names, argument meaning and error behaviour
so an engine written against crates/gpu reads the same here:

  GpuPreviewError        crates/gpu/src/lib.rs:55-111 (variants, is_routing)
  GpuSensorProcessor     crates/gpu/src/sensor/normalize.rs:75-157 (new, set_budget)
                         crates/gpu/src/sensor/develop.rs:54-141 (supports, develop)
  GpuDevelopedSource     crates/gpu/src/sensor/develop.rs:28-47
  GpuSpatialProcessor    crates/gpu/src/spatial/reduction.rs:15 (reduce_preview)
  GpuPreviewProcessor    crates/gpu/src/preview/processor.rs:1011-1060,1518 (render, histogram)

Everything runs in librd_gpu.so through the C ABI; numpy arrays are the host
buffers and nothing here computes pixels.
"""

from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass, field

import numpy as np

from . import _ffi


class GpuPreviewError(RuntimeError):
    """A failed call; `variant` is the GpuPreviewError variant name."""

    def __init__(self, code: int, message: str):
        self.code = code
        self.variant = _ffi.STATUS_NAMES[code] if 0 <= code < len(_ffi.STATUS_NAMES) else "Unknown"
        super().__init__(f"{self.variant}: {message}")

    def is_routing(self) -> bool:
        """UnsupportedEdits and OverBudget keep the device; callers route to another path."""
        return bool(_ffi.load().rd_status_is_routing(self.code))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


# ---------------------------------------------------------------- contracts
@dataclass
class SensorDescription:
    """NormalizationContract + SensorDevelopmentDescription (sensor.rs:56-67, 280-298)."""

    sensor_width: int
    sensor_height: int
    cfa: str = "RGGB"
    crop: tuple[int, int, int, int] | None = None  # x, y, w, h
    black: tuple[float, ...] = (0.0,)
    black_repeat: tuple[int, int] = (1, 1)
    white: tuple[float, ...] = (1.0,)
    highlight: str = "off"
    clip_levels: tuple[float, float, float] = (1.0, 1.0, 1.0)
    detection_levels: tuple[float, float, float] = (1.0, 1.0, 1.0)
    neutral_ceiling: tuple[float, float, float] | None = None
    demosaic: str = "amaze"
    demosaic_balance: tuple[float, float, float] = (1.0, 1.0, 1.0)

    def to_c(self) -> _ffi.SensorDesc:
        d = _ffi.SensorDesc()
        d.sensor_width, d.sensor_height = self.sensor_width, self.sensor_height
        cx, cy, cw, ch = self.crop or (0, 0, self.sensor_width, self.sensor_height)
        d.crop_x, d.crop_y, d.crop_width, d.crop_height = cx, cy, cw, ch
        d.cfa = _ffi.CFA[self.cfa.upper()]
        d.black_repeat_w, d.black_repeat_h = self.black_repeat
        for i, v in enumerate(self.black):
            d.black[i] = v
        d.white_count = len(self.white)
        for i, v in enumerate(self.white):
            d.white[i] = v
        d.highlight = _ffi.HIGHLIGHT[self.highlight]
        for c in range(3):
            d.clip_levels[c] = self.clip_levels[c]
            d.detection_levels[c] = self.detection_levels[c]
            d.demosaic_balance[c] = self.demosaic_balance[c]
        if self.neutral_ceiling is not None:
            d.has_neutral_ceiling = 1
            for c in range(3):
                d.neutral_ceiling[c] = self.neutral_ceiling[c]
        d.demosaic = _ffi.DEMOSAIC[self.demosaic]
        return d

    @property
    def crop_size(self) -> tuple[int, int]:
        if self.crop:
            return self.crop[2], self.crop[3]
        return self.sensor_width, self.sensor_height


DETECTION_SAFETY_MARGIN = np.float32(0.987)  # crates/highlight/src/lib.rs:27


def clip_levels(threshold: float, gains) -> tuple[float, float, float]:
    """HighlightExecution::Clip ceilings from the user WB gains (sensor.rs:407-420)."""
    g = [np.float32(x) for x in gains]
    common = np.float32(np.float32(threshold) * DETECTION_SAFETY_MARGIN) * min(g[0], g[1], g[2])
    return tuple(float(np.float32(common / x)) for x in g)


def opposed_levels(threshold: float, as_shot) -> tuple[tuple[float, ...], tuple[float, ...]]:
    """Opposed detection levels and neutral ceiling from the as-shot gains (sensor.rs:421-455)."""
    level = np.float32(np.float32(threshold) * DETECTION_SAFETY_MARGIN)
    g = [np.float32(x) for x in as_shot]
    common = np.float32(level * min(g[0], g[1], g[2]))
    return (float(level),) * 3, tuple(float(np.float32(common / x)) for x in g)


def capture_ceilings(highlight: str, threshold: float, gains) -> tuple[float, float, float]:
    """Capture-sharpening mask ceilings (crates/core/src/pipeline/detail.rs:323-337): Clip's common
    ceiling threshold * min(gains) / gain (no safety margin), Opposed's detection threshold, else 1."""
    if highlight == "clip":
        g = [np.float32(x) for x in gains]
        common = np.float32(np.float32(threshold) * min(g[0], g[1], g[2]))
        return tuple(float(np.float32(common / x)) for x in g)
    if highlight == "opposed":
        return (float(np.float32(threshold)),) * 3
    return (1.0, 1.0, 1.0)


@dataclass
class CaptureContract:
    """CaptureSharpeningContract (sharpening.rs:17-68) with an explicit iteration count."""

    amount: float = 0.5
    radius: float = 0.6
    noise_protection: float = 0.5
    ceilings: tuple[float, float, float] = (1.0, 1.0, 1.0)
    iterations: int = 8
    enabled: bool = True

    def to_c(self) -> _ffi.DetailDesc:
        d = _ffi.DetailDesc()
        d.enabled = 1 if self.enabled else 0
        d.amount, d.radius, d.noise_protection = self.amount, self.radius, self.noise_protection
        for c in range(3):
            d.ceilings[c] = self.ceilings[c]
        d.iterations = self.iterations
        return d


@dataclass
class OpticsExecution:
    """OpticsExecution (crates/optics/src/plan.rs:37-50), resolved on the host."""

    width: int
    height: int
    distortion: str = "none"
    distortion_k: tuple[float, float, float] = (0.0, 0.0, 0.0)
    tca: str = "none"
    tca_red: tuple[float, float, float] = (1.0, 0.0, 0.0)
    tca_blue: tuple[float, float, float] = (1.0, 0.0, 0.0)
    vignetting_k: tuple[float, float, float] | None = None
    crop_factor: float = 1.0
    real_focal: float = 35.0
    lens_center: tuple[float, float] = (0.0, 0.0)
    _c: _ffi.OpticsDesc | None = field(default=None, repr=False)

    def to_c(self) -> _ffi.OpticsDesc:
        if self._c is not None:
            return self._c
        d = _ffi.OpticsDesc()
        d.width, d.height = self.width, self.height
        d.distortion_model = _ffi.DISTORTION[self.distortion]
        d.tca_model = _ffi.TCA[self.tca]
        for c in range(3):
            d.distortion[c] = self.distortion_k[c]
            d.tca_red[c] = self.tca_red[c]
            d.tca_blue[c] = self.tca_blue[c]
        if self.vignetting_k is not None:
            d.vignetting = 1
            for c in range(3):
                d.vignetting_k[c] = self.vignetting_k[c]
        rc = _ffi.load().rd_optics_plan(ctypes.byref(d), self.crop_factor, self.real_focal, *self.lens_center)
        if rc != 0:
            raise GpuPreviewError(rc, "optics plan failed (no safe automatic scale)")
        self._c = d
        return d


@dataclass
class ColorContract:
    """White balance, camera matrix and the global adjustment chain with resolved LUTs."""

    wb_gains: tuple[float, float, float] = (1.0, 1.0, 1.0)
    camera_to_rec2020: tuple[float, ...] = (1, 0, 0, 0, 1, 0, 0, 0, 1)
    exposure_ev: float = 0.0
    base_lut: np.ndarray | None = None
    light_tone_lut: np.ndarray | None = None  # LightToneLut values, see light_tone_lut()
    tone_lut: np.ndarray | None = None
    saturation: float = 1.0
    vibrance: float = 0.0
    hsl: np.ndarray | None = None       # 8 x 3
    grading: np.ndarray | None = None   # 3 x 3

    def to_c(self) -> _ffi.ColorDesc:
        d = _ffi.ColorDesc()
        for c in range(3):
            d.wb_gains[c] = self.wb_gains[c]
        for k in range(9):
            d.camera_to_rec2020[k] = self.camera_to_rec2020[k]
        d.exposure_ev = self.exposure_ev
        if self.base_lut is not None:
            d.has_base_lut = 1
            ctypes.memmove(d.base_lut, _f32(self.base_lut).ctypes.data, 4096 * 4)
        if self.light_tone_lut is not None:
            d.has_light_tone_lut = 1
            ctypes.memmove(d.light_tone_lut, _f32(self.light_tone_lut).ctypes.data, 4096 * 4)
        if self.tone_lut is not None:
            d.has_tone_lut = 1
            ctypes.memmove(d.tone_lut, _f32(self.tone_lut).ctypes.data, 4096 * 4)
        d.saturation, d.vibrance = self.saturation, self.vibrance
        if self.hsl is not None:
            d.has_hsl = 1
            ctypes.memmove(d.hsl, _f32(self.hsl).ctypes.data, 24 * 4)
        if self.grading is not None:
            d.has_grading = 1
            ctypes.memmove(d.grading, _f32(self.grading).ctypes.data, 9 * 4)
        return d


@dataclass
class OutputSpec:
    """Output conversion of a render: format, target primaries, gamut policy,
    dither and OutputGeometry (orientation + normalized crop on the oriented
    canvas). Formats: "srgb8", "srgb16", "extended_f32", "extended_f16"."""

    format: str = "srgb8"
    primaries: str = "srgb"
    policy: str = "clip"
    dither: str = "none"
    orientation: str = "normal"
    crop: tuple[float, float, float, float] | None = None
    headroom: float = 1.0

    def to_c(self) -> _ffi.OutputDesc:
        d = _ffi.OutputDesc()
        d.format = _ffi.OUTPUT_FORMAT[self.format]
        d.primaries = _ffi.PRIMARIES[self.primaries]
        d.policy = _ffi.OUTPUT_POLICY[self.policy]
        d.dither = _ffi.DITHER[self.dither]
        d.orientation = _ffi.ORIENTATION[self.orientation]
        if self.crop is not None:
            d.has_crop = 1
            for k in range(4):
                d.crop[k] = self.crop[k]
        d.headroom = self.headroom
        return d

    @property
    def dtype(self):
        return {"srgb8": np.uint8, "srgb16": np.uint16, "extended_f32": np.float32,
                "extended_f16": np.float16}[self.format]

    def dimensions(self, width: int, height: int) -> tuple[int, int]:
        ow, oh, bpp = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        rc = _ffi.load().rd_output_dimensions(width, height, ctypes.byref(self.to_c()), ctypes.byref(ow),
                                              ctypes.byref(oh), ctypes.byref(bpp))
        if rc != 0:
            raise GpuPreviewError(rc, "invalid output description")
        return ow.value, oh.value


@dataclass
class GamutDiagnostics:
    """GamutMappingDiagnostics (crates/color/src/gamut.rs:60-98)."""

    in_gamut: int
    compressed: int
    limited: int
    clipped_fallback: int
    invalid: int

    @property
    def total(self) -> int:
        return self.in_gamut + self.compressed + self.limited + self.clipped_fallback + self.invalid


@dataclass
class RlLaunchShape:
    """The capture-sharpening launch shape chosen for one image shape."""

    segments: int
    default_segments: int
    best_ms: float
    default_ms: float


def rl_launch_shape(width: int, height: int, radius: float) -> RlLaunchShape | None:
    """rd_rl_launch_shape: the row-segment count the first develop of this
    (width, height, radius) picked by timing, or None before any develop of it."""
    segs, dflt = ctypes.c_int32(), ctypes.c_int32()
    best, dms = ctypes.c_float(), ctypes.c_float()
    code = _ffi.load().rd_rl_launch_shape(width, height, radius, ctypes.byref(segs), ctypes.byref(dflt),
                                         ctypes.byref(best), ctypes.byref(dms))
    if code == _ffi.STATUS_NAMES.index("Unsupported"):
        return None
    if code != 0:
        raise GpuPreviewError(code, "rd_rl_launch_shape")
    return RlLaunchShape(segs.value, dflt.value, best.value, dms.value)


def launch_shape(stage: str, width: int, height: int, radius: float = 0.0) -> RlLaunchShape | None:
    """rd_launch_shape: the launch shape tuned across calls for `stage` ("rl_mask": row segments of the
    capture guide / mask kernel; "color": CTAs per SM of the colour kernel; "optics": rows of the optics
    gather's 32-column tiles) at this image size, or None while it is still being tuned."""
    value, dflt = ctypes.c_int32(), ctypes.c_int32()
    best, dms = ctypes.c_float(), ctypes.c_float()
    code = _ffi.load().rd_launch_shape({"rl_mask": 0, "color": 1, "optics": 2}[stage], width, height, radius,
                                      ctypes.byref(value),
                                      ctypes.byref(dflt), ctypes.byref(best), ctypes.byref(dms))
    if code == _ffi.STATUS_NAMES.index("Unsupported"):
        return None
    if code != 0:
        raise GpuPreviewError(code, "rd_launch_shape")
    return RlLaunchShape(value.value, dflt.value, best.value, dms.value)


def standard_base_lut() -> np.ndarray:
    """BaseRenderingLut::standard_v1 values (crates/core/src/rendering.rs:36-50)."""
    out = np.zeros(4096, dtype=np.float32)
    _ffi.load().rd_standard_base_lut(_ptr(out, ctypes.c_float))
    return out


def light_tone_lut(contrast: float = 0.0, highlights: float = 0.0, shadows: float = 0.0, whites: float = 0.0,
                   blacks: float = 0.0) -> np.ndarray | None:
    """LightToneLut::new (crates/edit/src/light.rs:27-47) for the Light sliders, or None when all
    five are zero: the reference builds the table only then (crates/core/src/cpu/stages.rs:434-439)."""
    if contrast == 0.0 and highlights == 0.0 and shadows == 0.0 and whites == 0.0 and blacks == 0.0:
        return None
    out = np.zeros(4096, dtype=np.float32)
    f = ctypes.c_float
    _ffi.load().rd_light_tone_lut(f(contrast), f(highlights), f(shadows), f(whites), f(blacks),
                                  _ptr(out, ctypes.c_float))
    return out


# ---------------------------------------------------------------- processors
class Device:
    """One CUDA context (stream + budgeted memory pool) on one GPU."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        self.lib = _ffi.load()
        h = ctypes.c_void_p()
        rc = self.lib.rd_ctx_create(device, budget_bytes, ctypes.byref(h))
        if rc != 0:
            raise GpuPreviewError(rc, f"could not create a context on device {device}")
        self.handle = h
        # Resident objects must be released before the context that owns their memory.
        self._children = weakref.WeakSet()

    def check(self, rc: int):
        if rc != 0:
            raise GpuPreviewError(rc, self.lib.rd_ctx_last_error(self.handle).decode())

    def set_budget(self, budget_bytes: int):
        self.check(self.lib.rd_ctx_set_budget(self.handle, budget_bytes))

    def synchronize(self):
        self.check(self.lib.rd_ctx_synchronize(self.handle))

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.rd_ctx_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            for child in list(self._children):
                child.release()
            self.lib.rd_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuDevelopedSource:
    """Full-resolution camera RGB resident on the device."""

    def __init__(self, device: Device, handle: ctypes.c_void_p, metrics: _ffi.Metrics):
        self.device, self.handle, self.metrics = device, handle, metrics
        device._children.add(self)
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        device.check(device.lib.rd_source_dimensions(handle, ctypes.byref(w), ctypes.byref(h)))
        self.width, self.height = w.value, h.value

    def download(self) -> np.ndarray:
        out = np.empty((self.height, 3 * self.width), dtype=np.float32)
        self.device.check(self.device.lib.rd_source_download(self.device.handle, self.handle, _ptr(out, ctypes.c_float)))
        return out

    def release(self):
        if self.handle and self.device.handle:
            self.device.lib.rd_source_release(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class GpuBase:
    """Reduced linear Rec.2020 base resident on the device."""

    def __init__(self, device: Device, handle: ctypes.c_void_p, metrics: _ffi.Metrics):
        self.device, self.handle, self.metrics = device, handle, metrics
        device._children.add(self)
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        device.check(device.lib.rd_base_dimensions(handle, ctypes.byref(w), ctypes.byref(h)))
        self.width, self.height = w.value, h.value

    def download(self) -> np.ndarray:
        out = np.empty((self.height, 3 * self.width), dtype=np.float32)
        self.device.check(self.device.lib.rd_base_download(self.device.handle, self.handle, _ptr(out, ctypes.c_float)))
        return out

    def release(self):
        if self.handle and self.device.handle:
            self.device.lib.rd_base_release(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class GpuSensorProcessor:
    """normalize -> highlight -> demosaic -> capture sharpening on the device."""

    def __init__(self, device: Device):
        self.device = device

    def set_budget(self, budget_bytes: int):
        self.device.set_budget(budget_bytes)

    @staticmethod
    def supports(description: SensorDescription) -> bool:
        d = description.to_c()
        return bool(_ffi.load().rd_supports(ctypes.byref(d)))

    def develop(self, mosaic: np.ndarray, description: SensorDescription, capture: CaptureContract | None = None,
                cancel: np.ndarray | None = None) -> GpuDevelopedSource:
        mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
        row_stride = mosaic.shape[1]
        d = description.to_c()
        detail = capture.to_c() if capture is not None else None
        out = ctypes.c_void_p()
        m = _ffi.Metrics()
        cancel_ptr = cancel.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if cancel is not None else None
        self.device.check(self.device.lib.rd_develop(
            self.device.handle, _ptr(mosaic, ctypes.c_uint16), row_stride, ctypes.byref(d),
            ctypes.byref(detail) if detail is not None else None, cancel_ptr, ctypes.byref(out), ctypes.byref(m)))
        return GpuDevelopedSource(self.device, out, m)

    def develop_device(self, d_mosaic: int, row_stride: int, description: SensorDescription,
                       capture: CaptureContract | None = None) -> GpuDevelopedSource:
        d = description.to_c()
        detail = capture.to_c() if capture is not None else None
        out = ctypes.c_void_p()
        m = _ffi.Metrics()
        self.device.check(self.device.lib.rd_develop_device(
            self.device.handle, ctypes.c_void_p(d_mosaic), row_stride, ctypes.byref(d),
            ctypes.byref(detail) if detail is not None else None, None, ctypes.byref(out), ctypes.byref(m)))
        return GpuDevelopedSource(self.device, out, m)


class GpuSpatialProcessor:
    """Optics (vignetting, distortion, TCA) + exact area reduction + WB/matrix to Rec.2020."""

    def __init__(self, device: Device):
        self.device = device

    def reduce_preview(self, source: GpuDevelopedSource, optics: OpticsExecution | None, target: tuple[int, int],
                       wb_gains, camera_to_rec2020) -> GpuBase:
        o = optics.to_c() if optics is not None else None
        g = _f32(wb_gains)
        m = _f32(camera_to_rec2020).reshape(-1)
        out = ctypes.c_void_p()
        met = _ffi.Metrics()
        self.device.check(self.device.lib.rd_spatial(
            self.device.handle, source.handle, ctypes.byref(o) if o is not None else None, target[0], target[1],
            _ptr(g, ctypes.c_float), _ptr(m, ctypes.c_float), ctypes.byref(out), ctypes.byref(met)))
        return GpuBase(self.device, out, met)


@dataclass
class Histogram:
    """R, G, B and luma bins plus shadow/highlight clip counts (histogram.rs:13-21)."""

    red: np.ndarray
    green: np.ndarray
    blue: np.ndarray
    luminance: np.ndarray
    shadow_clipped: np.ndarray
    highlight_clipped: np.ndarray


class GpuPreviewProcessor:
    """Adjustments + sRGB 8-bit output + histogram of that output."""

    def __init__(self, device: Device):
        self.device = device

    def render(self, base: GpuBase, color: ColorContract) -> tuple[np.ndarray, Histogram]:
        c = color.to_c()
        out = np.empty((base.height, 3 * base.width), dtype=np.uint8)
        hist = np.zeros(1024, dtype=np.uint64)
        clipped = np.zeros(6, dtype=np.uint64)
        self.device.check(self.device.lib.rd_render(
            self.device.handle, base.handle, ctypes.byref(c), _ptr(out, ctypes.c_uint8), _ptr(hist, ctypes.c_uint64),
            _ptr(clipped, ctypes.c_uint64), None))
        return out, Histogram(hist[0:256], hist[256:512], hist[512:768], hist[768:1024], clipped[:3], clipped[3:])

    def render_output(self, base: GpuBase, color: ColorContract, output: OutputSpec,
                      histogram: bool = False) -> tuple[np.ndarray, Histogram | None, GamutDiagnostics]:
        """Display / extended output of the base: [out_h][3*out_w] of output.dtype."""
        ow, oh = output.dimensions(base.width, base.height)
        out = np.empty((oh, 3 * ow), dtype=output.dtype)
        hist = np.zeros(1024, dtype=np.uint64) if histogram else None
        gamut = np.zeros(5, dtype=np.uint64)
        self.device.check(self.device.lib.rd_render_output(
            self.device.handle, base.handle, ctypes.byref(color.to_c()), ctypes.byref(output.to_c()),
            out.ctypes.data_as(ctypes.c_void_p), out.nbytes, _ptr(hist, ctypes.c_uint64) if hist is not None else None,
            _ptr(gamut, ctypes.c_uint64), None))
        h = None
        if hist is not None:
            clipped = np.array([hist[256 * c] for c in range(3)] + [hist[256 * c + 255] for c in range(3)],
                               dtype=np.uint64)
            h = Histogram(hist[0:256], hist[256:512], hist[512:768], hist[768:1024], clipped[:3], clipped[3:])
        return out, h, GamutDiagnostics(*(int(v) for v in gamut))

    def render_device(self, base: GpuBase, color_c: _ffi.ColorDesc):
        self.device.check(self.device.lib.rd_render_device(self.device.handle, base.handle, ctypes.byref(color_c), None))


class PngEncoder:
    """The PNG arms of export::encode (crates/core/src/export.rs:155-219) on the device.

    `encode` takes interleaved RGB rows ([h][w][3] or [h][3w]; uint8 or uint16)
    and returns the file's bytes with the ICC profile in an iCCP chunk and EXIF
    in an eXIf chunk. Like the reference (ExportError::InvalidImageLayout,
    export.rs:136-150) it refuses rows that are not tightly packed: pass
    `row_stride` (samples) to describe a padded [h][row_stride] array.
    """

    def __init__(self, device: Device):
        self.device = device

    @staticmethod
    def bound(width: int, height: int, bit_depth: int, icc_len: int = 0, exif_len: int = 0) -> int:
        return int(_ffi.load().rd_png_bound(width, height, bit_depth, icc_len, exif_len))

    def encode(self, rgb: np.ndarray, icc_profile: bytes = b"", exif: bytes | None = None,
               row_stride: int | None = None, width: int | None = None) -> bytes:
        rgb = np.ascontiguousarray(rgb)
        if rgb.dtype not in (np.uint8, np.uint16):
            raise GpuPreviewError(8, f"PNG samples are uint8 or uint16, not {rgb.dtype}")
        depth = 16 if rgb.dtype == np.uint16 else 8
        height = rgb.shape[0]
        if width is None:
            width = rgb.shape[1] if rgb.ndim == 3 else rgb.shape[1] // 3
        stride = 3 * width if row_stride is None else row_stride
        icc = np.frombuffer(icc_profile, dtype=np.uint8) if icc_profile else None
        ex = np.frombuffer(exif, dtype=np.uint8) if exif else None
        capacity = self.bound(width, height, depth, len(icc_profile or b""), len(exif or b""))
        out = np.empty(max(capacity, 1), dtype=np.uint8)
        size = ctypes.c_uint64(0)
        self.device.check(self.device.lib.rd_encode_png(
            self.device.handle, rgb.ctypes.data_as(ctypes.c_void_p), width, height, stride, depth,
            _ptr(icc, ctypes.c_uint8) if icc is not None else None, len(icc_profile or b""),
            _ptr(ex, ctypes.c_uint8) if ex is not None else None, len(exif or b""),
            _ptr(out, ctypes.c_uint8), out.nbytes, ctypes.byref(size), None))
        return out[:size.value].tobytes()


class JpegEncoder:
    """The JPEG arm of export::encode (crates/core/src/export.rs:166-175) on the device.

    `encode` takes 8-bit interleaved RGB rows ([h][w][3] or [h][3w]) and a
    quality of 1..100 and returns a baseline JPEG file with the ICC profile in
    APP2 segments and the EXIF block in an APP1 segment. Rows that are not
    tightly packed (`row_stride` samples per row) and qualities outside 1..100
    are refused.
    """

    def __init__(self, device: Device):
        self.device = device

    @staticmethod
    def bound(width: int, height: int, icc_len: int = 0, exif_len: int = 0) -> int:
        return int(_ffi.load().rd_jpeg_bound(width, height, icc_len, exif_len))

    def encode(self, rgb: np.ndarray, quality: int, icc_profile: bytes = b"", exif: bytes | None = None,
               row_stride: int | None = None, width: int | None = None) -> bytes:
        rgb = np.ascontiguousarray(rgb)
        if rgb.dtype != np.uint8:
            raise GpuPreviewError(8, f"JPEG samples are uint8, not {rgb.dtype}")
        height = rgb.shape[0]
        if width is None:
            width = rgb.shape[1] if rgb.ndim == 3 else rgb.shape[1] // 3
        stride = 3 * width if row_stride is None else row_stride
        icc = np.frombuffer(icc_profile, dtype=np.uint8) if icc_profile else None
        ex = np.frombuffer(exif, dtype=np.uint8) if exif else None
        capacity = max(self.bound(width, height, len(icc_profile or b""), len(exif or b"")), 1)
        out = np.empty(capacity, dtype=np.uint8)
        size = ctypes.c_uint64(0)
        self.device.check(self.device.lib.rd_encode_jpeg(
            self.device.handle, rgb.ctypes.data_as(ctypes.c_void_p), width, height, stride, quality,
            _ptr(icc, ctypes.c_uint8) if icc is not None else None, len(icc_profile or b""),
            _ptr(ex, ctypes.c_uint8) if ex is not None else None, len(exif or b""),
            _ptr(out, ctypes.c_uint8), out.nbytes, ctypes.byref(size), None))
        return out[:size.value].tobytes()


# ---------------------------------------------------------------- stage API
class Stages:
    """The crates' stage functions, each run on the device with host buffers."""

    def __init__(self, device: Device):
        self.device = device
        self.lib = device.lib

    def highlight(self, mosaic: np.ndarray, description: SensorDescription) -> tuple[np.ndarray, np.ndarray]:
        mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
        d = description.to_c()
        w, h = description.crop_size
        out = np.empty((h, w), dtype=np.float32)
        stats = np.zeros(9, dtype=np.uint64)
        self.device.check(self.lib.rd_stage_highlight(self.device.handle, _ptr(mosaic, ctypes.c_uint16), mosaic.shape[1],
                                                      ctypes.byref(d), _ptr(out, ctypes.c_float),
                                                      _ptr(stats, ctypes.c_uint64)))
        return out, stats

    def opposed(self, mosaic: np.ndarray, cfa: str, levels, ceiling=None):
        """reconstruct_opposed on a normalized mosaic: (mosaic, stats[9], cell labels, region count)."""
        mosaic = _f32(mosaic)
        h, w = mosaic.shape
        lv = _f32(levels)
        ce = _f32(ceiling) if ceiling is not None else None
        out = np.empty_like(mosaic)
        stats = np.zeros(9, dtype=np.uint64)
        labels = np.zeros(((h + 1) // 2, (w + 1) // 2), dtype=np.uint32)
        count = ctypes.c_uint32()
        self.device.check(self.lib.rd_stage_opposed(
            self.device.handle, _ptr(mosaic, ctypes.c_float), w, h, _ffi.CFA[cfa.upper()], _ptr(lv, ctypes.c_float),
            _ptr(ce, ctypes.c_float) if ce is not None else None, _ptr(out, ctypes.c_float),
            _ptr(stats, ctypes.c_uint64), labels.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(count)))
        return out, stats, labels, count.value

    def demosaic(self, mosaic: np.ndarray, cfa: str, algorithm: str, balance=(1.0, 1.0, 1.0)) -> np.ndarray:
        mosaic = _f32(mosaic)
        h, w = mosaic.shape
        bal = _f32(balance)
        out = np.empty((h, 3 * w), dtype=np.float32)
        self.device.check(self.lib.rd_stage_demosaic(self.device.handle, _ptr(mosaic, ctypes.c_float), w, h,
                                                     _ffi.CFA[cfa.upper()], _ffi.DEMOSAIC[algorithm],
                                                     _ptr(bal, ctypes.c_float), _ptr(out, ctypes.c_float)))
        return out

    def capture(self, rgb: np.ndarray, capture: CaptureContract) -> np.ndarray:
        rgb = _f32(rgb).copy()
        h, w3 = rgb.shape
        d = capture.to_c()
        self.device.check(self.lib.rd_stage_capture(self.device.handle, _ptr(rgb, ctypes.c_float), w3 // 3, h,
                                                    ctypes.byref(d)))
        return rgb

    def optics(self, rgb: np.ndarray, optics: OpticsExecution) -> np.ndarray:
        rgb = _f32(rgb)
        out = np.empty_like(rgb)
        o = optics.to_c()
        self.device.check(self.lib.rd_stage_optics(self.device.handle, ctypes.byref(o), _ptr(rgb, ctypes.c_float),
                                                   _ptr(out, ctypes.c_float)))
        return out

    def area_reduce(self, rgb: np.ndarray, target: tuple[int, int]) -> np.ndarray:
        rgb = _f32(rgb)
        h, w3 = rgb.shape
        out = np.empty((target[1], 3 * target[0]), dtype=np.float32)
        self.device.check(self.lib.rd_stage_area_reduce(self.device.handle, _ptr(rgb, ctypes.c_float), w3 // 3, h,
                                                        target[0], target[1], _ptr(out, ctypes.c_float)))
        return out

    def output(self, rgb: np.ndarray, color: ColorContract, output: OutputSpec,
               histogram: bool = False) -> tuple[np.ndarray, np.ndarray | None, np.ndarray]:
        """Linear Rec.2020 [h][3w] -> adjustments -> output: (image, 1024 bins or None, gamut counts[5])."""
        rgb = _f32(rgb)
        h, w3 = rgb.shape
        ow, oh = output.dimensions(w3 // 3, h)
        out = np.empty((oh, 3 * ow), dtype=output.dtype)
        hist = np.zeros(1024, dtype=np.uint64) if histogram else None
        gamut = np.zeros(5, dtype=np.uint64)
        self.device.check(self.lib.rd_stage_output(
            self.device.handle, _ptr(rgb, ctypes.c_float), w3 // 3, h, ctypes.byref(color.to_c()),
            ctypes.byref(output.to_c()), out.ctypes.data_as(ctypes.c_void_p), out.nbytes,
            _ptr(hist, ctypes.c_uint64) if hist is not None else None, _ptr(gamut, ctypes.c_uint64)))
        return out, hist, gamut

    def check_math(self, which: int) -> int:
        """rd_check_math: 0 -> cube roots not correctly rounded; 1 -> largest powf distance in ulps;
        2, 3 -> transfer powers / quantised codes off the correctly rounded ones; 4 -> optics hypot mismatches."""
        v = ctypes.c_uint64()
        self.device.check(self.lib.rd_check_math(self.device.handle, which, ctypes.byref(v)))
        return v.value

    def color(self, rgb: np.ndarray, color: ColorContract) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        rgb = _f32(rgb)
        h, w3 = rgb.shape
        c = color.to_c()
        out = np.empty((h, w3), dtype=np.uint8)
        hist = np.zeros(1024, dtype=np.uint64)
        clipped = np.zeros(6, dtype=np.uint64)
        self.device.check(self.lib.rd_stage_color(self.device.handle, _ptr(rgb, ctypes.c_float), w3 // 3, h,
                                                  ctypes.byref(c), _ptr(out, ctypes.c_uint8),
                                                  _ptr(hist, ctypes.c_uint64), _ptr(clipped, ctypes.c_uint64)))
        return out, hist, clipped
