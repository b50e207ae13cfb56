"""Parameters of the benchmark workloads, with no dependency on either implementation.

The GPU library (rohditor_gb300.workloads builds its contracts from these)
and the CPU oracle (oracle/develop.py) both read the same description, so
the two benchmark arms develop the same seeded mosaic with the same settings
without one loading the other. Everything here is plain numbers and numpy:
level ceilings, optics plans and base LUTs are derived by each side with
its own implementation of the reference's rules.

  plain_3mp        3008x2008 RGGB 14-bit (black 512, white 16383), ~2% clipped;
                   Clip + AMaZE; WB (2.0, 1.0, 1.6), fixed camera matrix; no
                   sharpening or optics; full-resolution sRGB8 + histogram.
  full_24mp        6048x4024 RGGB 14-bit, ~5% clipped in Gaussian blobs;
                   Opposed, AMaZE (or RCD / MHC); RL K=10 (sigma 0.7); Poly5
                   distortion (-0.02, 0.005), PA vignetting, linear TCA
                   1.0003 / 0.9997; area reduction to a 2560 px long edge; WB
                   + matrix; exposure +0.5 EV, 16-knot tone curve, 8-band HSL.
  batched_uneven   48 mosaics of 12/24/45/60 MP, random CFA phase, black,
                   WB and matrix; Opposed + AMaZE + RL K=5 + optics.
  large_export     11648x8736 (101.8 MP) RGGB 16-bit with hot pixels and
                   specular blobs; Opposed + AMaZE + RL K=20 + optics.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

CFA_CODES = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}

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


@dataclass(frozen=True)
class Scene:
    """The seeded synthetic mosaic: shape, CFA, levels and the generator's inputs."""

    width: int
    height: int
    cfa: str
    bits: int
    black: float
    white: float
    clip_fraction: float
    blobs: bool
    as_shot: tuple[float, float, float]
    seed: int
    hot_pixel_fraction: float = 0.0

    def channel_gains(self) -> tuple[float, float, float]:
        """The sensor's channel response: the inverse of its as-shot WB, green-normalised."""
        return tuple(min(self.as_shot) / g for g in self.as_shot)


@dataclass(frozen=True)
class Lens:
    """OpticsExecution inputs before the plan is built (plan.rs:173-326 derives the rest)."""

    distortion: str = "poly5"
    distortion_k: tuple[float, float, float] = (-0.02, 0.005, 0.0)
    tca: str = "linear"
    tca_red: tuple[float, float, float] = (1.0003, 0.0, 0.0)
    tca_blue: tuple[float, float, float] = (0.9997, 0.0, 0.0)
    vignetting_k: tuple[float, float, float] | None = None
    crop_factor: float = 1.0
    real_focal: float = 35.0


@dataclass(frozen=True)
class Capture:
    amount: float = 0.5
    radius: float = 0.7
    noise_protection: float = 0.5
    iterations: int = 10


@dataclass
class Develop:
    """One develop: the scene, the sensor-side settings, and the preview's colour settings."""

    name: str
    scene: Scene
    highlight: str                      # "opposed" or "clip"
    demosaic: str                       # "amaze", "rcd", "mhc" or "bilinear"
    capture: Capture | None
    lens: Lens | None
    target: tuple[int, int]
    wb_gains: tuple[float, float, float]
    camera_to_rec2020: tuple[float, ...]
    exposure_ev: float = 0.0
    base_rendering: bool = True
    tone_lut: np.ndarray | None = None
    hsl: np.ndarray | None = None
    light: tuple[float, float, float, float, float] = (0.0, 0.0, 0.0, 0.0, 0.0)
    highlight_threshold: float = 1.0
    extra: dict = field(default_factory=dict)

    @property
    def width(self) -> int:
        return self.scene.width

    @property
    def height(self) -> int:
        return self.scene.height

    def describe(self) -> str:
        """One line naming the workload; both benchmark arms print this same string."""
        s = self.scene
        parts = [f"{self.name} {s.width}x{s.height} {s.cfa} {s.bits}-bit", self.highlight, self.demosaic]
        if self.capture:
            parts.append(f"RL{self.capture.iterations}")
        if self.lens:
            parts.append("optics(poly5, PA vignetting, linear TCA)")
        tw, th = self.target
        parts.append(f"area->{tw}x{th}" if (tw, th) != (s.width, s.height) else "full resolution")
        parts.append("WB/matrix")
        if self.exposure_ev or self.tone_lut is not None or self.hsl is not None:
            parts.append("exposure/tone/HSL")
        parts.append("sRGB8 + histogram")
        return " + ".join(parts)


def plain_3mp(seed: int = 1) -> Develop:
    wb = (2.0, 1.0, 1.6)
    scene = Scene(3008, 2008, "RGGB", 14, 512.0, 16383.0, 0.02, False, wb, seed)
    return Develop("plain_3mp", scene, "clip", "amaze", None, None, (3008, 2008), wb, CAMERA_TO_REC2020)


def full_24mp(demosaic: str = "amaze", iterations: int = 10, seed: int = 2, highlight: str = "opposed",
              width: int = 6048, height: int = 4024) -> Develop:
    wb = (2.0, 1.0, 1.6)
    scene = Scene(width, height, "RGGB", 14, 512.0, 16383.0, 0.05, True, wb, seed)
    rng = np.random.default_rng(seed)
    vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
    return Develop("full_24mp", scene, highlight, demosaic, Capture(iterations=iterations), Lens(vignetting_k=vig),
                   preview_dimensions(width, height, 2560), wb, CAMERA_TO_REC2020, exposure_ev=0.5,
                   tone_lut=sixteen_knot_curve(), hsl=hsl_bands())


# Sizes and bit depths of the uneven batch (12-, 24-, 45- and 60-megapixel sensors).
BATCH_SENSORS = ((4000, 3000, 12), (6048, 4024, 14), (8256, 5504, 14), (9504, 6336, 14))


def batched_uneven(count: int = 48, seed: int = 3, iterations: int = 5) -> list[Develop]:
    """Sizes drawn from BATCH_SENSORS, random CFA phase, black U(256, 1024) (14-bit) or
    U(64, 256) (12-bit), per-image as-shot WB and camera matrix from seeded ranges."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        width, height, bits = BATCH_SENSORS[int(rng.integers(len(BATCH_SENSORS)))]
        cfa = ("RGGB", "BGGR", "GRBG", "GBRG")[int(rng.integers(4))]
        white = float((1 << bits) - 1)
        black = float(rng.uniform(256.0, 1024.0)) if bits == 14 else float(rng.uniform(64.0, 256.0))
        wb = (float(rng.uniform(1.6, 2.4)), 1.0, float(rng.uniform(1.3, 2.0)))
        cam = tuple(float(v) for v in (np.asarray(CAMERA_TO_REC2020) * rng.uniform(0.95, 1.05, 9)))
        vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
        exposure = float(rng.uniform(-0.5, 0.8))
        tone = sixteen_knot_curve(seed=int(rng.integers(1 << 30)))
        hsl = hsl_bands(seed=int(rng.integers(1 << 30)))
        scene = Scene(width, height, cfa, bits, black, white, 0.05, True, wb, seed * 1000 + k)
        out.append(Develop(f"batch_{k}", scene, "opposed", "amaze", Capture(iterations=iterations),
                           Lens(vignetting_k=vig), preview_dimensions(width, height, 2560), wb, cam,
                           exposure_ev=exposure, tone_lut=tone, hsl=hsl))
    return out


def large_export(count: int = 24, seed: int = 5, iterations: int = 20) -> list[Develop]:
    """11648x8736 RGGB 16-bit (white 65535, black 1024) with specular blobs; hot pixels (0.5% of
    samples) come from the generator's hot-pixel draw."""
    out = []
    width, height, bits = 11648, 8736, 16
    for k in range(count):
        rng = np.random.default_rng(seed * 1000 + k)
        wb = (float(rng.uniform(1.7, 2.3)), 1.0, float(rng.uniform(1.4, 1.9)))
        vig = tuple(float(v) for v in (-rng.uniform(0.2, 0.4), rng.uniform(0.02, 0.08), -rng.uniform(0.0, 0.02)))
        scene = Scene(width, height, "RGGB", bits, 1024.0, 65535.0, 0.05, True, wb, seed * 1000 + k,
                      hot_pixel_fraction=0.005)
        out.append(Develop(f"export_{k}", scene, "opposed", "amaze", Capture(iterations=iterations),
                           Lens(vignetting_k=vig), preview_dimensions(width, height, 2560), wb, CAMERA_TO_REC2020,
                           exposure_ev=0.3, tone_lut=sixteen_knot_curve(seed=k), hsl=hsl_bands(seed=k)))
    return out
