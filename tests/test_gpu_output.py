"""Display and extended-range output on the GPU against the oracle.

The CUDA path computes the OkLab cube root and the sRGB transfer power
correctly rounded. Against the oracle's exact-math mode (the same functions)
every format, policy, primaries, orientation, crop and dither is bit-exact,
and so are the gamut diagnostics. Against the oracle's libm mode (what the
reference computes with glibc's cbrtf / powf) the clip policy stays bit-exact
and chroma compression stays within the bounds below, measured on the oracle
itself between its two modes: 8-bit codes within 1, 16-bit codes within 32
(the reference's own GPU export allows 16), linear values within 5e-5.
"""

import numpy as np
import pytest

from rohditor_gb300 import ColorContract, GpuPreviewError, OutputSpec

pytestmark = pytest.mark.gpu

FORMATS = ("srgb8", "srgb16", "extended_f32", "extended_f16")
ORIENTATIONS = ("normal", "horizontal_flip", "rotate180", "vertical_flip", "transpose", "rotate90", "transverse",
                "rotate270", "unknown")


def wide_gamut_image(w, h, seed, highlights=1.4):
    """Linear Rec.2020 with saturated colours outside sRGB and P3, negatives,
    highlights above diffuse white and a few non-finite samples."""
    rng = np.random.default_rng(seed)
    img = rng.uniform(-0.08, highlights, size=(h, w, 3)).astype(np.float32)
    img[..., 0] *= rng.uniform(0.0, 1.0, size=(h, w)).astype(np.float32)
    img[..., 2] *= rng.uniform(0.0, 1.0, size=(h, w)).astype(np.float32)
    img[0, 0] = (np.nan, 0.5, 0.5)
    img[0, 1] = (np.inf, 0.2, -np.inf)
    img[1, 0] = (3.0, 3.0, 3.0)
    img[1, 1] = (0.0, 0.0, 0.0)
    return img.reshape(h, 3 * w)


def adjustments(**kw):
    from rohditor_gb300 import standard_base_lut
    from rohditor_gb300.workloads import hsl_bands, sixteen_knot_curve

    base = dict(exposure_ev=0.3, base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=2),
                saturation=1.15, vibrance=0.2, hsl=hsl_bands(seed=3))
    base.update(kw)
    return ColorContract(**base)


def oracle_output(oracle, rgb, color, spec, exact):
    x = oracle.adjust(rgb, color.exposure_ev, color.base_lut, color.tone_lut, color.saturation, color.vibrance,
                      color.hsl, color.grading, light_lut=color.light_tone_lut,
                      extended=spec.format.startswith("extended"))
    fmt = "extended_f32" if spec.format == "extended_f16" else spec.format
    desc = oracle.output_desc(fmt, spec.primaries, spec.policy, spec.dither, spec.orientation, spec.crop,
                              spec.headroom)
    oracle.set_exact_math(exact)
    try:
        res = oracle.render_output(x, desc)
    finally:
        oracle.set_exact_math(False)
    out, gamut = res
    if spec.format == "extended_f16":
        out = out.astype(np.float16)
    return out, gamut


def same_bits(a, b):
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(
        a.view(np.uint8).reshape(-1), b.view(np.uint8).reshape(-1))


def test_cube_root_is_correctly_rounded_for_every_f32(stages):
    assert stages.check_math(0) == 0


def test_transfer_power_is_within_the_quantisation_bound(stages):
    assert stages.check_math(1) <= 1


def test_transfer_power_is_correctly_rounded_for_every_f32(stages):
    assert stages.check_math(2) == 0


def test_quantised_codes_follow_the_correctly_rounded_power_for_every_f32(stages):
    assert stages.check_math(3) == 0


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("policy", ["clip", "chroma_compress"])
@pytest.mark.parametrize("primaries", ["srgb", "display_p3"])
def test_output_bit_exact_against_exact_math(stages, oracle, fmt, policy, primaries):
    rgb = wide_gamut_image(133, 71, seed=11)
    color = adjustments()
    spec = OutputSpec(format=fmt, primaries=primaries, policy=policy, headroom=2.5,
                      dither="ordered8x8" if fmt == "srgb16" else "none")
    ours, hist, gamut = stages.output(rgb, color, spec, histogram=fmt == "srgb8")
    ref, ref_gamut = oracle_output(oracle, rgb, color, spec, exact=True)
    assert same_bits(ours, ref)
    assert np.array_equal(gamut, ref_gamut) and int(gamut.sum()) == 133 * 71
    if fmt == "srgb8":
        ref_hist, _ = oracle.histogram(ref)
        assert np.array_equal(hist, ref_hist)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("sliders", [(0.5, -0.6, 0.4, -1.0, 0.3), (-0.7, 0.8, -0.5, 0.6, -0.4)])
def test_light_tone_in_every_rendition(stages, oracle, fmt, sliders):
    """The Light tone step (contrast, highlights, shadows, whites, blacks) between the base
    rendering and the tone curve: SDR formats sample the table, extended formats continue it
    above 1 with unit slope (LightToneLut::sample_extended); lowered Whites make the two differ."""
    from rohditor_gb300 import light_tone_lut

    rgb = wide_gamut_image(127, 67, seed=21, highlights=3.0)
    color = adjustments(light_tone_lut=light_tone_lut(*sliders))
    spec = OutputSpec(format=fmt, primaries="srgb", policy="clip", headroom=4.0)
    ours, hist, gamut = stages.output(rgb, color, spec, histogram=fmt == "srgb8")
    ref, ref_gamut = oracle_output(oracle, rgb, color, spec, exact=True)
    assert same_bits(ours, ref)
    assert np.array_equal(gamut, ref_gamut)
    if fmt.startswith("extended"):
        # The step is live above 1 in the extended rendition: an SDR-sampled table gives other values.
        sdr = oracle.adjust(rgb, color.exposure_ev, color.base_lut, color.tone_lut, color.saturation,
                            color.vibrance, color.hsl, color.grading, light_lut=color.light_tone_lut, extended=False)
        ext = oracle.adjust(rgb, color.exposure_ev, color.base_lut, color.tone_lut, color.saturation,
                            color.vibrance, color.hsl, color.grading, light_lut=color.light_tone_lut, extended=True)
        assert not np.array_equal(sdr, ext)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("policy", ["clip", "chroma_compress"])
def test_output_against_the_platform_libm(stages, oracle, fmt, policy):
    rgb = wide_gamut_image(160, 96, seed=12)
    color = adjustments()
    spec = OutputSpec(format=fmt, primaries="display_p3", policy=policy, headroom=2.0)
    ours, _, gamut = stages.output(rgb, color, spec)
    ref, ref_gamut = oracle_output(oracle, rgb, color, spec, exact=False)
    assert np.array_equal(gamut, ref_gamut)
    if policy == "clip":
        assert same_bits(ours, ref)
        return
    d = np.abs(ours.astype(np.float64) - ref.astype(np.float64))
    bound = {"srgb8": 1, "srgb16": 32, "extended_f32": 5e-5, "extended_f16": 2e-3}[fmt]
    assert d.max() <= bound
    if fmt == "srgb8":
        assert (d > 0).mean() <= 1e-3


@pytest.mark.parametrize("orientation", ORIENTATIONS)
def test_orientation_and_crop(stages, oracle, orientation):
    rgb = wide_gamut_image(97, 61, seed=13)
    color = adjustments(hsl=None)
    for crop in (None, (0.13, 0.21, 0.77, 0.94)):
        for fmt in ("srgb8", "extended_f32"):
            spec = OutputSpec(format=fmt, policy="chroma_compress", orientation=orientation, crop=crop, headroom=1.5)
            ours, hist, gamut = stages.output(rgb, color, spec, histogram=fmt == "srgb8")
            ref, ref_gamut = oracle_output(oracle, rgb, color, spec, exact=True)
            assert same_bits(ours, ref), (orientation, crop, fmt)
            assert np.array_equal(gamut, ref_gamut)


def test_dithered_outputs_follow_the_output_coordinates(stages, oracle):
    rgb = wide_gamut_image(75, 44, seed=14)
    color = adjustments(base_lut=None)
    for fmt in ("srgb8", "srgb16"):
        for orientation in ("normal", "rotate270"):
            spec = OutputSpec(format=fmt, dither="ordered8x8", orientation=orientation, crop=(0.05, 0.1, 0.9, 1.0))
            ours, _, _ = stages.output(rgb, color, spec)
            ref, _ = oracle_output(oracle, rgb, color, spec, exact=True)
            assert same_bits(ours, ref)


def test_large_tile_spanning_output(stages, oracle):
    """Several 32x32 tiles per CTA and ragged tile edges on both axes."""
    rgb = wide_gamut_image(1031, 517, seed=15, highlights=3.0)
    color = adjustments()
    for orientation in ("normal", "rotate90"):
        spec = OutputSpec(format="extended_f16", primaries="display_p3", policy="chroma_compress",
                          orientation=orientation, headroom=4.0)
        ours, _, gamut = stages.output(rgb, color, spec)
        ref, ref_gamut = oracle_output(oracle, rgb, color, spec, exact=True)
        assert same_bits(ours, ref) and np.array_equal(gamut, ref_gamut)


def test_invalid_output_descriptions_are_rejected(stages):
    rgb = wide_gamut_image(16, 8, seed=16)
    color = adjustments()
    bad = [OutputSpec(format="extended_f32", headroom=0.5), OutputSpec(format="extended_f16", headroom=float("nan")),
           OutputSpec(crop=(0.5, 0.0, 0.5, 1.0)), OutputSpec(crop=(0.0, 0.0, 1.2, 1.0)),
           OutputSpec(crop=(0.0, 0.0, 0.01, 1.0))]
    for spec in bad:
        with pytest.raises(GpuPreviewError) as err:
            stages.output(rgb, color, spec)
        assert err.value.code == 8  # RD_INVALID_INPUT
    with pytest.raises(GpuPreviewError):
        stages.output(rgb, color, OutputSpec(format="srgb16"), histogram=True)


def test_render_output_of_a_base_matches_render_and_the_stage(device, oracle):
    """rd_render_output on a developed full-resolution base: the 8-bit normal,
    uncropped, clipped output equals rd_render; every format equals the stage
    entry point on the downloaded base."""
    from rohditor_gb300 import (CaptureContract, GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor,
                                OpticsExecution, SensorDescription, Stages, clip_levels)
    from rohditor_gb300.workloads import CAMERA_TO_REC2020

    w, h = 640, 480
    rng = np.random.default_rng(21)
    raw = rng.integers(300, 4000, size=(h, w), dtype=np.uint16)
    wb = (2.0, 1.0, 1.6)
    desc = SensorDescription(w, h, cfa="RGGB", black=(256.0,), white=(4095.0,), highlight="clip",
                             clip_levels=clip_levels(1.0, wb), demosaic="amaze", demosaic_balance=wb)
    cap = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=clip_levels(1.0, wb), iterations=4)
    src = GpuSensorProcessor(device).develop(raw, desc, cap)
    base = GpuSpatialProcessor(device).reduce_preview(src, OpticsExecution(w, h), (w, h), wb, CAMERA_TO_REC2020)
    color = adjustments(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020)
    preview = GpuPreviewProcessor(device)
    ref8, ref_hist = preview.render(base, color)
    out8, hist8, gamut8 = preview.render_output(base, color, OutputSpec(), histogram=True)
    assert np.array_equal(out8, ref8) and np.array_equal(hist8.luminance, ref_hist.luminance)
    assert gamut8.total == w * h
    planar = base.download()
    stages = Stages(device)
    for spec in (OutputSpec(format="srgb16", policy="chroma_compress", orientation="rotate90"),
                 OutputSpec(format="extended_f16", primaries="display_p3", policy="chroma_compress", headroom=4.0,
                            crop=(0.1, 0.1, 0.9, 0.8))):
        ours, _, gamut = preview.render_output(base, color, spec)
        staged, _, staged_gamut = stages.output(planar, color, spec)
        assert same_bits(ours, staged)
        assert gamut.total == int(staged_gamut.sum())
    base.release()
    src.release()
