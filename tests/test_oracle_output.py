"""Display / extended output oracle pinned to the reference's own tests.

Known answers from crates/color/src/gamut.rs (tests module), crates/color/src/
oklab.rs (tests), crates/core/src/color/display_output.rs (tests),
crates/core/tests/hdr_output.rs, crates/image/src/orientation.rs (tests) and
crates/core/src/geometry.rs (tests), restated against the C oracle in
oracle/output.cpp. The exactly rounded cube root of the oracle's exact-math
mode is checked with rational arithmetic.
"""

import math
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle

F = np.float32
P3_TO_XYZ = np.array([[0.48657095, 0.2656677, 0.1982173], [0.22897456, 0.6917385, 0.07928691],
                      [0.0, 0.04511338, 1.0439444]], dtype=F)
XYZ_TO_REC2020 = np.array([[1.7166512, -0.35567078, -0.2533663], [-0.6666843, 1.6164812, 0.015768546],
                           [0.017639857, -0.042770613, 0.94210315]], dtype=F)


def then(first, nxt):
    """Matrix3::then with the sum starting at -0.0, in f32."""
    out = np.zeros((3, 3), dtype=F)
    for r in range(3):
        for c in range(3):
            s = F(-0.0)
            for k in range(3):
                s = F(s + F(nxt[r, k] * first[k, c]))
            out[r, c] = s
    return out


def transform(m, v):
    v = [F(x) for x in v]
    return np.array([F(F(F(m[r, 0] * v[0]) + F(m[r, 1] * v[1])) + F(m[r, 2] * v[2])) for r in range(3)], dtype=F)


def p3_to_rec2020(p3):
    return transform(then(P3_TO_XYZ, XYZ_TO_REC2020), p3)


def srgb_encode(v):
    v = F(v)
    return F(12.92) * v if v <= F(0.0031308) else F(F(F(1.055) * F(np.power(v, F(1.0) / F(2.4)))) - F(0.055))


def image(pixels, w=3, h=2):
    return np.array(pixels, dtype=F).reshape(h, 3 * w)


# ---- gamut.rs ---------------------------------------------------------------
def test_in_gamut_values_are_bit_exact():
    for rgb in ([0, 0, 0], [1, 1, 1], [0.13, 0.47, 0.91], [np.finfo(F).tiny, 0.5, 1.0 - np.finfo(F).eps]):
        src = np.array(rgb, dtype=F)
        out, status = oracle.gamut_map(src)
        assert status == "in_gamut" and out.tobytes() == src.tobytes()


def test_saturated_values_compress_without_independent_channel_clipping():
    for rgb in ([1.4, 0.2, 0.1], [-0.2, 0.7, 1.3], [2.0, -0.4, 0.8], [0.2, 1.8, -0.3]):
        out, status = oracle.gamut_map(rgb)
        assert np.all((out >= 0) & (out <= 1))
        assert status in ("compressed", "limited")
        assert not np.array_equal(out, np.clip(np.array(rgb, dtype=F), 0, 1))


def test_oklab_round_trip_handles_asymmetric_signed_values():
    for rgb in ([0.17, 0.43, 0.81], [-0.08, 0.61, 1.24], [1.7, -0.2, 0.35]):
        back = oracle.oklab(oracle.oklab(rgb), inverse=True)
        assert np.max(np.abs(back - np.array(rgb, dtype=F))) <= 2.0e-6


def test_compression_preserves_oklch_hue_and_lightness_when_feasible():
    src = [1.4, 0.2, 0.1]
    out, _ = oracle.gamut_map(src)
    a, b = oracle.oklab(src), oracle.oklab(out)
    assert abs(math.atan2(a[2], a[1]) - math.atan2(b[2], b[1])) < 2.0e-5
    assert abs(a[0] - b[0]) < 2.0e-5
    assert math.hypot(b[1], b[2]) < math.hypot(a[1], a[2])


def test_mapping_is_continuous_across_an_srgb_boundary():
    inside, _ = oracle.gamut_map([1.0, 0.2, 0.1])
    outside, _ = oracle.gamut_map([1.0001, 0.2, 0.1])
    assert np.max(np.abs(inside - outside)) < 0.002


def test_gray_axis_and_lightness_limits_remain_neutral():
    for rgb, expected in (([-0.25] * 3, [0.0] * 3), ([1.25] * 3, [1.0] * 3)):
        out, status = oracle.gamut_map(rgb)
        assert np.max(np.abs(out - np.array(expected, dtype=F))) <= 2.0e-6 and status == "limited"


def test_invalid_values_never_escape_as_non_finite():
    for rgb in ([np.nan, 0.5, 1.0], [np.inf, 0.5, -np.inf]):
        out, status = oracle.gamut_map(rgb)
        assert status == "invalid" and np.all(np.isfinite(out))


def test_p3_values_inside_p3_but_outside_srgb_are_preserved():
    out, status = oracle.gamut_map([0.0, 0.9, 0.1], "display_p3")
    assert status == "in_gamut" and np.array_equal(out, np.array([0.0, 0.9, 0.1], dtype=F))


def test_p3_compression_keeps_hue_and_lands_in_the_p3_gamut():
    src = [-0.12, 1.15, 0.2]
    out, status = oracle.gamut_map(src, "display_p3")
    assert np.all((out >= 0) & (out <= 1)) and status == "compressed"
    a, b = oracle.oklab(src, "display_p3"), oracle.oklab(out, "display_p3")
    assert abs(math.atan2(a[2], a[1]) - math.atan2(b[2], b[1])) < 2.0e-4
    assert abs(a[0] - b[0]) < 2.0e-4


def test_ceiling_keeps_highlights_above_diffuse_white():
    bright = np.array([3.2, 2.5, 1.1], dtype=F)
    out, status = oracle.gamut_map(bright, "display_p3", ceiling=4.0)
    assert status == "in_gamut" and np.array_equal(out, bright)
    out, _ = oracle.gamut_map([3.0, -0.2, 1.0], "display_p3", ceiling=4.0)
    assert np.all((out >= 0) & (out <= 4)) and out[0] > 1.5


def test_values_above_the_ceiling_are_limited_and_stay_neutral():
    out, status = oracle.gamut_map([9.0] * 3, "display_p3", ceiling=4.0)
    assert status == "limited" and np.max(np.abs(out - 4.0)) <= 1.0e-4


def test_clipping_respects_the_ceiling_for_invalid_values():
    out, status = oracle.gamut_map([np.inf, -1.0, 2.5], policy="clip", ceiling=4.0)
    assert list(out) == [4.0, 0.0, 2.5] and status == "invalid"


# ---- oklab.rs ---------------------------------------------------------------
def test_display_p3_oklab_round_trips_asymmetric_values():
    for rgb in ([0.17, 0.43, 0.81], [-0.05, 0.61, 1.3], [1.5, -0.1, 0.3]):
        back = oracle.oklab(oracle.oklab(rgb, "display_p3"), "display_p3", inverse=True)
        assert np.max(np.abs(back - np.array(rgb, dtype=F))) < 3.0e-6


def test_p3_neutral_axis_stays_neutral_in_oklab():
    lab = oracle.oklab([0.4, 0.4, 0.4], "display_p3")
    assert abs(lab[1]) < 1.0e-4 and abs(lab[2]) < 1.0e-4


# ---- display_output.rs ------------------------------------------------------
def test_p3_encoding_round_trips_a_p3_colour_that_srgb_must_compress():
    p3 = [0.05, 0.8, 0.12]
    img = image([p3_to_rec2020(p3)], 1, 1)
    out, gamut = oracle.render_output(img, oracle.output_desc("extended_f32", "display_p3", "chroma_compress"))
    assert gamut[0] == 1  # in gamut
    enc = [srgb_encode(v) for v in out[0]]
    assert max(abs(e - srgb_encode(v)) for e, v in zip(enc, p3)) < 1.0e-4
    _, gamut = oracle.render_output(img, oracle.output_desc("srgb8", "srgb", "chroma_compress"))
    assert gamut[1] == 1  # compressed


def test_extended_ceiling_passes_highlights_that_the_sdr_ceiling_limits():
    img = image([[3.0, 3.0, 3.0]], 1, 1)
    sdr = oracle.render_output(img, oracle.output_desc("srgb8", "display_p3", "chroma_compress"))[1]
    out, hdr = oracle.render_output(img, oracle.output_desc("extended_f32", "display_p3", "chroma_compress",
                                                            headroom=4.0))
    assert sdr[2] == 1 and hdr[0] == 1
    assert abs(out[0, 1] - 3.0) < 1.0e-3


# ---- crates/core/tests/hdr_output.rs ----------------------------------------
def test_p3_8_bit_matches_srgb_on_neutrals_in_every_position():
    img = image([[v] * 3 for v in (0.0, 0.02, 0.18, 0.4, 0.75, 1.0)])
    for orientation in ("normal", "rotate90"):
        p3, _ = oracle.render_output(img, oracle.output_desc("srgb8", "display_p3", "chroma_compress",
                                                             orientation=orientation))
        srgb, _ = oracle.render_output(img, oracle.output_desc("srgb8", "srgb", "chroma_compress",
                                                               orientation=orientation))
        assert p3.shape == srgb.shape and np.array_equal(p3, srgb)


def test_p3_8_bit_keeps_colours_that_srgb_cannot_represent():
    p3_linear = [0.05, 0.8, 0.12]
    pixels = [[0.5] * 3 for _ in range(6)]
    pixels[4] = list(p3_to_rec2020(p3_linear))
    img = image(pixels)
    expected = [int(np.round(F(srgb_encode(v) * F(255.0)))) for v in p3_linear]
    for policy in ("clip", "chroma_compress"):
        p3, _ = oracle.render_output(img, oracle.output_desc("srgb8", "display_p3", policy))
        assert list(p3[1, 3:6]) == expected, policy
    srgb, _ = oracle.render_output(img, oracle.output_desc("srgb8", "srgb", "chroma_compress"))
    p3, _ = oracle.render_output(img, oracle.output_desc("srgb8", "display_p3", "chroma_compress"))
    assert list(srgb[1, 3:6]) != list(p3[1, 3:6])


def test_extended_output_keeps_values_above_diffuse_white_and_orientation():
    values = (0.25, 0.5, 1.0, 1.5, 2.5, 3.5)
    img = image([[v] * 3 for v in values])

    def render(orientation):
        out, _ = oracle.render_output(img, oracle.output_desc("extended_f32", "display_p3", "chroma_compress",
                                                              orientation=orientation, headroom=4.0))
        px = out.reshape(out.shape[0], -1, 3)
        assert np.all(np.abs(px[..., 0] - px[..., 1]) < 1.0e-4) and np.all(np.abs(px[..., 2] - px[..., 1]) < 1.0e-4)
        return px[..., 1]

    normal = render("normal")
    assert np.all(np.abs(normal.reshape(-1) - np.array(values)) < 1.0e-4)
    rotated = render("rotate90")  # EXIF 6: [[a, b, c], [d, e, f]] -> [[d, a], [e, b], [f, c]]
    assert rotated.shape == (3, 2)
    assert np.all(np.abs(rotated - np.array([[1.5, 0.25], [2.5, 0.5], [3.5, 1.0]])) < 1.0e-4)


def test_extended_output_has_a_p3_base_with_a_per_pixel_ratio():
    p3_linear = [2.0, 1.2, 0.4]
    pixels = [[0.5] * 3 for _ in range(6)]
    pixels[0] = list(p3_to_rec2020(p3_linear))
    out, gamut = oracle.render_output(image(pixels), oracle.output_desc("extended_f32", "display_p3",
                                                                        "chroma_compress", headroom=4.0))
    assert np.all(np.abs(out[0, :3] - np.array(p3_linear)) < 1.0e-4)
    assert gamut.sum() == 6 and gamut[0] == 6


def test_extended_output_maps_out_of_gamut_colours_into_the_range():
    pixels = [[1.0] * 3 for _ in range(6)]
    pixels[0] = [0.0, 1.0, 0.0]
    pixels[1] = [3.0] * 3
    for policy in ("clip", "chroma_compress"):
        out, gamut = oracle.render_output(image(pixels), oracle.output_desc("extended_f32", "display_p3", policy,
                                                                            headroom=4.0))
        assert np.all((out >= 0) & (out <= 4)), policy
        assert abs(out[0, 4] - 3.0) < 1.0e-4 and gamut[0] == 5, policy


def test_extended_output_rejects_bad_headroom():
    img = image([[0.5] * 3 for _ in range(6)])
    for headroom in (0.5, float("nan"), float("inf")):
        assert oracle.render_output(img, oracle.output_desc("extended_f32", "display_p3", headroom=headroom)) is None


# ---- orientation.rs / geometry.rs -------------------------------------------
def test_orientation_map_rejects_out_of_range_and_maps_rotate90():
    assert oracle.output_geometry(2, 3, oracle.output_desc(orientation="rotate90"))[:2] == (3, 2)
    import ctypes
    sx, sy = ctypes.c_int(), ctypes.c_int()
    oracle.load().ro_source_coordinate(2, 3, 5, 0, 0, sx, sy)
    assert (sx.value, sy.value) == (0, 2)


def test_every_orientation_is_a_bijection_matching_its_inverse():
    # Each orientation permutes the pixels; the oriented image of an index grid
    # holds every source index exactly once, and a second application of the
    # self-inverse orientations restores the grid.
    w, h = 5, 3
    idx = np.arange(w * h, dtype=F)
    img = np.repeat(idx, 3).reshape(h, 3 * w) / F(w * h)
    for k, name in enumerate(oracle.ORIENTATIONS):
        out, _ = oracle.render_output(img, oracle.output_desc("extended_f32", orientation=name, headroom=1.0))
        got = np.round(out[:, 0::3] * (w * h)).astype(int)
        swapped = name in ("transpose", "rotate90", "transverse", "rotate270")
        assert got.shape == ((w, h) if swapped else (h, w))
        assert sorted(got.reshape(-1)) == list(range(w * h))


def test_adjusted_geometry_follows_the_orientation_override_and_the_crop():
    assert oracle.output_geometry(600, 400, oracle.output_desc())[:2] == (600, 400)
    assert oracle.output_geometry(600, 400, oracle.output_desc(orientation="rotate90"))[:2] == (400, 600)
    geo = oracle.output_geometry(600, 400, oracle.output_desc(orientation="rotate90",
                                                              crop=(0.25, 0.0, 0.75, 0.5)))
    assert geo[:2] == (200, 300) and geo[2] == (100, 0, 300, 300)
    for crop in ((0.5, 0.0, 0.5, 1.0), (0.0, 0.0, 1.5, 1.0), (float("nan"), 0.0, 1.0, 1.0), (0.0, 0.0, 0.0004, 1.0)):
        assert oracle.output_geometry(600, 400, oracle.output_desc(crop=crop)) is None


# ---- correctly rounded cube root --------------------------------------------
def _is_correctly_rounded_cbrt(x: float, y: float) -> bool:
    y32 = np.float32(y)
    below = float(np.nextafter(y32, np.float32(0)))
    above = float(np.nextafter(y32, np.float32(np.inf)))
    lo = (Fraction(float(y32)) + Fraction(below)) / 2
    hi = (Fraction(float(y32)) + Fraction(above)) / 2
    fx = Fraction(x)
    return lo ** 3 < fx < hi ** 3


def test_correctly_rounded_cube_root_on_a_sample():
    rng = np.random.default_rng(7)
    bits = rng.integers(1, 0x7F800000, size=4000, dtype=np.uint32)
    xs = bits.view(np.float32)
    lib = oracle.load()
    for x in xs:
        y = lib.ro_cbrt_correctly_rounded(float(x))
        assert _is_correctly_rounded_cbrt(float(x), y), x
        assert lib.ro_cbrt_correctly_rounded(-float(x)) == -y
    # Exact cubes stay exact.
    for k in (1, 2, 3, 10, 1000):
        assert lib.ro_cbrt_correctly_rounded(float(k ** 3)) == k


def test_exact_math_mode_switches_the_cube_root_and_transfer():
    lib = oracle.load()
    x = float(np.float32(0.7))
    try:
        oracle.set_exact_math(True)
        assert lib.ro_cbrt(x) == lib.ro_cbrt_correctly_rounded(x)
    finally:
        oracle.set_exact_math(False)


def test_libm_and_exact_modes_agree_on_clip_outputs():
    """The clip policy uses no cube root; the transfer differs from the correctly
    rounded one on too few f32 inputs to meet a random 8-bit or 16-bit image."""
    rng = np.random.default_rng(3)
    img = rng.uniform(-0.2, 1.3, size=(48, 3 * 64)).astype(F)
    outs = []
    for exact in (False, True):
        oracle.set_exact_math(exact)
        try:
            outs.append([oracle.render_output(img, oracle.output_desc(fmt, policy="clip"))[0]
                         for fmt in ("srgb8", "srgb16", "extended_f32")])
        finally:
            oracle.set_exact_math(False)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
