"""The reference's own behavioural tests of capture sharpening, Opposed and the
colour chain, restated and run against both the oracle (CPU) and the GPU path.

The reference holds no golden values for these stages, only behaviour; each
test below restates one of its tests with the same fixture and the same
assertions, and every `gpu` run also checks the GPU result equal to the
oracle's bit for bit (Opposed samples within 1e-4, the tolerance its
cube-root / log2 libm difference needs).

  capture sharpening   crates/core/src/sharpening/tests.rs:23-213
  Opposed              crates/highlight/tests/opposed.rs:77-526
  colour chain         crates/gpu/src/preview/color_tests.rs:59-227 (fixture and
                       recipe sweep; the reference allows 2e-5 + 0.15% linear
                       and 2 codes, the GPU here is bit-exact)
"""

import ctypes

import numpy as np
import pytest

IMPLS = ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)]
CFA = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}
COLORS = {"RGGB": ((0, 1), (1, 2)), "BGGR": ((2, 1), (1, 0)), "GRBG": ((1, 0), (2, 1)), "GBRG": ((1, 2), (0, 1))}


def color_at(pattern, x, y):
    return COLORS[pattern][y & 1][x & 1]


class Rejected(Exception):
    pass


@pytest.fixture(params=IMPLS)
def impl(request, oracle):
    if request.param == "oracle":
        return OracleImpl(oracle)
    stages = request.getfixturevalue("stages")
    return GpuImpl(stages, oracle)


class OracleImpl:
    name = "oracle"

    def __init__(self, o):
        self.o = o

    def capture(self, rgb, enabled=True, amount=0.5, radius=0.6, noise=0.5, ceilings=(1.0, 1.0, 1.0)):
        if not enabled:  # CaptureSharpening::is_active (crates/edit/src/sharpening.rs:47-49)
            return np.array(rgb, dtype=np.float32, copy=True)
        if not (0.3 <= radius <= 1.2):
            raise Rejected("radius")
        try:
            return self.o.capture(rgb, amount, radius, noise, ceilings, 8)
        except ValueError as e:
            raise Rejected(str(e))

    def opposed(self, mosaic, pattern, levels, ceiling=None):
        try:
            m, stats, _, _ = self.o.opposed(mosaic, CFA[pattern], levels, ceiling)
        except ValueError as e:
            raise Rejected(str(e))
        return m, stats


class GpuImpl:
    name = "gpu"

    def __init__(self, stages, o):
        self.stages = stages
        self.ref = OracleImpl(o)

    def capture(self, rgb, enabled=True, amount=0.5, radius=0.6, noise=0.5, ceilings=(1.0, 1.0, 1.0)):
        from rohditor_gb300 import CaptureContract, GpuPreviewError

        c = CaptureContract(amount=amount, radius=radius, noise_protection=noise, ceilings=ceilings, iterations=8,
                            enabled=enabled)
        try:
            out = self.stages.capture(rgb, c)
        except GpuPreviewError as e:
            raise Rejected(str(e))
        ref = self.ref.capture(rgb, enabled, amount, radius, noise, ceilings)
        assert out.view(np.uint32).tolist() == ref.view(np.uint32).tolist(), "GPU capture differs from the oracle"
        return out

    def opposed(self, mosaic, pattern, levels, ceiling=None):
        from rohditor_gb300 import GpuPreviewError

        try:
            out, stats, _, _ = self.stages.opposed(mosaic, pattern, levels, ceiling)
        except GpuPreviewError as e:
            raise Rejected(str(e))
        ref, ref_stats = self.ref.opposed(mosaic, pattern, levels, ceiling)
        assert np.array_equal(stats, ref_stats)
        assert float(np.max(np.abs(out - ref))) <= 1e-4
        return out, stats


# ---------------------------------------------------------------- capture sharpening
def gray_image(width, height, guide):
    g = np.asarray(guide, dtype=np.float32).reshape(height, width)
    return np.repeat(g[:, :, None], 3, axis=2).reshape(height, 3 * width)


def capture_fixture(width, height):
    out = np.full((height, width), 0.2, dtype=np.float32)
    for y in range(height):
        for x in range(width):
            if (width // 3 < x < width * 2 // 3 and y > height // 4) or (x == 3 and y == 5):
                out[y, x] = 0.65
    return out


def gaussian(oracle, radius):
    buf = (ctypes.c_float * 64)()
    n = oracle.load().ro_gaussian_kernel(ctypes.c_float(radius), buf, 64)
    return np.array(buf[:n], dtype=np.float32)


def mirror(index, length):
    period = 2 * length
    folded = index % period
    return folded if folded < length else 2 * length - 1 - folded


def blurred(oracle, image):
    """sharpening.rs blur (separable, half-sample mirror) with gaussian(0.6), in f32."""
    k = gaussian(oracle, 0.6)
    r = len(k) // 2
    h, w = image.shape
    tmp = np.zeros_like(image)
    for x in range(w):
        acc = np.zeros(h, dtype=np.float32)
        for j, wt in enumerate(k):
            acc = (acc + image[:, mirror(x + j - r, w)] * wt).astype(np.float32)
        tmp[:, x] = acc
    out = np.zeros_like(image)
    for y in range(h):
        acc = np.zeros(w, dtype=np.float32)
        for j, wt in enumerate(k):
            acc = (acc + tmp[mirror(y + j - r, h)] * wt).astype(np.float32)
        out[y] = acc
    return out


def mse(a, b):
    return float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))


def test_capture_disabled_and_zero_amount_are_bit_exact_with_signed_hdr(impl):
    data = np.array([[-0.0, -0.1, 2.0, 0.2, 0.3, 0.4]], dtype=np.float32)
    for kw in ({"enabled": False}, {"amount": 0.0}):
        out = impl.capture(data, **kw)
        assert out.view(np.uint32).tolist() == data.view(np.uint32).tolist()


@pytest.mark.parametrize("size", [(1, 1), (1, 7), (9, 1), (3, 5)])
def test_capture_constants_and_tiny_images_remain_unchanged(impl, size):
    w, h = size
    for value in (-0.1, 0.0, 0.2, 1.0, 2.0):
        img = gray_image(w, h, np.full(w * h, value))
        out = impl.capture(img)
        assert np.array_equal(out, img)


def test_capture_recovers_a_known_blur_with_bounded_overshoot(impl, oracle):
    original = capture_fixture(53, 37)
    observation = blurred(oracle, original)
    usm = observation + 0.5 * (observation - blurred(oracle, observation))
    out = impl.capture(gray_image(53, 37, observation))
    sharpened = out.reshape(37, 53, 3)[:, :, 0]
    off_error, rl_error, usm_error = mse(observation, original), mse(sharpened, original), mse(usm, original)
    overshoot = max(float(sharpened.max()), 0.65) - 0.65
    undershoot = 0.2 - min(float(sharpened.min()), 0.2)
    assert rl_error < off_error * 0.9, (off_error, rl_error, usm_error)
    assert overshoot < 0.025 and undershoot < 0.025


def test_capture_mask_protects_flat_noise_and_highlight_boundaries(impl):
    i = np.arange(53 * 37)
    noise = (0.15 + (((i * 7919) % 101).astype(np.float32) / 100.0 - 0.5) * 0.002).astype(np.float32)
    out = impl.capture(gray_image(53, 37, noise)).reshape(-1, 3)[:, 0]
    mean = np.full(noise.shape, 0.15)
    assert np.sqrt(mse(out, mean) / mse(noise, mean)) <= 1.01
    clipped = np.where(np.arange(63) % 9 > 3, 1.0, 0.1).astype(np.float32)
    res = impl.capture(gray_image(9, 7, clipped)).reshape(-1, 3)
    for k in range(63):
        if k % 9 > 3:
            assert res[k].tolist() == [1.0, 1.0, 1.0]


def test_capture_gain_preserves_signed_channel_ratios_and_is_deterministic(impl, oracle):
    guide = blurred(oracle, capture_fixture(53, 37))
    img = gray_image(53, 37, guide).reshape(-1, 3)
    img[:, 0] *= np.float32(-0.2)
    img[:, 2] *= np.float32(2.0)
    img = img.reshape(37, 3 * 53)
    a = impl.capture(img, ceilings=(10.0, 10.0, 10.0))
    b = impl.capture(img, ceilings=(10.0, 10.0, 10.0))
    assert np.array_equal(a, b)
    assert not np.array_equal(a, img)
    px = a.reshape(-1, 3)
    assert np.all(np.abs(px[:, 0] / px[:, 1] + 0.2) < 1e-6)
    assert np.all(np.abs(px[:, 2] / px[:, 1] - 2.0) < 1e-6)


def test_capture_invalid_settings_and_non_finite_samples_are_rejected(impl):
    img = gray_image(3, 5, capture_fixture(3, 5))
    with pytest.raises(Rejected):
        impl.capture(img, radius=float("nan"))
    bad = img.copy()
    bad.reshape(-1)[4] = np.inf
    with pytest.raises(Rejected):
        impl.capture(bad)


# ---------------------------------------------------------------- Opposed
def double_clipped(pattern):
    m = np.full((14, 14), 0.01, dtype=np.float32)
    for y in range(14):
        for x in range(14):
            c = color_at(pattern, x, y)
            if (x // 2, y // 2) == (3, 3):
                m[y, x] = 0.8 if c == 2 else 0.9
            elif (x // 2, y // 2) in ((2, 2), (3, 2), (4, 2)):
                m[y, x] = (0.8, 0.7, 0.4)[c]
    return m


def single_clipped():
    m = np.full((14, 14), 0.01, dtype=np.float32)
    for y in range(14):
        for x in range(14):
            c = color_at("RGGB", x, y)
            if (x // 2, y // 2) == (3, 3):
                m[y, x] = (0.9, 0.88, 0.44)[c]
            elif (x // 2, y // 2) in ((2, 2), (3, 2), (4, 2)):
                m[y, x] = (0.75, 0.5, 0.25)[c]
    return m


def blown_cell():
    m = np.full((5, 5), 0.2, dtype=np.float32)
    m[:2, :2] = 1.0
    return m


L09 = (0.9, 0.9, 0.9)
# OpposedStats order: suspected, reconstructed, changed, fallback, fully_unsupported, neutralised, by channel.
SUSPECTED, RECONSTRUCTED, CHANGED, FALLBACK, UNSUPPORTED, NEUTRALISED = range(6)


def test_opposed_recovers_multiple_clipped_channels(impl):
    out, stats = impl.opposed(double_clipped("RGGB"), "RGGB", L09)
    assert stats.tolist() == [3, 3, 3, 0, 0, 0, 1, 2, 0]
    assert out[6, 6] > 0.9 and out[6, 7] > 0.9 and out[7, 6] > 0.9


@pytest.mark.parametrize("pattern", ["RGGB", "BGGR", "GRBG", "GBRG"])
def test_opposed_all_bayer_phases_recover_their_center_channels(impl, pattern):
    _, stats = impl.opposed(double_clipped(pattern), pattern, L09)
    assert stats[SUSPECTED] == 3 and stats[RECONSTRUCTED] == 3


def test_opposed_one_channel_recovery_is_bounded(impl):
    out, stats = impl.opposed(single_clipped(), "RGGB", (0.9, 1.0, 1.0))
    assert stats[SUSPECTED] == 1 and stats[RECONSTRUCTED] == 1 and stats[CHANGED] == 1
    assert np.isfinite(out[6, 6]) and out[6, 6] > 0.9
    assert np.all(np.isfinite(out)) and np.all(out <= 3.6)


def test_opposed_ratio_guard_rejects_a_red_green_edge_candidate(impl):
    m = single_clipped()
    for y in range(4, 6):
        for x in range(4, 6):
            if color_at("RGGB", x, y) == 0:
                m[y, x] = 0.9
    for cx, cy in ((2, 2), (3, 2), (4, 2)):
        for y in range(2 * cy, 2 * cy + 2):
            for x in range(2 * cx, 2 * cx + 2):
                m[y, x] = (0.8, 0.2, 0.6)[color_at("RGGB", x, y)]
    out, stats = impl.opposed(m, "RGGB", L09)
    assert stats[SUSPECTED] == 1 and stats[RECONSTRUCTED] == 0 and stats[FALLBACK] == 1
    assert out[6, 6] == m[6, 6]


def test_opposed_fully_unsupported_cells_are_reported(impl):
    _, stats = impl.opposed(blown_cell(), "RGGB", L09)
    assert stats[SUSPECTED] == 4 and stats[RECONSTRUCTED] == 0
    assert stats[FALLBACK] == 4 and stats[UNSUPPORTED] == 4


def test_opposed_no_suspected_sites_is_bit_identical(impl):
    m = np.array([[0.1, 0.2, 0.3, 0.4, 0.5], [0.6, 0.7, 0.8, 0.1, 0.2], [0.3, 0.4, 0.5, 0.6, 0.7]], np.float32)
    out, stats = impl.opposed(m, "BGGR", L09)
    assert out.view(np.uint32).tolist() == m.view(np.uint32).tolist()
    assert stats.tolist() == [0] * 9


def test_opposed_invalid_levels_and_samples_are_rejected(impl):
    with pytest.raises(Rejected):
        impl.opposed(double_clipped("RGGB"), "RGGB", (float("nan"), 0.9, 0.9))
    bad = double_clipped("RGGB")
    bad[2, 3] = np.nan
    with pytest.raises(Rejected):
        impl.opposed(bad, "RGGB", L09)
    for ceiling in ((float("nan"), 0.65, 0.7), (0.0, 0.65, 0.7), (0.6, 0.65, float("nan"))):
        with pytest.raises(Rejected):
            impl.opposed(blown_cell(), "RGGB", L09, ceiling)


def test_opposed_is_deterministic(impl):
    a = impl.opposed(double_clipped("GRBG"), "GRBG", L09)
    b = impl.opposed(double_clipped("GRBG"), "GRBG", L09)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_opposed_without_a_ceiling_reproduces_the_legacy_output(impl):
    m = blown_cell()
    out, stats = impl.opposed(m, "RGGB", L09)
    assert np.array_equal(out, m)
    assert stats[NEUTRALISED] == 0 and stats[FALLBACK] == 4


def test_opposed_fallback_sites_above_the_ceiling_land_exactly_on_it(impl):
    out, stats = impl.opposed(blown_cell(), "RGGB", L09, (0.6, 0.65, 0.7))
    assert stats[FALLBACK] == 4 and stats[NEUTRALISED] == 4 and stats[CHANGED] == 0
    assert out[0, 0] == np.float32(0.6) and out[0, 1] == np.float32(0.65)
    assert out[1, 0] == np.float32(0.65) and out[1, 1] == np.float32(0.7)


def test_opposed_suspected_sites_at_or_below_the_ceiling_stay_untouched(impl):
    m = blown_cell()
    out, stats = impl.opposed(m, "RGGB", L09, (1.0, 1.0, 1.0))
    assert np.array_equal(out, m) and stats[NEUTRALISED] == 0


def test_opposed_raised_sites_are_not_lowered_to_the_ceiling(impl):
    out, stats = impl.opposed(double_clipped("RGGB"), "RGGB", L09, (0.85, 0.85, 0.85))
    assert stats[CHANGED] == 3 and stats[NEUTRALISED] == 0
    assert out[6, 6] > 0.85 and out[6, 7] > 0.85 and out[7, 6] > 0.85


def test_opposed_unsuspected_sites_above_the_ceiling_are_never_touched(impl):
    m = single_clipped()
    m[13, 12] = 0.6
    out, stats = impl.opposed(m, "RGGB", L09, (0.5, 0.5, 0.5))
    assert out[13, 12] == m[13, 12] and stats[NEUTRALISED] == 0


def test_opposed_reconstructed_but_not_applied_sites_are_neutralised(impl):
    m = single_clipped()
    m[6, 6] = 4.0
    out, stats = impl.opposed(m, "RGGB", (0.9, 1.0, 1.0), (0.95, 1.0, 1.0))
    assert stats[RECONSTRUCTED] == 1 and stats[CHANGED] == 0 and stats[NEUTRALISED] == 1
    assert out[6, 6] == np.float32(0.95)


def test_opposed_neutral_ceiling_never_feeds_estimation(impl):
    _, low = impl.opposed(blown_cell(), "RGGB", L09, (0.6, 0.65, 0.7))
    _, high = impl.opposed(blown_cell(), "RGGB", L09, (1.0, 1.0, 1.0))
    assert low[SUSPECTED] == high[SUSPECTED] and low[RECONSTRUCTED] == high[RECONSTRUCTED]
    assert low[FALLBACK] == high[FALLBACK]
    assert low[NEUTRALISED] == 4 and high[NEUTRALISED] == 0


def test_opposed_neutralisation_on_odd_dimensions(impl):
    m = np.full((7, 11), 0.2, dtype=np.float32)
    m[:4, :4] = 1.0
    a = impl.opposed(m, "RGGB", L09, (0.5, 0.5, 0.5))
    b = impl.opposed(m, "RGGB", L09, (0.5, 0.5, 0.5))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[1][NEUTRALISED] == 16


def test_opposed_neutralised_sites_aggregate_over_many_rows(impl):
    m = np.full((60, 64), 0.2, dtype=np.float32)
    blown = 0
    for cy in range(0, 30, 3):
        for cx in range(0, 32, 3):
            m[2 * cy:2 * cy + 2, 2 * cx:2 * cx + 2] = 1.0
            blown += 1
    _, stats = impl.opposed(m, "RGGB", L09, (0.8, 0.8, 0.8))
    assert stats[SUSPECTED] == 4 * blown and stats[NEUTRALISED] == 4 * blown


# ---------------------------------------------------------------- colour chain sweep (GPU vs oracle)
HSL_CENTERS = [0.0, 30 / 360, 60 / 360, 120 / 360, 180 / 360, 240 / 360, 270 / 360, 300 / 360]


def colour_fixture():
    """The 13x7 linear Rec.2020 fixture of color_tests.rs:108-139: edge values, signed and HDR
    pixels, the HSL band centres and halfway hues (saturated and over-range), both sides of red."""
    px = [[0.0] * 3, [0.5] * 3, [0.5001, 0.5, 0.5], [1e-8, 0.0, 0.0], [1e-6, 2e-6, 0.0], [-0.1, 0.0, 0.3],
          [-2.0, -1.0, -0.5], [4.0, 0.5, 0.1], [16.0, 8.0, -2.0], [-0.678, 0.2627, 0.0], [0.001, -0.0004, 0.0]]
    hues = []
    for i, c in enumerate(HSL_CENTERS):
        nxt = HSL_CENTERS[i + 1] if i + 1 < len(HSL_CENTERS) else 1.0
        hues += [c, (c + nxt) * 0.5]
    hues += [0.0001, 0.9999]
    for hue in hues:
        rgb = [min(max(abs((hue * 6.0 + ph) % 6.0 - 3.0) - 1.0, 0.0), 1.0) for ph in (0.0, 4.0, 2.0)]
        px.append([v * 0.75 for v in rgb])
        px.append([v * 4.0 - 0.25 for v in rgb])
    return np.array([px[i % len(px)] for i in range(13 * 7)], dtype=np.float32).reshape(7, 39)


def colour_recipes():
    """color_tests.rs:59-106: every HSL band and control at -1 and +1, every grading range and channel
    at -1 and +1, all bands at once, plus Light and saturation cases."""
    rec = [{}]
    for band in range(8):
        for control in range(3):
            for v in (-1.0, 1.0):
                h = np.zeros((8, 3), np.float32)
                h[band, control] = v
                rec.append({"hsl": h})
    for rng in range(3):
        for ch in range(3):
            for v in (-1.0, 1.0):
                g = np.zeros((3, 3), np.float32)
                g[rng, ch] = v
                rec.append({"grading": g})
    for v in (-1.0, 1.0):
        rec.append({"hsl": np.full((8, 3), v, np.float32)})
    rec.append({"light": (0.6, -0.4, 0.5, -0.3, 0.2), "exposure_ev": 0.7, "saturation": 1.3, "vibrance": 0.4})
    rec.append({"light": (-1.0, 1.0, -1.0, 1.0, -1.0), "exposure_ev": -1.0, "saturation": 0.2})
    return rec


@pytest.mark.gpu
@pytest.mark.parametrize("fmt,policy", [("srgb8", "clip"), ("srgb8", "chroma_compress"), ("extended_f32", "clip")])
def test_colour_fixture_recipe_sweep_matches_the_oracle(stages, oracle, fmt, policy):
    from rohditor_gb300 import ColorContract, OutputSpec, light_tone_lut, standard_base_lut

    rgb = colour_fixture()
    base = standard_base_lut()
    for k, r in enumerate(colour_recipes()):
        c = ColorContract(exposure_ev=r.get("exposure_ev", 0.0), base_lut=base,
                          light_tone_lut=light_tone_lut(*r.get("light", (0.0,) * 5)),
                          saturation=r.get("saturation", 1.0), vibrance=r.get("vibrance", 0.0),
                          hsl=r.get("hsl"), grading=r.get("grading"))
        spec = OutputSpec(format=fmt, policy=policy, headroom=8.0)
        ours, _, gamut = stages.output(rgb, c, spec)
        x = oracle.adjust(rgb, c.exposure_ev, c.base_lut, None, c.saturation, c.vibrance, c.hsl, c.grading,
                          light_lut=c.light_tone_lut, extended=fmt.startswith("extended"))
        desc = oracle.output_desc(fmt, "srgb", policy, "none", "normal", None, 8.0)
        oracle.set_exact_math(True)
        try:
            ref, ref_gamut = oracle.render_output(x, desc)
        finally:
            oracle.set_exact_math(False)
        assert ours.view(np.uint8).tolist() == ref.view(np.uint8).tolist(), f"recipe {k}"
        assert np.array_equal(gamut, ref_gamut), f"recipe {k}"
