"""The CPU oracle against the reference's own known-answer tests.

Pins (read from the reference's test sources into tests/golden/reference_pins.json
by tests/golden/make_golden.py):
  * AMaZE FNV-1a output hashes, 4 CFA layouts x {identity, balanced}
    (crates/demosaic/tests/amaze_golden.rs:52-87);
  * AMaZE per-stage probes, bit for bit (crates/demosaic/src/amaze/mod.rs:336-427);
  * exact 2x2 area reduction (crates/core/src/resample.rs:381-398);
  * compact raster-order region labels (crates/highlight/src/regions.rs:315-336).
Plus restated behavioural tests: normalization 1.3 / 0.5 at all crop-shifted
phases (crates/core/src/pipeline/sensor.rs:767-803), MHC kernel impulses
(malvar_he_cutler.rs:124-148), constant reconstruction (demosaic.rs:17-64),
Clip >= vs > semantics (highlight/tests/clip.rs), histogram luma rounding
(analysis/histogram.rs:185-195) and the radial multiplier table's guard
decisions, pinned freeze boundaries and formula-bound coordinate parity
(crates/optics/src/radial/tests.rs: radial_lut_parity,
radial_lut_freeze_ambiguity_guard, radial_lut_determinism).
"""

import json
import os

import numpy as np
import pytest

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
PATTERNS = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}


@pytest.mark.parametrize("name", sorted(PINS["amaze_hashes"]))
def test_amaze_golden_hashes(oracle, name):
    layout, label = name.split()
    mosaic = oracle.amaze_golden_fixture()
    balance = (1.0, 1.0, 1.0) if label == "identity" else (2.1, 1.0, 2.6)
    out = oracle.demosaic(mosaic, PATTERNS[layout], balance, 3)
    assert f"{oracle.fnv1a(out):016x}" == PINS["amaze_hashes"][name]


def test_amaze_stage_probes_bit_exact(oracle):
    mosaic = oracle.amaze_probe_fixture()
    stage = PINS["amaze_stage"]
    planes = {}
    for probe in stage["probes"]:
        name = probe["plane"]
        if name not in planes:
            planes[name] = oracle.amaze_probe_plane(mosaic, 0, 1.0, name)
        plane = planes[name]
        col = probe["col"] if plane.shape[1] == 256 else probe["col"] // 2
        got = np.float32(plane[probe["row"], col])
        assert got.tobytes() == np.float32(float(probe["value"])).tobytes(), probe
    nyq = oracle.amaze_probe_plane(mosaic, 0, 1.0, "nyquist").sum()
    nyq2 = oracle.amaze_probe_plane(mosaic, 0, 1.0, "nyquist2").sum()
    assert (int(nyq), int(nyq2)) == (stage["nyquist_sites"], stage["voted_sites"])


def test_area_reduction_exact_2x2(oracle):
    data = []
    for y in range(4):
        for x in range(4):
            v = float(y * 4 + x)
            data += [v, v + 100.0, -v]
    img = np.array(data, dtype=np.float32).reshape(4, 12)
    out = oracle.area_reduce(img, (2, 2))
    for pin in PINS["area_2x2"]:
        got = out[pin["y"], 3 * pin["x"]: 3 * pin["x"] + 3]
        assert list(got) == pin["rgb"]


def test_area_reduction_preserves_constant(oracle):
    img = np.tile(np.array([0.25, -0.5, 1.5], dtype=np.float32), (5, 7))
    out = oracle.area_reduce(img, (3, 2))
    expected = np.tile(np.array([0.25, -0.5, 1.5], dtype=np.float32), (2, 3))
    assert np.max(np.abs(out - expected)) <= 2e-7


def test_connected_component_labels(oracle):
    for case in PINS["ccl"]:
        grid = np.array([[1 if ch == "#" else 0 for ch in row] for row in case["grid"]], dtype=np.uint32)
        labels, count = oracle.label_components(grid)
        assert count == case["count"]
        assert labels.reshape(-1).tolist() == case["labels"]


def test_connected_components_u_shape_and_diagonal(oracle):
    grid = np.array([[1, 0, 0, 0, 1], [1, 0, 0, 0, 1], [1, 1, 1, 1, 1], [0, 0, 0, 0, 0], [0, 0, 1, 0, 0]])
    labels, count = oracle.label_components(grid)
    assert count == 2 and labels[0, 0] == 1 and labels[0, 4] == 1 and labels[4, 2] == 2
    diag = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]])
    labels, count = oracle.label_components(diag)
    assert count == 1 and int((labels == 1).sum()) == 3


def _normalize_fixture(pattern: str):
    # sensor.rs:701-765: 6x5 sensor, row stride 8, crop (1,1,4,4), black 2x2 {0,10,20,30},
    # white per pattern {100,110,120,130}; samples 50/60/70/80 by phase, 160 at the crop origin.
    samples = np.full((5, 8), 65535, dtype=np.uint16)
    for y in range(5):
        for x in range(6):
            samples[y, x] = [50, 60, 70, 80][(y & 1) * 2 + (x & 1)]
    samples[1, 1] = 160
    return samples


@pytest.mark.parametrize("pattern", ["RGGB", "BGGR", "GRBG", "GBRG"])
def test_normalize_known_values(oracle, pattern):
    samples = _normalize_fixture(pattern)
    desc = oracle.sensor_desc(6, 5, 8, (1, 1, 4, 4), PATTERNS[pattern], [0, 10, 20, 30], (2, 2),
                              [100, 110, 120, 130])
    out, crop_pattern = oracle.normalize(samples, desc)
    shifted = {"RGGB": "BGGR", "BGGR": "RGGB", "GRBG": "GBRG", "GBRG": "GRBG"}[pattern]
    assert crop_pattern == PATTERNS[shifted]
    assert out[0, 0] == np.float32(1.3)
    assert np.all(out.reshape(-1)[1:] == np.float32(0.5))


def test_mhc_kernel_impulses(oracle):
    # malvar_he_cutler.rs:124-148 through the full demosaic at the centre of a 5x5 impulse image:
    # RGGB has red at (2,2), so green uses GREEN_AT_RED and blue RED_AT_BLUE.
    cases = [((2, 2), 1, 0.5), ((2, 0), 1, -0.125), ((2, 1), 1, 0.25), ((2, 2), 2, 0.75), ((1, 1), 2, 0.25),
             ((2, 0), 2, -0.1875)]
    for (ix, iy), channel, expected in cases:
        img = np.zeros((5, 5), dtype=np.float32)
        img[iy, ix] = 1.0
        out = oracle.demosaic(img, 0, (1, 1, 1), 1)
        assert out[2, 3 * 2 + channel] == np.float32(expected)
    # A green site at the centre (GRBG): colour at green, same-row kernel and its transpose.
    for (ix, iy), channel, expected in [((2, 2), 0, 0.625), ((1, 2), 0, 0.5), ((2, 1), 2, 0.5)]:
        img = np.zeros((5, 5), dtype=np.float32)
        img[iy, ix] = 1.0
        out = oracle.demosaic(img, 2, (1, 1, 1), 1)
        assert out[2, 3 * 2 + channel] == np.float32(expected)


@pytest.mark.parametrize("algorithm,size,tol", [(1, (9, 8), 1e-6), (2, (40, 40), 1e-5), (3, (40, 40), 1e-5)])
@pytest.mark.parametrize("pattern", [0, 1, 2, 3])
def test_demosaic_reconstructs_constants(oracle, algorithm, size, tol, pattern):
    w, h = size
    rgb = (0.2, 0.4, 0.8)
    mosaic = np.zeros((h, w), dtype=np.float32)
    table = {0: [0, 1, 1, 2], 1: [2, 1, 1, 0], 2: [1, 0, 2, 1], 3: [1, 2, 0, 1]}[pattern]
    for y in range(h):
        for x in range(w):
            mosaic[y, x] = rgb[table[(y & 1) * 2 + (x & 1)]]
    out = oracle.demosaic(mosaic, pattern, (1, 1, 1), algorithm).reshape(h, w, 3)
    assert np.max(np.abs(out - np.array(rgb, dtype=np.float32))) <= tol


def test_clip_semantics(oracle):
    m = np.array([[1.0, 0.5], [0.99, 1.2]], dtype=np.float32)
    out, stats = oracle.clip(m, 0, (1.0, 1.0, 1.0))
    # (0,0) R == limit: affected, unchanged; (1,1) B > limit: affected, changed, over white.
    assert out[0, 0] == 1.0 and out[1, 1] == 1.0
    assert stats.tolist() == [2, 1, 1, 1, 0, 1]


def test_histogram_luma_rounding(oracle):
    def luma(r, g, b):
        img = np.array([[r, g, b]], dtype=np.uint8)
        hist, _ = oracle.histogram(img)
        return int(np.nonzero(hist[768:])[0][0])

    for v in (0, 17, 128, 255):
        assert luma(v, v, v) == v
    assert luma(255, 0, 0) == 54 and luma(0, 255, 0) == 182 and luma(0, 0, 255) == 18
    assert luma(0, 3, 4) == 2 and luma(0, 3, 5) == 3


def test_standard_base_lut_endpoints(oracle):
    lut = oracle.standard_base_lut()
    assert lut[0] == 0.0 and lut[4095] == 1.0
    # Middle gray maps to itself within 2e-6 (rendering.rs:240-248).
    coordinate = np.float32(0.18) / np.float32(1.18)
    pos = coordinate * np.float32(4095.0)
    lo = int(np.floor(pos))
    val = lut[lo] + (lut[lo + 1] - lut[lo]) * (pos - np.float32(lo))
    assert abs(val - 0.18) < 2e-6


def test_opposed_leaves_unclipped_mosaics_alone(oracle):
    rng = np.random.default_rng(3)
    m = rng.uniform(0.05, 0.6, size=(40, 46)).astype(np.float32)
    out, stats, labels, count = oracle.opposed(m, 0, (0.987, 0.987, 0.987))
    assert np.array_equal(out, m) and stats[0] == 0 and count == 0


def test_opposed_raises_clipped_sites_from_opposing_channels(oracle):
    # A smooth warm scene with a blown disc: red clips first; estimates come from G and B.
    h, w = 64, 80
    yy, xx = np.mgrid[0:h, 0:w]
    base = np.where((xx & 1) == (yy & 1), 0.5, 0.35).astype(np.float32)
    red = ((yy & 1) == 0) & ((xx & 1) == 0)
    disc = (yy - 32) ** 2 + (xx - 40) ** 2 < 100
    m = base.copy()
    m[red] = 0.7
    m[red & disc] = 1.2
    out, stats, labels, count = oracle.opposed(m, 0, (0.987,) * 3, ceiling=(0.4935, 0.987, 0.616875))
    assert stats[0] == int((red & disc).sum()) and count >= 1
    assert stats[1] + stats[3] == stats[0]


def test_counted_amaze_build_is_bit_exact_and_counts(oracle):
    """The FLOP-census build of AMaZE (counting floats) reconstructs the same
    bits as the oracle, so its operation counts describe the real algorithm."""
    m = oracle.amaze_golden_fixture()
    for balance in ((1.0, 1.0, 1.0), (2.0, 1.0, 1.6)):
        ref = oracle.demosaic(m, 0, balance, 3)
        out, ops = oracle.amaze_counted(m, 0, balance)
        assert np.array_equal(ref.view(np.uint32), out.view(np.uint32))
        per_px = {k: v / m.size for k, v in ops.items()}
        assert 300 < per_px["add_sub"] < 600 and 100 < per_px["mul"] < 400 and per_px["div"] > 10


# Lens models for the radial multiplier table (distortion model, k, TCA model,
# red, blue) and the rule the build applies to each on a 320x213 frame.
RADIAL_LENSES = {
    "poly5_linear_tca": ((2, (-0.02, 0.005, 0.0), 1, (1.0003, 0, 0), (0.9997, 0, 0)), "accepted"),
    "ptlens": ((3, (0.01, -0.03, 0.02), 0, (1, 0, 0), (1, 0, 0)), "accepted"),
    "linear_tca_only": ((0, (0, 0, 0), 1, (1.0003, 0, 0), (0.9997, 0, 0)), "accepted"),
    # Poly3 truncates rd / k1 to f32 in its step-0 residual: its freeze band is
    # too wide, as radial.rs:44-57 measures for every bundled Poly3 profile.
    "poly3": ((1, (-0.01, 0, 0), 0, (1, 0, 0), (1, 0, 0)), "freeze ambiguity"),
    # Symmetric red / blue TCA flips land in the same knot segment.
    "poly5_poly3_tca": ((2, (-0.02, 0.005, 0.0), 2, (1.0002, 0.0001, -0.0001), (0.9998, -0.0001, 0.0001)),
                        "break collision"),
}


def radial_lens(oracle, name, w=320, h=213):
    (dm, dk, tm, red, blue), _ = RADIAL_LENSES[name]
    return oracle.optics_plan(w, h, dm, dk, tm, red, blue)


@pytest.mark.parametrize("name", sorted(RADIAL_LENSES))
def test_radial_table_guard_decisions(oracle, name):
    guard, step, table, segments = oracle.optics_radial(radial_lens(oracle, name))
    assert guard == RADIAL_LENSES[name][1]
    assert step > 0 and np.all(np.isfinite(table))


@pytest.mark.parametrize("name", ["poly5_linear_tca", "ptlens"])
def test_radial_table_pins_each_freeze_boundary_inside_its_segment(oracle, name):
    d = radial_lens(oracle, name)
    guard, step, table, segments = oracle.optics_radial(d)
    assert guard == "accepted" and len(segments) == 1
    for index, radius in segments:
        assert np.float32(index) * np.float32(step) <= radius <= np.float32(index + 1) * np.float32(step)
    # Inside the freeze radius the kernel returns its input: the multiplier is 1.
    kr = d.tca_red[0] if d.tca_model == 1 else 1.0
    kb = d.tca_blue[0] if d.tca_model == 1 else 1.0
    assert np.array_equal(table[0], np.array([kr, 1.0, kb], dtype=np.float32))


@pytest.mark.parametrize("name", ["poly5_linear_tca", "ptlens", "linear_tca_only"])
def test_radial_table_coordinates_within_the_formula_bound(oracle, name):
    """radial.rs:60-72: B = max(0.15 px, 1.5 * NEWTON_EPS * norm_unscale) between
    the table branch and the Newton path, here checked on every fourth pixel."""
    import ctypes

    d = radial_lens(oracle, name)
    bound = max(0.15, 1.5e-5 * d.norm_unscale)
    newton = np.zeros(6, dtype=np.float32)
    worst = 0.0
    for y in range(0, d.height, 4):
        for x in range(0, d.width, 4):
            lut = oracle.optics_map_lut(d, x, y)
            assert oracle.load().ro_optics_map(ctypes.byref(d), x, y, oracle.ptr(newton)) == 0
            worst = max(worst, float(np.max(np.abs(lut - newton))))
    assert worst <= bound


def test_radial_table_is_deterministic(oracle):
    a = oracle.optics_radial(radial_lens(oracle, "poly5_linear_tca"))
    b = oracle.optics_radial(radial_lens(oracle, "poly5_linear_tca"))
    assert a[0] == b[0] and a[1] == b[1] and a[3] == b[3]
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))


def test_newton_and_table_coordinates_against_the_converged_root(oracle):
    """The 24 MP workload's lens (Poly5 k1 = -0.02, k2 = 0.005, Linear TCA
    1.0003 / 0.9997, crop 1, 35 mm, centred): the lensfun-style Newton path
    (break at |F| < 1e-5) and the radial table both stay within the formula bound
    B = max(0.15 px, 1.5 * 1e-5 * norm_unscale) (radial.rs:60-72) of the root
    solved to convergence in f64, on a 63 x 42 grid of pixels."""
    import ctypes

    w, h = 6048, 4024
    d = oracle.optics_plan(w, h, 2, (-0.02, 0.005, 0.0), 1, (1.0003, 0, 0), (0.9997, 0, 0))
    k1, k2 = -0.02, 0.005
    bound = max(0.15, 1.5e-5 * d.norm_unscale)
    cpx, cpy = d.center_x * d.norm_unscale, d.center_y * d.norm_unscale
    newton = np.zeros(6, dtype=np.float32)
    worst_newton = worst_table = 0.0
    for y in np.linspace(0, h - 1, 42).astype(int):
        for x in np.linspace(0, w - 1, 63).astype(int):
            ix = np.float32((cpx + (x - cpx) / np.float64(d.scale)) * d.norm_scale - d.center_x)
            iy = np.float32((cpy + (y - cpy) / np.float64(d.scale)) * d.norm_scale - d.center_y)
            rd = np.sqrt(np.float64(ix * ix + iy * iy))
            ru = rd
            for _ in range(60):
                ru -= (ru * (1 + k1 * ru * ru + k2 * ru ** 4) - rd) / (1 + 3 * k1 * ru * ru + 5 * k2 * ru ** 4)
            ratio = ru / rd if rd > 0 else 1.0
            gx, gy = np.float64(ix) * ratio, np.float64(iy) * ratio
            exact = []
            for m in (1.0003, 1.0, 0.9997):
                exact += [(gx * m + d.center_x) * d.norm_unscale, (gy * m + d.center_y) * d.norm_unscale]
            exact = np.array(exact)
            assert oracle.load().ro_optics_map(ctypes.byref(d), int(x), int(y), oracle.ptr(newton)) == 0
            table = oracle.optics_map_lut(d, int(x), int(y))
            worst_newton = max(worst_newton, float(np.max(np.abs(newton - exact))))
            worst_table = max(worst_table, float(np.max(np.abs(table - exact))))
    assert worst_newton <= bound and worst_table <= bound, (worst_newton, worst_table, bound)
