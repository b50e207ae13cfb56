"""Parity of the sm_103a kernels (through the C ABI) with the CPU oracle.

Bars (from the path's contract):
  * bit-exact: crop, CFA indexing, the Clip mask and its statistics, every
    demosaic (bilinear, MHC, RCD, AMaZE, incl. the reference's golden hashes),
    the area reduction, and the histogram of the kernel's own 8-bit output;
  * linear f32 within 1e-4 max abs after a stage, 5e-4 after 10 RL iterations;
  * optics within the reference's own GPU gate, 2e-4 + 2e-4 |x|
    (crates/gpu/src/spatial/tests.rs:174);
  * sRGB8 within 1 LSB on at most 0.1% of the samples.
Sizes are small enough for the oracle to finish in seconds; they include odd
sizes, image edges, several AMaZE/RCD tiles and the size gates.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
PATTERNS = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}
ALGOS = {"bilinear": 0, "mhc": 1, "rcd": 2, "amaze": 3}


def textured_mosaic(w, h, seed, clip_frac=0.03):
    """Signed, textured mosaic with flat areas, hard edges and clipped patches."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    v = 0.35 + 0.25 * np.sin(xx * 0.37 + yy * 0.11) * np.cos(yy * 0.29)
    v += 0.1 * rng.standard_normal((h, w)).astype(np.float32)
    v[(xx // 17 + yy // 13) % 7 == 0] = 0.05
    blob = rng.uniform(size=(h, w)) < clip_frac
    v[blob] = 1.3
    v[(xx.astype(int) + 2 * yy.astype(int)) % 97 == 0] = -0.02
    return v.astype(np.float32)


@pytest.mark.parametrize("name", sorted(PINS["amaze_hashes"]))
def test_amaze_golden_hashes_on_gpu(stages, oracle, name):
    layout, label = name.split()
    mosaic = oracle.amaze_golden_fixture()
    balance = (1.0, 1.0, 1.0) if label == "identity" else (2.1, 1.0, 2.6)
    out = stages.demosaic(mosaic, layout, "amaze", balance)
    assert f"{oracle.fnv1a(out):016x}" == PINS["amaze_hashes"][name]


@pytest.mark.parametrize("algorithm", ["bilinear", "mhc", "rcd", "amaze"])
@pytest.mark.parametrize("layout", ["RGGB", "BGGR", "GRBG", "GBRG"])
@pytest.mark.parametrize("size", [(517, 389), (53, 47), (256, 200), (704, 480)])
def test_demosaic_bit_exact(stages, oracle, algorithm, layout, size):
    w, h = size
    mosaic = textured_mosaic(w, h, seed=w * 7 + h)
    for balance in [(1.0, 1.0, 1.0), (2.0, 1.0, 1.6)]:
        ours = stages.demosaic(mosaic, layout, algorithm, balance)
        ref = oracle.demosaic(mosaic, PATTERNS[layout], balance, ALGOS[algorithm])
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), (
            algorithm, layout, size, balance, float(np.max(np.abs(ours - ref))))


@pytest.mark.parametrize("size", [(33, 33), (32, 40), (24, 30), (25, 25), (2, 2), (240, 225)])
def test_demosaic_size_gates_and_edges(stages, oracle, size):
    w, h = size
    mosaic = textured_mosaic(w, h, seed=5)
    for algorithm in ["rcd", "amaze", "mhc"]:
        ours = stages.demosaic(mosaic, "GBRG", algorithm, (1.9, 1.0, 1.4))
        ref = oracle.demosaic(mosaic, 3, (1.9, 1.0, 1.4), ALGOS[algorithm])
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), (algorithm, size)


def raw_mosaic(sw, sh, stride, seed):
    rng = np.random.default_rng(seed)
    raw = rng.integers(0, 4096, size=(sh, stride), dtype=np.uint16)
    raw[rng.uniform(size=raw.shape) < 0.05] = 4095
    raw[rng.uniform(size=raw.shape) < 0.01] = 0
    return raw


@pytest.mark.parametrize("layout", ["RGGB", "GBRG"])
@pytest.mark.parametrize("highlight", ["off", "clip"])
def test_normalize_and_clip_bit_exact(stages, oracle, layout, highlight):
    from rohditor_gb300 import SensorDescription

    sw, sh, stride = 131, 97, 136
    raw = raw_mosaic(sw, sh, stride, seed=11)
    crop = (3, 2, 120, 90)
    black = (200.0, 210.0, 190.0, 205.0)
    white = (4000.0, 4095.0, 3900.0)
    desc = SensorDescription(sw, sh, cfa=layout, crop=crop, black=black, black_repeat=(2, 2), white=white,
                             highlight=highlight, clip_levels=(0.91, 0.987, 0.8), demosaic="amaze")
    ours, stats = stages.highlight(raw, desc)
    odesc = oracle.sensor_desc(sw, sh, stride, crop, PATTERNS[layout], black, (2, 2), white)
    ref, crop_pattern = oracle.normalize(raw, odesc)
    if highlight == "clip":
        ref, ref_stats = oracle.clip(ref, crop_pattern, (0.91, 0.987, 0.8))
        assert stats[:6].tolist() == ref_stats.tolist()
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("algorithm", ["mhc", "bilinear", "rcd", "amaze"])
@pytest.mark.parametrize("crop", [(8, 2, 496, 380), (0, 0, 512, 389), (3, 5, 500, 377), (16, 0, 130, 70)])
def test_raw_tile_staging_bit_exact(device, oracle, algorithm, crop):
    """Every demosaic stages its tiles (AMaZE: its tiles' rows) from the raw
    u16 samples: by a tensor copy when the crop's x and the row pitch lie on
    the 16-byte grid (the first, second and last crops; windows or rows that
    reach past the image edge are always loaded with their mirrored samples),
    by plain loads otherwise (x = 3). Both must give the staged oracle's
    output and the Clip statistics bit for bit."""
    from rohditor_gb300 import GpuSensorProcessor, SensorDescription

    sw, sh, stride = 512, 389, 520
    raw = raw_mosaic(sw, sh, stride, seed=31)
    black = (200.0, 210.0, 190.0, 205.0)
    white = (4000.0, 4095.0, 3900.0)
    levels = (0.91, 0.987, 0.8)
    desc = SensorDescription(sw, sh, cfa="GBRG", crop=crop, black=black, black_repeat=(2, 2), white=white,
                             highlight="clip", clip_levels=levels, demosaic=algorithm,
                             demosaic_balance=(2.0, 1.0, 1.6))
    src = GpuSensorProcessor(device).develop(raw, desc)
    ours = src.download()
    odesc = oracle.sensor_desc(sw, sh, stride, crop, PATTERNS["GBRG"], black, (2, 2), white)
    m, pattern = oracle.normalize(raw, odesc)
    m, stats = oracle.clip(m, pattern, levels)
    ref = oracle.demosaic(m, pattern, (2.0, 1.0, 1.6), ALGOS[algorithm])
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), float(np.max(np.abs(ours - ref)))
    assert list(src.metrics.highlight_stats)[:6] == stats.tolist()
    src.release()


def test_fused_develop_matches_staged_oracle(device, oracle):
    """rd_develop fuses normalize + Clip + balance into the AMaZE tile load."""
    from rohditor_gb300 import GpuSensorProcessor, SensorDescription

    sw, sh, stride = 517, 389, 520
    raw = raw_mosaic(sw, sh, stride, seed=21)
    desc = SensorDescription(sw, sh, cfa="GRBG", crop=(0, 0, sw, sh), black=(256.0,), white=(4095.0,),
                             highlight="clip", clip_levels=(0.6, 0.987, 0.75), demosaic="amaze",
                             demosaic_balance=(2.0, 1.0, 1.6))
    src = GpuSensorProcessor(device).develop(raw, desc)
    ours = src.download()
    odesc = oracle.sensor_desc(sw, sh, stride, (0, 0, sw, sh), 2, [256.0], (1, 1), [4095.0])
    m, pattern = oracle.normalize(raw, odesc)
    m, stats = oracle.clip(m, pattern, (0.6, 0.987, 0.75))
    ref = oracle.demosaic(m, pattern, (2.0, 1.0, 1.6), 3)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))
    assert list(src.metrics.highlight_stats)[:6] == stats.tolist()


@pytest.mark.parametrize("iterations", [8, 10])
def test_capture_sharpening(stages, oracle, iterations):
    from rohditor_gb300 import CaptureContract

    mosaic = np.clip(textured_mosaic(301, 203, seed=31, clip_frac=0.01), 0.0, None)
    rgb = oracle.demosaic(mosaic, 0, (1, 1, 1), 1)
    cap = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=(1.0, 1.0, 1.0),
                          iterations=iterations)
    ours = stages.capture(rgb, cap)
    ref = oracle.capture(rgb, 0.5, 0.7, 0.5, (1.0, 1.0, 1.0), iterations)
    err = float(np.max(np.abs(ours - ref)))
    assert err <= 5e-4, err
    # The kernels keep the reference's tap order, so they agree bit for bit.
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), err


def test_capture_radius_range_and_edges(stages, oracle):
    from rohditor_gb300 import CaptureContract

    rgb = np.abs(textured_mosaic(3 * 37, 29, seed=7)).reshape(29, 111)
    for radius in (0.3, 1.2):
        cap = CaptureContract(amount=1.0, radius=radius, noise_protection=0.0, ceilings=(0.9, 1.0, 0.8),
                              iterations=3)
        ours = stages.capture(rgb, cap)
        ref = oracle.capture(rgb, 1.0, radius, 0.0, (0.9, 1.0, 0.8), 3)
        assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), radius


@pytest.mark.parametrize("radius", [0.3, 0.6, 0.9, 1.2])
@pytest.mark.parametrize("size", [(260, 67), (517, 389), (1032, 300)])
def test_capture_constant_lag_kernel(stages, oracle, radius, size):
    """Images of at least 256 x 64 take the constant-lag RL kernel: mirrored
    top and bottom rows, ragged right strips, widths with (1032) and without
    (260, 517) 16-byte rows for the tensor-copy ring, kernel radii 1..4."""
    from rohditor_gb300 import CaptureContract

    w, h = size
    rgb = np.abs(textured_mosaic(3 * w, h, seed=int(radius * 10) + w)).reshape(h, 3 * w)
    cap = CaptureContract(amount=0.7, radius=radius, noise_protection=0.4, ceilings=(1.0, 0.9, 1.1), iterations=5)
    ours = stages.capture(rgb, cap)
    ref = oracle.capture(rgb, 0.7, radius, 0.4, (1.0, 0.9, 1.1), 5)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("radius", [0.3, 1.2])
@pytest.mark.parametrize("size", [(256, 64), (263, 71), (384, 129), (300, 65)])
def test_capture_constant_lag_kernel_at_its_size_limits(stages, oracle, radius, size):
    """The smallest images the constant-lag kernels take (256 x 64) and ragged
    heights: segments of one 8-row unit, the last segment's alignment to the
    bottom row and the first segment's mirrored top in the same few steps."""
    from rohditor_gb300 import CaptureContract

    w, h = size
    rgb = np.abs(textured_mosaic(3 * w, h, seed=int(radius * 10) + h)).reshape(h, 3 * w)
    cap = CaptureContract(amount=0.8, radius=radius, noise_protection=0.2, ceilings=(1.0, 1.0, 1.0), iterations=4)
    ours = stages.capture(rgb, cap)
    ref = oracle.capture(rgb, 0.8, radius, 0.2, (1.0, 1.0, 1.0), 4)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_capture_launch_shape_tuning_keeps_results(stages, oracle):
    """The first sharpening of an image shape times its iterations under several
    row-segment counts; the second uses the fastest. Both equal the oracle bit
    for bit, so the segmentation is a pure scheduling choice."""
    from rohditor_gb300 import CaptureContract, rl_launch_shape

    w, h = 1204, 1130  # 4-column multiple: estimate rows go through the TMA ring
    rgb = np.abs(textured_mosaic(3 * w, h, seed=41)).reshape(h, 3 * w)
    cap = CaptureContract(amount=0.6, radius=0.9, noise_protection=0.3, ceilings=(1.0, 1.0, 1.0), iterations=8)
    assert rl_launch_shape(w, h, 0.9) is None
    first = stages.capture(rgb, cap)
    shape = rl_launch_shape(w, h, 0.9)
    assert shape is not None and shape.segments >= 1 and shape.default_segments >= 1
    assert shape.best_ms > 0.0 and shape.best_ms <= shape.default_ms
    assert h // shape.segments >= 32 or shape.segments == shape.default_segments
    second = stages.capture(rgb, cap)
    assert rl_launch_shape(w, h, 0.9) == shape
    ref = oracle.capture(rgb, 0.6, 0.9, 0.3, (1.0, 1.0, 1.0), 8)
    assert np.array_equal(first.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(second.view(np.uint32), ref.view(np.uint32))


def test_cross_call_shape_tuning_keeps_results(stages, oracle):
    """The guide / mask kernel's row segments, the colour kernel's grid and
    the optics gather's tile rows are tuned across calls: the first calls of
    an image shape each launch one candidate, timed, until every candidate has
    two timings. Every call's result equals the oracle (or the first call)
    bit for bit, and the shape is then reported."""
    from rohditor_gb300 import CaptureContract, ColorContract, launch_shape, standard_base_lut

    w, h = 1532, 1020
    rgb = np.abs(textured_mosaic(3 * w, h, seed=43)).reshape(h, 3 * w)
    cap = CaptureContract(amount=0.5, radius=0.8, noise_protection=0.4, ceilings=(1.0, 1.0, 1.0), iterations=2)
    ref = oracle.capture(rgb, 0.5, 0.8, 0.4, (1.0, 1.0, 1.0), 2)
    assert launch_shape("rl_mask", w, h, 0.8) is None
    for _ in range(14):
        assert np.array_equal(stages.capture(rgb, cap).view(np.uint32), ref.view(np.uint32))
    shape = launch_shape("rl_mask", w, h, 0.8)
    assert shape is not None and shape.segments >= 1 and shape.best_ms <= shape.default_ms
    color = ColorContract(wb_gains=(1.8, 1.0, 1.5), exposure_ev=0.2, base_lut=standard_base_lut())
    base = np.abs(textured_mosaic(3 * 900, 700, seed=44)).reshape(700, 3 * 900)
    outs = [stages.color(base, color) for _ in range(10)]
    for out, hist, _ in outs[1:]:
        assert np.array_equal(out, outs[0][0]) and np.array_equal(hist, outs[0][1])
    assert launch_shape("color", 900, 700) is not None
    from rohditor_gb300 import OpticsExecution

    ow, oh = 523, 391  # a size no other test remaps
    orgb = smooth_rgb(ow, oh, seed=45)
    ex = OpticsExecution(ow, oh, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                         tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0), vignetting_k=(-0.3, 0.05, -0.01))
    oref = oracle.optics_apply(oracle.optics_desc_from(ex.to_c()), orgb)
    assert launch_shape("optics", ow, oh) is None
    for _ in range(8):
        assert np.array_equal(stages.optics(orgb, ex).view(np.uint32), oref.view(np.uint32))
    assert launch_shape("optics", ow, oh) is not None


def smooth_rgb(w, h, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    r = 0.4 + 0.3 * np.sin(xx / 13.0) * np.cos(yy / 17.0)
    g = 0.5 + 0.2 * np.cos(xx / 7.0 + yy / 11.0)
    b = 0.3 + 0.25 * np.sin((xx + yy) / 19.0)
    rgb = np.stack([r, g, b], axis=-1)
    rgb[(xx.astype(int) // 23 + yy.astype(int) // 19) % 5 == 0] = [0.9, 0.1, 0.05]
    rgb += 0.01 * rng.standard_normal(rgb.shape)
    return rgb.reshape(h, 3 * w).astype(np.float32)


@pytest.mark.parametrize("size", [(320, 213), (161, 97)])
def test_optics(stages, oracle, size):
    from rohditor_gb300 import OpticsExecution

    w, h = size
    rgb = smooth_rgb(w, h, seed=4)
    ex = OpticsExecution(w, h, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                         tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0), vignetting_k=(-0.3, 0.05, -0.01))
    ours = stages.optics(rgb, ex)
    ref = oracle.optics_apply(oracle.optics_desc_from(ex.to_c()), rgb)
    tol = 2e-4 + 2e-4 * np.abs(ref)
    assert np.all(np.abs(ours - ref) <= tol), float(np.max(np.abs(ours - ref)))
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


RADIAL_CASES = {
    "poly5_linear_tca": dict(distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                             tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0)),
    "ptlens": dict(distortion="ptlens", distortion_k=(0.01, -0.03, 0.02)),
    "linear_tca_only": dict(tca="linear", tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0)),
    "poly3": dict(distortion="poly3", distortion_k=(-0.01, 0, 0)),
    "poly5_poly3_tca": dict(distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="poly3",
                            tca_red=(1.0002, 0.0001, -0.0001), tca_blue=(0.9998, -0.0001, 0.0001)),
    # Blue sampled 5% nearer the centre: away from the centre a tile's three
    # channel footprints no longer fit the shared-memory box and the gather
    # reads global memory, near the centre they do.
    "strong_linear_tca": dict(distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                              tca_red=(1.0, 0, 0), tca_blue=(0.95, 0, 0)),
}


@pytest.mark.parametrize("vignetting", [False, True])
@pytest.mark.parametrize("name", sorted(RADIAL_CASES))
@pytest.mark.parametrize("size", [(97, 61), (517, 389), (1536, 1024)])
def test_optics_radial_table_and_newton_branches(stages, oracle, name, size, vignetting):
    """The remap takes the radial multiplier table when its build accepts it and
    the Newton path otherwise (correction.rs:110-181), bit for bit with the
    oracle either way. Poly3 is refused (freeze ambiguity) at every size, the
    symmetric Poly3 TCA pair collides except at 97x61, where it is accepted with
    three pinned freeze boundaries."""
    from rohditor_gb300 import OpticsExecution

    w, h = size
    kw = dict(RADIAL_CASES[name])
    if vignetting:
        kw["vignetting_k"] = (-0.3, 0.05, -0.01)
    ex = OpticsExecution(w, h, **kw)
    desc = oracle.optics_desc_from(ex.to_c())
    guard, _, _, pins = oracle.optics_radial(desc)
    refused = name == "poly3" or (name == "poly5_poly3_tca" and size != (97, 61))
    assert (guard != "accepted") == refused
    rgb = smooth_rgb(w, h, seed=17)
    ours = stages.optics(rgb, ex)
    ref = oracle.optics_apply(desc, rgb)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_optics_hypot_matches_glibc(stages):
    """The table branch looks up f32::hypot of the input coordinates; the device
    hypot equals glibc's double-evaluated one on ~110 M sampled pairs."""
    assert stages.check_math(4) == 0


def test_vignetting_only(stages, oracle):
    from rohditor_gb300 import OpticsExecution

    rgb = smooth_rgb(203, 131, seed=9)
    ex = OpticsExecution(203, 131, vignetting_k=(-0.35, 0.06, -0.015))
    ours = stages.optics(rgb, ex)
    ref = oracle.optics_apply(oracle.optics_desc_from(ex.to_c()), rgb)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("src,dst", [((611, 409), (256, 171)), ((97, 53), (41, 23)), ((40, 30), (40, 30)),
                                     ((64, 48), (1, 1))])
def test_area_reduce_bit_exact(stages, oracle, src, dst):
    rgb = smooth_rgb(src[0], src[1], seed=2)
    ours = stages.area_reduce(rgb, dst)
    ref = oracle.area_reduce(rgb, dst)
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def colour_contract(**kw):
    from rohditor_gb300 import ColorContract, standard_base_lut
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hsl_bands, sixteen_knot_curve

    base = dict(wb_gains=(2.0, 1.0, 1.6), camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.5,
                base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(), hsl=hsl_bands())
    base.update(kw)
    return ColorContract(**base)


def oracle_colour(oracle, rgb, c):
    x = oracle.white_balance(rgb, c.wb_gains)
    x = oracle.camera_matrix(x, c.camera_to_rec2020)
    x = oracle.adjust(x, c.exposure_ev, c.base_lut, c.tone_lut, c.saturation, c.vibrance, c.hsl, c.grading,
                      light_lut=c.light_tone_lut)
    return oracle.display_srgb8(x)


@pytest.mark.parametrize("variant", ["config", "grading_saturation", "neutral", "light", "light_extreme"])
def test_colour_output_and_histogram(stages, oracle, variant):
    rng = np.random.default_rng(17)
    u = rng.uniform(-0.05, 0.8, size=(173, 3 * 251))
    rgb = (np.sign(u) * np.abs(u) ** 1.5).astype(np.float32)
    rgb[:5] = 2.5  # over-range rows clip to white
    if variant == "config":
        c = colour_contract()
    elif variant == "grading_saturation":
        c = colour_contract(saturation=1.2, vibrance=0.3,
                            grading=np.array([[0.2, -0.1, 0.05], [0.0, 0.1, -0.2], [-0.1, 0.0, 0.3]], np.float32))
    elif variant == "light":
        from rohditor_gb300 import light_tone_lut

        # Light sliders (contrast, highlights, shadows, whites, blacks) between
        # the base rendering and the tone curve.
        c = colour_contract(light_tone_lut=light_tone_lut(0.4, -0.5, 0.35, -0.2, 0.15))
        assert np.array_equal(c.light_tone_lut, oracle.light_tone_lut(0.4, -0.5, 0.35, -0.2, 0.15))
    elif variant == "light_extreme":
        from rohditor_gb300 import light_tone_lut

        c = colour_contract(tone_lut=None, light_tone_lut=light_tone_lut(1.0, 1.0, -1.0, -1.0, 1.0))
    else:
        c = colour_contract(exposure_ev=0.0, base_lut=None, tone_lut=None, hsl=None)
    ours, hist, clipped = stages.color(rgb, c)
    ref = oracle_colour(oracle, rgb, c)
    # The 8-bit code of the correctly rounded transfer equals glibc powf's on
    # every f32 of the transfer's domain, so the output is bit-exact.
    assert np.array_equal(ours, ref)
    # The histogram of the kernel's own 8-bit output is exact.
    ref_hist, ref_clipped = oracle.histogram(ours)
    assert np.array_equal(hist, ref_hist) and np.array_equal(clipped, ref_clipped)


def test_processor_pipeline_end_to_end(device, oracle):
    """develop -> spatial -> render through the processor API, stage by stage against the oracle."""
    from rohditor_gb300 import (CaptureContract, GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor,
                                OpticsExecution, SensorDescription, clip_levels)
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, preview_dimensions

    sw, sh = 700, 467
    raw = raw_mosaic(sw, sh, sw, seed=41)
    wb = (2.0, 1.0, 1.6)
    levels = clip_levels(1.0, wb)
    desc = SensorDescription(sw, sh, cfa="RGGB", black=(256.0,), white=(4095.0,), highlight="clip",
                             clip_levels=levels, demosaic="amaze", demosaic_balance=wb)
    cap = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=levels, iterations=10)
    src = GpuSensorProcessor(device).develop(raw, desc, cap)
    odesc = oracle.sensor_desc(sw, sh, sw, (0, 0, sw, sh), 0, [256.0], (1, 1), [4095.0])
    m, pattern = oracle.normalize(raw, odesc)
    m, _ = oracle.clip(m, pattern, levels)
    ref = oracle.demosaic(m, pattern, wb, 3)
    ref = oracle.capture(ref, 0.5, 0.7, 0.5, levels, 10)
    got = src.download()
    assert float(np.max(np.abs(got - ref))) <= 5e-4
    ex = OpticsExecution(sw, sh, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                         tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0), vignetting_k=(-0.3, 0.05, -0.01))
    target = preview_dimensions(sw, sh, 256)
    base = GpuSpatialProcessor(device).reduce_preview(src, ex, target, wb, CAMERA_TO_REC2020)
    ref_o = oracle.optics_apply(oracle.optics_desc_from(ex.to_c()), ref)
    ref_r = oracle.area_reduce(ref_o, target)
    ref_b = oracle.camera_matrix(oracle.white_balance(ref_r, wb), CAMERA_TO_REC2020)
    got_b = base.download()
    assert float(np.max(np.abs(got_b - ref_b))) <= 1e-4 + 1e-4 * float(np.max(np.abs(ref_b)))
    c = colour_contract()
    out, hist = GpuPreviewProcessor(device).render(base, c)
    x = oracle.adjust(got_b, c.exposure_ev, c.base_lut, c.tone_lut, c.saturation, c.vibrance, c.hsl, c.grading)
    ref8 = oracle.display_srgb8(x)
    diff = np.abs(out.astype(int) - ref8.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() <= 1e-3
    ref_hist, _ = oracle.histogram(out)
    assert np.array_equal(np.concatenate([hist.red, hist.green, hist.blue, hist.luminance]), ref_hist)


def test_cancellation_before_start(device):
    from rohditor_gb300 import GpuPreviewError, GpuSensorProcessor, SensorDescription

    raw = raw_mosaic(64, 48, 64, seed=1)
    cancel = np.ones(1, dtype=np.uint32)
    with pytest.raises(GpuPreviewError) as err:
        GpuSensorProcessor(device).develop(raw, SensorDescription(64, 48, black=(0.0,), white=(4095.0,)),
                                           cancel=cancel)
    assert err.value.variant == "Cancelled" and not err.value.is_routing()


def test_develop_rejects_invalid_geometry_and_keeps_the_context(device, oracle):
    """Inputs the reference refuses before any work (NormalizationContract
    validation, sensor.rs): a sensor or crop below 2x2, a crop outside the
    sensor, a row stride shorter than the sensor width. Each call fails with
    its status and the context then develops a valid mosaic bit-exact."""
    from rohditor_gb300 import GpuPreviewError, GpuSensorProcessor, SensorDescription

    proc = GpuSensorProcessor(device)
    raw = raw_mosaic(64, 48, 64, seed=2)
    cases = [
        (raw[:1, :1], SensorDescription(1, 1, black=(0.0,), white=(4095.0,)), "InvalidInput"),
        (raw, SensorDescription(64, 48, crop=(0, 0, 1, 48), black=(0.0,), white=(4095.0,)), "InvalidInput"),
        (raw, SensorDescription(64, 48, crop=(40, 0, 32, 48), black=(0.0,), white=(4095.0,)), "InvalidInput"),
        (raw[:, :60], SensorDescription(64, 48, black=(0.0,), white=(4095.0,)), "InvalidDimensions"),
    ]
    for mosaic, desc, variant in cases:
        with pytest.raises(GpuPreviewError) as err:
            proc.develop(mosaic, desc)
        assert err.value.variant == variant, (desc, str(err.value))
        assert not err.value.is_routing()
    desc = SensorDescription(64, 48, cfa="GRBG", black=(256.0,), white=(4095.0,), demosaic="mhc")
    got = proc.develop(raw, desc).download()
    odesc = oracle.sensor_desc(64, 48, 64, (0, 0, 64, 48), PATTERNS["GRBG"], [256.0], (1, 1), [4095.0])
    m, pattern = oracle.normalize(raw, odesc)
    ref = oracle.demosaic(m, pattern, (1.0, 1.0, 1.0), ALGOS["mhc"])
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_budget_is_a_routing_answer(device):
    from rohditor_gb300 import GpuPreviewError, GpuSensorProcessor, SensorDescription

    raw = raw_mosaic(640, 480, 640, seed=1)
    device.set_budget(1 << 20)
    try:
        with pytest.raises(GpuPreviewError) as err:
            GpuSensorProcessor(device).develop(raw, SensorDescription(640, 480, black=(0.0,), white=(4095.0,)))
        assert err.value.variant == "OverBudget" and err.value.is_routing()
    finally:
        device.set_budget(0)


def test_kernel_launches_are_counted(device, stages):
    before = device.kernel_launches
    stages.demosaic(textured_mosaic(64, 64, 1), "RGGB", "mhc")
    assert device.kernel_launches > before


def opposed_scene(w, h, seed, layout="RGGB"):
    """Bayer samples of a smooth warm scene with blown discs of varying size, some at the borders."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    rgb = np.stack([0.55 + 0.1 * np.sin(xx / 9.0), 0.45 + 0.1 * np.cos(yy / 7.0),
                    0.30 + 0.05 * np.sin((xx + yy) / 11.0)], axis=-1)
    for _ in range(12):
        cx, cy, r = rng.uniform(0, w), rng.uniform(0, h), rng.uniform(2, 14)
        amp = rng.uniform(1.0, 2.5)
        d2 = ((xx - cx) ** 2 + (yy - cy) ** 2) / (r * r)
        tint = rng.uniform(0.6, 1.0, size=3)
        rgb += (amp * np.exp(-d2))[..., None] * tint
    rgb += 0.004 * rng.standard_normal(rgb.shape)
    table = {"RGGB": [0, 1, 1, 2], "BGGR": [2, 1, 1, 0], "GRBG": [1, 0, 2, 1], "GBRG": [1, 2, 0, 1]}[layout]
    ch = np.array(table)[((yy.astype(int) & 1) << 1) | (xx.astype(int) & 1)]
    return np.take_along_axis(rgb, ch[..., None], axis=-1)[..., 0].astype(np.float32)


@pytest.mark.parametrize("layout", ["RGGB", "GBRG"])
@pytest.mark.parametrize("size", [(120, 94), (333, 257), (41, 37)])
def test_opposed_matches_oracle(stages, oracle, layout, size):
    from rohditor_gb300 import opposed_levels

    w, h = size
    mosaic = opposed_scene(w, h, seed=w + h, layout=layout)
    det, ceiling = opposed_levels(1.0, (2.0, 1.0, 1.6))
    ours, stats, labels, count = stages.opposed(mosaic, layout, det, ceiling)
    ref, ref_stats, ref_labels, ref_count = oracle.opposed(mosaic, PATTERNS[layout], det, ceiling)
    # Region labelling (compact, raster order) and the clipped mask are exact.
    assert count == ref_count
    assert np.array_equal(labels, ref_labels)
    assert stats.tolist() == ref_stats.tolist()
    assert float(np.max(np.abs(ours - ref))) <= 1e-4


def test_opposed_without_clipping_is_identity(stages, oracle):
    mosaic = np.full((50, 64), 0.4, dtype=np.float32)
    ours, stats, labels, count = stages.opposed(mosaic, "RGGB", (0.987,) * 3, None)
    assert np.array_equal(ours, mosaic) and stats[0] == 0 and count == 0 and not labels.any()


def test_develop_with_opposed(device, oracle):
    from rohditor_gb300 import GpuSensorProcessor, SensorDescription, opposed_levels

    w, h = 301, 203
    mosaic = opposed_scene(w, h, seed=3)
    raw = np.clip(np.rint(256 + mosaic * (4095 - 256)), 0, 4095).astype(np.uint16)
    det, ceiling = opposed_levels(1.0, (2.0, 1.0, 1.6))
    desc = SensorDescription(w, h, cfa="RGGB", black=(256.0,), white=(4095.0,), highlight="opposed",
                             detection_levels=det, neutral_ceiling=ceiling, demosaic="amaze",
                             demosaic_balance=(2.0, 1.0, 1.6))
    src = GpuSensorProcessor(device).develop(raw, desc)
    odesc = oracle.sensor_desc(w, h, w, (0, 0, w, h), 0, [256.0], (1, 1), [4095.0])
    m, pattern = oracle.normalize(raw, odesc)
    m, stats, _, _ = oracle.opposed(m, pattern, det, ceiling)
    ref = oracle.demosaic(m, pattern, (2.0, 1.0, 1.6), 3)
    got = src.download()
    assert list(src.metrics.highlight_stats) == stats.tolist()
    assert float(np.max(np.abs(got - ref))) <= 1e-4


def test_full_24mp_workload_against_the_oracle(device, stages, oracle):
    """The bench's 6048x4024 workload end to end (Opposed + AMaZE + RL K=10, then
    table-branch optics with vignetting, area reduction to 2560x1703, WB +
    matrix, adjustments, sRGB8 + histogram) against the oracle at full size,
    stage by stage, each stage fed the GPU's own output of the stage before:
    Opposed statistics exact and samples within 1e-4 (the libm cube root /
    log2 and the f64 summation order of the region means leave last-bit
    differences); AMaZE + 10 RL iterations bit-exact; the spatial stage
    bit-exact; sRGB8 within one code on at most 0.1% of samples; histogram
    exact. Chained through the whole develop (the oracle fed only its own
    outputs) the last-bit Opposed differences move some of AMaZE's
    per-pixel decisions; that spread is bounded by the reference's own
    GPU-vs-CPU AMaZE criterion (crates/gpu/src/sensor/amaze_tests.rs: at most
    0.5% of samples outside 2e-5 (1 + |x|)), and its maximum, after the RL
    gain, by 1e-2."""
    from rohditor_gb300 import GpuPreviewProcessor, GpuSensorProcessor, GpuSpatialProcessor
    from rohditor_gb300.workloads import full_24mp

    wl = full_24mp()
    w, h = wl.width, wl.height
    raw = wl.mosaic(device)
    src = GpuSensorProcessor(device).develop(raw, wl.sensor, wl.capture)
    got = src.download()
    odesc = oracle.sensor_desc(w, h, w, (0, 0, w, h), 0, [512.0], (1, 1), [16383.0])
    m, pattern = oracle.normalize(raw, odesc)
    ref_h, stats, _, _ = oracle.opposed(m, pattern, wl.sensor.detection_levels, wl.sensor.neutral_ceiling)
    gpu_h, gpu_stats = stages.highlight(raw, wl.sensor)
    assert list(src.metrics.highlight_stats) == stats.tolist() == gpu_stats.tolist()
    assert float(np.max(np.abs(gpu_h - ref_h))) <= 1e-4
    # Demosaic + RL from the GPU's own highlight output: bit-exact.
    ref = oracle.capture(oracle.demosaic(gpu_h, pattern, wl.as_shot, 3), 0.5, 0.7, 0.5, wl.capture.ceilings, 10)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # Chained: the oracle fed its own Opposed output.
    chained = oracle.capture(oracle.demosaic(ref_h, pattern, wl.as_shot, 3), 0.5, 0.7, 0.5, wl.capture.ceilings, 10)
    d = np.abs(got - chained)
    assert (d > 2e-5 * (1.0 + np.abs(chained))).mean() <= 5e-3
    assert float(d.max()) <= 1e-2
    del ref, m, chained, d, gpu_h, ref_h
    c = wl.color
    base = GpuSpatialProcessor(device).reduce_preview(src, wl.optics, wl.target, c.wb_gains, c.camera_to_rec2020)
    ref_o = oracle.optics_apply(oracle.optics_desc_from(wl.optics.to_c()), got)
    ref_b = oracle.camera_matrix(oracle.white_balance(oracle.area_reduce(ref_o, wl.target), c.wb_gains),
                                 c.camera_to_rec2020)
    got_b = base.download()
    assert np.array_equal(got_b.view(np.uint32), ref_b.view(np.uint32))
    out, hist = GpuPreviewProcessor(device).render(base, c)
    x = oracle.adjust(got_b, c.exposure_ev, c.base_lut, c.tone_lut, c.saturation, c.vibrance, c.hsl, c.grading)
    diff = np.abs(out.astype(int) - oracle.display_srgb8(x).astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() <= 1e-3
    ref_hist, _ = oracle.histogram(out)
    assert np.array_equal(np.concatenate([hist.red, hist.green, hist.blue, hist.luminance]), ref_hist)
    base.release()
    src.release()


def test_largest_export_workload_against_the_oracle(device, stages, oracle):
    """The largest configured frame, one image of the export stream: 11648x8736
    RGGB 16-bit (white 65535, black 1024) with 0.5% hot pixels and specular
    blobs, Opposed + AMaZE + RL K=20, then the full optics (Poly5 distortion,
    linear TCA, vignetting) and the area reduction to 2560x1920 with WB +
    matrix. Checked at full size like the 24 MP workload: Opposed statistics
    exact and samples within 1e-4; AMaZE + 20 RL iterations from the GPU's
    own highlight output bit-exact; the spatial stage bit-exact."""
    from rohditor_gb300 import GpuSensorProcessor, GpuSpatialProcessor
    from rohditor_gb300.workloads import large_export

    wl = large_export(count=1)[0]
    w, h = wl.width, wl.height
    raw = wl.mosaic(device)
    src = GpuSensorProcessor(device).develop(raw, wl.sensor, wl.capture)
    got = src.download()
    odesc = oracle.sensor_desc(w, h, w, (0, 0, w, h), 0, [wl.black], (1, 1), [wl.white])
    m, pattern = oracle.normalize(raw, odesc)
    ref_h, stats, _, _ = oracle.opposed(m, pattern, wl.sensor.detection_levels, wl.sensor.neutral_ceiling)
    del m
    gpu_h, gpu_stats = stages.highlight(raw, wl.sensor)
    assert list(src.metrics.highlight_stats) == stats.tolist() == gpu_stats.tolist()
    assert float(np.max(np.abs(gpu_h - ref_h))) <= 1e-4
    del ref_h, raw
    cap = wl.capture
    ref = oracle.capture(oracle.demosaic(gpu_h, pattern, wl.as_shot, 3), cap.amount, cap.radius,
                         cap.noise_protection, cap.ceilings, cap.iterations)
    assert cap.iterations == 20
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    del ref, gpu_h
    c = wl.color
    base = GpuSpatialProcessor(device).reduce_preview(src, wl.optics, wl.target, c.wb_gains, c.camera_to_rec2020)
    ref_o = oracle.optics_apply(oracle.optics_desc_from(wl.optics.to_c()), got)
    ref_b = oracle.camera_matrix(oracle.white_balance(oracle.area_reduce(ref_o, wl.target), c.wb_gains),
                                 c.camera_to_rec2020)
    assert np.array_equal(base.download().view(np.uint32), ref_b.view(np.uint32))
    base.release()
    src.release()


def test_concurrent_lanes_with_different_widths_repeat_exactly(device):
    """Lanes on several threads launch the same kernels with different image
    widths at once (per-launch shared-memory sizes, work counters, tuning
    runs); repeated runs and a single lane give the same bytes."""
    from rohditor_gb300 import CaptureContract, ColorContract, OpticsExecution, SensorDescription, clip_levels
    from rohditor_gb300.batch import BatchImage, develop_batch
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, preview_dimensions

    images = []
    for k, (w, h) in enumerate([(1024, 96), (260, 300), (704, 128), (392, 200), (896, 72), (264, 264),
                                (640, 160), (512, 112)]):
        wb = (2.0, 1.0, 1.6)
        sensor = SensorDescription(w, h, cfa="RGGB", black=(256.0,), white=(4095.0,), highlight="clip",
                                   clip_levels=clip_levels(1.0, wb), demosaic="amaze", demosaic_balance=wb)
        cap = CaptureContract(amount=0.5, radius=0.3 + 0.3 * (k % 4), noise_protection=0.5,
                              ceilings=clip_levels(1.0, wb), iterations=3)
        optics = OpticsExecution(w, h, vignetting_k=(-0.3, 0.05, -0.01))
        images.append(BatchImage(raw_mosaic(w, h, w, seed=90 + k), sensor, cap, optics,
                                 preview_dimensions(w, h, 256), wb, CAMERA_TO_REC2020,
                                 ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020)))
    ref = develop_batch(images, lanes=1)[0]
    for _ in range(3):
        outs = develop_batch(images, lanes=4)[0]
        for (a, ha), (b, hb) in zip(outs, ref):
            assert np.array_equal(a, b) and np.array_equal(ha, hb)


@pytest.mark.parametrize("mode", ["lanes", "graph", "flat", "flat_graph"])
def test_batched_develop_matches_one_at_a_time(device, mode):
    """rd_develop_batch (concurrent lanes), rd_develop_batch_graph (one
    captured CUDA graph), rd_develop_batch_flat (stage by stage: one AMaZE
    launch over every image's tiles, one launch per RL iteration over the work
    items of the images that share their taps) and rd_develop_batch_flat_graph
    (the stage-by-stage batch as one CUDA graph) over uneven sizes, CFA phases,
    highlight modes, capture radii and iteration counts equal the per-image
    path, bit for bit. The 702-wide image has no tensor maps (its rows are not
    a multiple of 16 bytes) and the 200x150 one is below the step kernel's
    size, so both leave the flat RL launches of the others; the last two
    images are demosaiced with RCD and MHC, outside the flat AMaZE launch."""
    graph = mode in ("graph", "flat_graph")
    from rohditor_gb300 import (CaptureContract, ColorContract, GpuPreviewProcessor, GpuSensorProcessor,
                                GpuSpatialProcessor, OpticsExecution, SensorDescription, clip_levels, opposed_levels)
    from rohditor_gb300.batch import BatchImage, develop_batch
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, hsl_bands, preview_dimensions, sixteen_knot_curve

    shapes = [(700, 467, "RGGB", "clip", "amaze"), (1024, 768, "GBRG", "opposed", "amaze"),
              (512, 384, "BGGR", "clip", "amaze"), (640, 480, "GRBG", "opposed", "amaze"),
              (702, 300, "RGGB", "clip", "amaze"), (200, 150, "GBRG", "clip", "amaze"),
              (384, 256, "GRBG", "opposed", "rcd"), (320, 240, "BGGR", "clip", "mhc")]
    images = []
    for k, (w, h, cfa, hl, dm) in enumerate(shapes):
        raw = raw_mosaic(w, h, w, seed=70 + k)
        wb = (2.0 - 0.1 * k, 1.0, 1.6 + 0.1 * k)
        if hl == "clip":
            sensor = SensorDescription(w, h, cfa=cfa, black=(256.0,), white=(4095.0,), highlight="clip",
                                       clip_levels=clip_levels(1.0, wb), demosaic=dm, demosaic_balance=wb)
            ceil = clip_levels(1.0, wb)
        else:
            det, neutral = opposed_levels(1.0, wb)
            sensor = SensorDescription(w, h, cfa=cfa, black=(256.0,), white=(4095.0,), highlight="opposed",
                                       detection_levels=det, neutral_ceiling=neutral, demosaic=dm,
                                       demosaic_balance=wb)
            ceil = (1.0, 1.0, 1.0)
        cap = CaptureContract(amount=0.5, radius=0.7 if k % 2 == 0 else 1.1, noise_protection=0.5, ceilings=ceil,
                              iterations=5 - k % 3)
        optics = OpticsExecution(w, h, distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                                 tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0), vignetting_k=(-0.3, 0.05, -0.01))
        color = ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020, exposure_ev=0.1 * k,
                              tone_lut=sixteen_knot_curve(seed=k), hsl=hsl_bands(seed=k))
        images.append(BatchImage(raw, sensor, cap, optics, preview_dimensions(w, h, 256), wb, CAMERA_TO_REC2020,
                                 color))
    res = develop_batch(images, lanes=3, graph=graph, flat=mode.startswith("flat"))
    outs, ms, wall = res[:3]
    assert wall > 0 and (graph or all(m > 0 for m in ms))
    if graph:
        # Pinned buffers used in place by the graph give the same outputs.
        from rohditor_gb300.batch import PinnedBatch
        pinned = PinnedBatch(images)
        pinned.run(lanes=2, graph=True, flat=mode == "flat_graph")
        for (a, ha), (b, hb) in zip(outs, pinned.outputs()):
            assert np.array_equal(a, b) and np.array_equal(ha, hb)
        pinned.close()
    for im, (srgb, hist) in zip(images, outs):
        src = GpuSensorProcessor(device).develop(im.mosaic, im.sensor, im.capture)
        base = GpuSpatialProcessor(device).reduce_preview(src, im.optics, im.target, im.wb_gains,
                                                          im.camera_to_rec2020)
        ref, ref_hist = GpuPreviewProcessor(device).render(base, im.color)
        base.release()
        src.release()
        assert np.array_equal(srgb, ref)
        assert np.array_equal(hist[:256], ref_hist.red) and np.array_equal(hist[768:], ref_hist.luminance)


@pytest.mark.parametrize("mode", ["lanes", "graph", "flat", "flat_graph"])
def test_batched_develop_reports_an_invalid_image_and_recovers(device, mode):
    """A batch holding an image the develop refuses (its crop lies outside the
    sensor) fails with that status in every batched form, including the
    captured ones, whose graph is then abandoned; the next batch of valid
    images runs and equals the per-image path."""
    from rohditor_gb300 import (CaptureContract, ColorContract, GpuPreviewError, GpuPreviewProcessor,
                                GpuSensorProcessor, GpuSpatialProcessor, OpticsExecution, SensorDescription,
                                clip_levels)
    from rohditor_gb300.batch import BatchImage, develop_batch
    from rohditor_gb300.workloads import CAMERA_TO_REC2020, preview_dimensions

    def image(k, crop=None):
        w, h = 512, 320
        wb = (2.0, 1.0, 1.6)
        sensor = SensorDescription(w, h, cfa="RGGB", crop=crop, black=(256.0,), white=(4095.0,), highlight="clip",
                                   clip_levels=clip_levels(1.0, wb), demosaic="amaze", demosaic_balance=wb)
        cap = CaptureContract(amount=0.5, radius=0.7, noise_protection=0.5, ceilings=clip_levels(1.0, wb),
                              iterations=3)
        return BatchImage(raw_mosaic(w, h, w, seed=110 + k), sensor, cap, OpticsExecution(w, h),
                          preview_dimensions(w, h, 256), wb, CAMERA_TO_REC2020,
                          ColorContract(wb_gains=wb, camera_to_rec2020=CAMERA_TO_REC2020))

    graph, flat = mode in ("graph", "flat_graph"), mode.startswith("flat")
    bad = [image(0), image(1, crop=(400, 0, 200, 320)), image(2)]
    with pytest.raises(GpuPreviewError) as err:
        develop_batch(bad, lanes=2, graph=graph, flat=flat)
    assert err.value.variant == "InvalidInput", str(err.value)
    good = [image(3), image(4)]
    outs = develop_batch(good, lanes=2, graph=graph, flat=flat)[0]
    for im, (srgb, hist) in zip(good, outs):
        src = GpuSensorProcessor(device).develop(im.mosaic, im.sensor, im.capture)
        base = GpuSpatialProcessor(device).reduce_preview(src, im.optics, im.target, im.wb_gains,
                                                          im.camera_to_rec2020)
        ref, ref_hist = GpuPreviewProcessor(device).render(base, im.color)
        base.release()
        src.release()
        assert np.array_equal(srgb, ref)
        assert np.array_equal(hist[:256], ref_hist.red)
