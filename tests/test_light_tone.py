"""The Light tone table (contrast, highlights, shadows, whites, blacks) on the CPU.

The oracle's LightToneLut against the reference's own tests of it
(crates/edit/src/light.rs:144-265, restated: neutral identity with identity
extensions, extended sampling through 1 without a jump, an extreme
combination bounded and monotone, small signed changes without new clipping,
local shadow / highlight masks, black and white points owning the
endpoints), and the library's host builder rd_light_tone_lut bit for bit
against the oracle. The GPU chain step is checked in test_gpu_parity.py and
test_gpu_output.py.
"""

import numpy as np
import pytest

BLACK_STRENGTH = 0.25


def sample(lut, x):
    """LightToneLut::sample (light.rs:49-52 with sample_lut :78-88) in f32."""
    x = np.float32(x)
    if not (np.float32(0) <= x <= np.float32(1)):
        return x
    pos = np.float32(x * np.float32(4095))
    lo = int(np.floor(pos))
    hi = min(lo + 1, 4095)
    frac = np.float32(pos - np.float32(lo))
    return np.float32(lut[lo] + np.float32(np.float32(lut[hi] - lut[lo]) * frac))


def sample_extended(lut, x):
    """LightToneLut::sample_extended (light.rs:59-64)."""
    x = np.float32(x)
    if np.isfinite(x) and x > 1:
        return np.float32(np.float32(x + lut[4095]) - np.float32(1))
    return sample(lut, x)


def test_neutral_lut_is_identity_with_identity_extensions(oracle):
    lut = oracle.light_tone_lut()
    for x in (0.0, 0.01, 0.18, 0.5, 0.91, 1.0):
        assert abs(sample(lut, x) - np.float32(x)) < 1e-6
    assert sample(lut, -0.25) == np.float32(-0.25)
    assert sample(lut, 1.5) == np.float32(1.5)
    assert np.isnan(sample(lut, np.nan))


def test_extended_sampling_continues_through_one_without_a_jump(oracle):
    lut = oracle.light_tone_lut(whites=-1.0)
    at_one = sample(lut, 1.0)
    assert at_one < 0.9
    assert sample(lut, 1.01) == np.float32(1.01)
    assert abs(sample_extended(lut, 1.01) - (at_one + np.float32(0.01))) < 1e-6
    prev = np.float32(0)
    for i in range(801):
        out = sample_extended(lut, np.float32(i) / np.float32(100))
        assert out >= prev
        prev = out
    for x in (-0.5, 0.0, 0.3, 0.97, 1.0):
        assert sample_extended(lut, x) == sample(lut, x)
    assert np.isnan(sample_extended(lut, np.nan))
    assert sample_extended(oracle.light_tone_lut(), 3.0) == np.float32(3.0)


def test_extreme_combination_is_bounded_and_monotonic(oracle):
    lut = oracle.light_tone_lut(contrast=1.0, highlights=1.0, shadows=-1.0, whites=-1.0, blacks=1.0)
    assert lut.min() >= 0.0 and lut.max() <= 1.0
    assert np.all(np.diff(lut) >= 0)


@pytest.mark.parametrize("slider", ["contrast", "shadows", "highlights", "blacks", "whites"])
@pytest.mark.parametrize("amount", [-0.05, 0.05])
def test_small_signed_changes_move_without_creating_new_clipping(oracle, slider, amount):
    lut = oracle.light_tone_lut(**{slider: amount})
    for x in (0.02, 0.09, 0.22, 0.47, 0.73, 0.91, 0.98):
        out = sample(lut, x)
        assert 0.0 < out < 1.0


def test_shadow_and_highlight_masks_are_local(oracle):
    shadows = oracle.light_tone_lut(shadows=0.5)
    assert sample(shadows, 0.2) - np.float32(0.2) > 0.05
    assert abs(sample(shadows, 0.9) - np.float32(0.9)) < 1e-5
    highlights = oracle.light_tone_lut(highlights=-0.5)
    assert np.float32(0.8) - sample(highlights, 0.8) > 0.05
    assert abs(sample(highlights, 0.1) - np.float32(0.1)) < 1e-5


def test_black_and_white_controls_own_the_endpoints(oracle):
    raised_blacks = oracle.light_tone_lut(blacks=1.0)
    assert abs(sample(raised_blacks, 0.0) - BLACK_STRENGTH) < 1e-6
    assert abs(sample(raised_blacks, 0.8) - np.float32(0.8)) < 1e-5
    lowered_whites = oracle.light_tone_lut(whites=-1.0)
    assert sample(lowered_whites, 1.0) < 1.0
    assert abs(sample(lowered_whites, 0.2) - np.float32(0.2)) < 1e-5


@pytest.mark.parametrize("sliders", [(0.4, -0.5, 0.35, -0.2, 0.15), (1.0, 1.0, -1.0, -1.0, 1.0),
                                     (-0.8, 0.0, 0.0, 0.0, 0.0), (0.0, 0.0, 0.0, 0.7, -0.6),
                                     (0.05, -0.05, 0.05, -0.05, 0.05)])
def test_library_table_equals_the_oracle_bit_for_bit(oracle, sliders):
    from rohditor_gb300 import light_tone_lut

    ours = light_tone_lut(*sliders)
    ref = oracle.light_tone_lut(*sliders)
    assert ours.view(np.uint32).tolist() == ref.view(np.uint32).tolist()


def test_table_is_skipped_when_every_slider_is_neutral():
    """stages.rs:434-439: no Light tone step unless a slider is non-zero."""
    from rohditor_gb300 import ColorContract, light_tone_lut

    assert light_tone_lut() is None
    assert light_tone_lut(0.0, 0.0, 0.0, 0.0, 0.0) is None
    d = ColorContract(light_tone_lut=light_tone_lut()).to_c()
    assert d.has_light_tone_lut == 0
    d = ColorContract(light_tone_lut=light_tone_lut(contrast=0.2)).to_c()
    assert d.has_light_tone_lut == 1
