"""Both benchmark arms resolve the same workload from workload_spec.

The GPU arm (rohditor_gb300.workloads, the library's host helpers) and the CPU
arm (oracle/develop.py, the oracle's restatements) must describe the same
develop: the same level ceilings, capture ceilings, optics plan, LUTs and
workload string. The mosaic itself is compared bit for bit on the GPU
(test_gpu_synth.py); here the oracle's generator is checked for determinism
and for the scene statistics the workloads ask for.
"""

import numpy as np
import pytest

import workload_spec as spec


def test_oracle_generator_is_deterministic_and_clips_as_asked(oracle):
    from oracle import develop as od

    dv = spec.full_24mp(width=1024, height=768)
    a = od.mosaic(dv)
    b = od.mosaic(dv)
    assert a.dtype == np.uint16 and a.shape == (768, 1024)
    assert np.array_equal(a, b)
    clipped = (a >= 16383).mean()
    assert 0.01 < clipped < 0.08
    assert 512 - 50 < np.median(a) < 16383
    other = od.mosaic(spec.full_24mp(width=1024, height=768, seed=3))
    assert not np.array_equal(a, other)


def test_hot_pixels_come_from_the_generator(oracle):
    from oracle import develop as od

    dv = spec.large_export(1)[0]
    s = dv.scene
    small = spec.Develop(dv.name, spec.Scene(512, 384, s.cfa, s.bits, s.black, s.white, s.clip_fraction, s.blobs,
                                             s.as_shot, s.seed, s.hot_pixel_fraction), dv.highlight, dv.demosaic,
                         dv.capture, dv.lens, dv.target, dv.wb_gains, dv.camera_to_rec2020)
    m = od.mosaic(small)
    hot = (m == 65535).mean()
    assert 0.004 < hot < 0.1


@pytest.mark.parametrize("highlight", ["opposed", "clip"])
def test_both_arms_resolve_the_same_levels(oracle, highlight):
    from oracle import develop as od
    from rohditor_gb300 import capture_ceilings, clip_levels, opposed_levels

    for dv in [spec.full_24mp(highlight=highlight)] + spec.batched_uneven(6):
        s = dv.scene
        assert np.array_equal(np.float32(clip_levels(1.0, dv.wb_gains)), np.float32(od.clip_levels(1.0, dv.wb_gains)))
        det_a, ceil_a = opposed_levels(1.0, s.as_shot)
        det_b, ceil_b = od.opposed_levels(1.0, s.as_shot)
        assert np.array_equal(np.float32(det_a), np.float32(det_b))
        assert np.array_equal(np.float32(ceil_a), np.float32(ceil_b))
        assert np.array_equal(np.float32(capture_ceilings(highlight, 1.0, dv.wb_gains)),
                              np.float32(od.capture_ceilings(highlight, 1.0, dv.wb_gains)))


def test_capture_ceilings_follow_the_reference_rule():
    """detail.rs:323-337: Clip without the detection margin, Opposed the bare threshold."""
    from rohditor_gb300 import capture_ceilings

    assert capture_ceilings("opposed", 1.0, (2.0, 1.0, 1.6)) == (1.0, 1.0, 1.0)
    c = capture_ceilings("clip", 1.0, (2.0, 1.0, 1.6))
    assert c == (float(np.float32(0.5)), 1.0, float(np.float32(np.float32(1.0) / np.float32(1.6))))
    assert capture_ceilings("off", 1.0, (2.0, 1.0, 1.6)) == (1.0, 1.0, 1.0)


def test_both_arms_resolve_the_same_optics_plan_and_luts(oracle):
    from oracle import develop as od
    from rohditor_gb300 import standard_base_lut
    from rohditor_gb300.workloads import from_spec

    for dv in (spec.full_24mp(), spec.batched_uneven(3)[2], spec.large_export(1)[0]):
        wl = from_spec(dv)
        ours = wl.optics.to_c()
        ref = od.optics_desc(dv)
        for f in ("norm_scale", "norm_unscale", "center_x", "center_y"):
            assert getattr(ours, f) == getattr(ref, f), f
        assert np.float32(ours.scale) == np.float32(ref.scale)
        assert list(ours.vignetting_k) == list(ref.vignetting)
    assert np.array_equal(standard_base_lut(), oracle.standard_base_lut())


def test_workload_string_names_the_develop():
    s = spec.full_24mp().describe()
    assert s.startswith("full_24mp 6048x4024 RGGB 14-bit + opposed + amaze + RL10")
    assert "area->2560x1703" in s
    assert "full resolution" in spec.plain_3mp().describe()
    assert spec.full_24mp(demosaic="rcd").describe() != s
