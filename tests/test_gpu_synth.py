"""The library's device scene generator equals the oracle's host restatement bit for bit.

Both benchmark arms develop the same seeded mosaic: the GPU arm generates it
on the device (rd_synth_mosaic), the CPU arm with the oracle (synth.cpp)
without loading the library. Every sample is compared.
"""

import numpy as np
import pytest

import workload_spec as spec

pytestmark = pytest.mark.gpu


def device_mosaic(device, dv):
    from rohditor_gb300.workloads import from_spec

    return from_spec(dv).mosaic(device)


@pytest.mark.parametrize("case", ["full_24mp_small", "plain_3mp", "batch_bggr_12bit", "export_hot_pixels",
                                  "no_clipping"])
def test_device_generator_equals_the_oracle(device, oracle, case):
    from oracle import develop as od

    if case == "full_24mp_small":
        dv = spec.full_24mp(width=1536, height=1030)
    elif case == "plain_3mp":
        dv = spec.plain_3mp()
    elif case == "batch_bggr_12bit":
        dv = next(d for d in spec.batched_uneven(12) if d.scene.cfa != "RGGB" and d.scene.bits == 12)
        s = dv.scene
        dv.scene = spec.Scene(1000, 750, s.cfa, s.bits, s.black, s.white, s.clip_fraction, s.blobs, s.as_shot,
                              s.seed)
    elif case == "export_hot_pixels":
        dv = spec.large_export(1)[0]
        s = dv.scene
        dv.scene = spec.Scene(1165, 874, s.cfa, s.bits, s.black, s.white, s.clip_fraction, s.blobs, s.as_shot,
                              s.seed, s.hot_pixel_fraction)
    else:
        dv = spec.full_24mp(width=640, height=480)
        s = dv.scene
        dv.scene = spec.Scene(s.width, s.height, s.cfa, s.bits, s.black, s.white, 0.0, False, s.as_shot, 9)
    ours = device_mosaic(device, dv)
    ref = od.mosaic(dv)
    assert ours.shape == ref.shape
    bad = np.flatnonzero(ours != ref)
    assert bad.size == 0, f"{bad.size} samples differ, first at {np.unravel_index(bad[0], ours.shape)}"


def test_full_24mp_mosaic_equals_the_oracle(device, oracle):
    from oracle import develop as od

    dv = spec.full_24mp()
    assert np.array_equal(device_mosaic(device, dv), od.mosaic(dv))
