"""The kernels' bounded device waits, made to run out on purpose.

AMaZE's phase B waits for its tile's phase A to publish the tile's slab (a
flag in global memory), and AMaZE and the capture-sharpening, bilinear / MHC
and RCD kernels wait on shared-memory barriers for their tensor copies. Each
wait gives up after an iteration limit, records why in the context's error
word and returns. Here rd_ctx_set_wait_test shortens the limits and withholds
one completion (the flag of AMaZE tile 0; AMaZE's mosaic-row copies; the
first tensor copy of every capture-sharpening block; the tile copy of every
bilinear / MHC and RCD block), so the wait runs out: the
call must fail with RD_INVALID_INPUT naming the wait, nothing may trap or
hang, and the same context must then give the oracle's result again.
"""

import numpy as np
import pytest

from rohditor_gb300 import CaptureContract, GpuPreviewError

pytestmark = pytest.mark.gpu

RD_INVALID_INPUT = 8
RD_WAIT_NONE, RD_WAIT_AMAZE_TILE, RD_WAIT_RL_COPY, RD_WAIT_DEMOSAIC_COPY, RD_WAIT_AMAZE_COPY = 0, 1, 2, 3, 4


def mosaic(w, h, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.02, 0.9, size=(h, w)).astype(np.float32)


def test_amaze_tile_wait_runs_out_and_the_context_stays_usable(device, stages, oracle):
    m = mosaic(600, 500, 1)
    ref = oracle.demosaic(m, 0, (1.0, 1.0, 1.0), 3)
    device.check(device.lib.rd_ctx_set_wait_test(device.handle, 2000, RD_WAIT_AMAZE_TILE))
    try:
        with pytest.raises(GpuPreviewError) as err:
            stages.demosaic(m, "RGGB", "amaze")
    finally:
        device.check(device.lib.rd_ctx_set_wait_test(device.handle, 0, RD_WAIT_NONE))
    assert err.value.code == RD_INVALID_INPUT
    assert "demosaic tile wait timed out" in str(err.value)
    out = stages.demosaic(m, "RGGB", "amaze")
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("size", [(640, 128), (1280, 600)])
def test_capture_copy_wait_runs_out_and_the_context_stays_usable(device, stages, oracle, size):
    w, h = size
    rgb = np.repeat(mosaic(w, h, 2)[:, :, None], 3, axis=2).reshape(h, 3 * w)
    rgb[:, 0::3] *= np.float32(0.8)
    cap = CaptureContract(amount=0.6, radius=0.7, noise_protection=0.4, ceilings=(1.0, 1.0, 1.0), iterations=4)
    ref = oracle.capture(rgb, cap.amount, cap.radius, cap.noise_protection, cap.ceilings, cap.iterations)
    device.check(device.lib.rd_ctx_set_wait_test(device.handle, 2000, RD_WAIT_RL_COPY))
    try:
        with pytest.raises(GpuPreviewError) as err:
            stages.capture(rgb, cap)
    finally:
        device.check(device.lib.rd_ctx_set_wait_test(device.handle, 0, RD_WAIT_NONE))
    assert err.value.code == RD_INVALID_INPUT
    assert "tensor copy timed out" in str(err.value)
    out = stages.capture(rgb, cap)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("algorithm", ["mhc", "bilinear", "rcd"])
def test_demosaic_tile_copy_wait_runs_out_and_the_context_stays_usable(device, stages, oracle, algorithm):
    m = mosaic(640, 320, 3)  # rows of 2560 bytes: the tiles arrive by tensor copy
    ref = oracle.demosaic(m, 0, (1.0, 1.0, 1.0), {"bilinear": 0, "mhc": 1, "rcd": 2}[algorithm])
    device.check(device.lib.rd_ctx_set_wait_test(device.handle, 2000, RD_WAIT_DEMOSAIC_COPY))
    try:
        with pytest.raises(GpuPreviewError) as err:
            stages.demosaic(m, "RGGB", algorithm)
    finally:
        device.check(device.lib.rd_ctx_set_wait_test(device.handle, 0, RD_WAIT_NONE))
    assert err.value.code == RD_INVALID_INPUT
    assert "demosaic tile copy timed out" in str(err.value)
    out = stages.demosaic(m, "RGGB", algorithm)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_amaze_row_copy_wait_runs_out_and_the_context_stays_usable(device, stages, oracle):
    m = mosaic(704, 480, 4)  # rows of 2816 bytes: the inner tiles' rows arrive by tensor copy
    ref = oracle.demosaic(m, 0, (1.0, 1.0, 1.0), 3)
    device.check(device.lib.rd_ctx_set_wait_test(device.handle, 2000, RD_WAIT_AMAZE_COPY))
    try:
        with pytest.raises(GpuPreviewError) as err:
            stages.demosaic(m, "RGGB", "amaze")
    finally:
        device.check(device.lib.rd_ctx_set_wait_test(device.handle, 0, RD_WAIT_NONE))
    assert err.value.code == RD_INVALID_INPUT
    assert "demosaic tile copy timed out" in str(err.value)
    out = stages.demosaic(m, "RGGB", "amaze")
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_unknown_withheld_completion_is_rejected(device):
    assert device.lib.rd_ctx_set_wait_test(device.handle, 0, 7) == RD_INVALID_INPUT
    device.check(device.lib.rd_ctx_set_wait_test(device.handle, 0, RD_WAIT_NONE))
