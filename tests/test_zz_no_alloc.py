"""rd_render_device_noalloc against the allocating render entry point.

The allocation-free render runs the same colour kernel with its LUTs staged in a
static device array. With unit white balance and an identity camera matrix,
rd_stage_color applies exactly the same arithmetic to the same base, so the
8-bit output and the histogram must be identical; both are also checked
against the oracle directly (the adjustment chain, the sRGB8 conversion and
the histogram of the kernel's own output). Two calls in a row with different
LUTs check that nothing stale survives in the static array or in the
histogram. This file is collected last so it also runs after every other GPU
test in one process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IDENTITY = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)


def _base(seed: int, h: int, w: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = rng.uniform(-0.05, 0.8, size=(h, 3 * w))
    rgb = (np.sign(u) * np.abs(u) ** 1.5).astype(np.float32)
    rgb[:3] = 2.5
    return rgb


def _contract(variant: str):
    from rohditor_gb300 import ColorContract, standard_base_lut
    from rohditor_gb300.workloads import hsl_bands, sixteen_knot_curve

    if variant == "config":
        return ColorContract(wb_gains=(1.0, 1.0, 1.0), camera_to_rec2020=IDENTITY, exposure_ev=0.5,
                             base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(), hsl=hsl_bands())
    return ColorContract(wb_gains=(1.0, 1.0, 1.0), camera_to_rec2020=IDENTITY, exposure_ev=-0.25,
                         base_lut=standard_base_lut(), tone_lut=sixteen_knot_curve(seed=23), saturation=1.2,
                         vibrance=0.3,
                         grading=np.array([[0.2, -0.1, 0.05], [0.0, 0.1, -0.2], [-0.1, 0.0, 0.3]], np.float32))


def test_noalloc_render_matches_render_entry_point(device, stages, oracle):
    torch = pytest.importorskip("torch")
    lib = device.lib
    h, w = 181, 263
    runs = [(_base(3, h, w), _contract("config")), (_base(4, h, w), _contract("grading"))]
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    for rgb, contract in runs:
        ref_out, ref_hist, _ = stages.color(rgb, contract)
        planar = np.ascontiguousarray(rgb.reshape(h, w, 3).transpose(2, 0, 1))
        d_base = torch.from_numpy(planar).cuda()
        d_out = torch.full((h, 3 * w), 7, dtype=torch.uint8, device="cuda")
        d_hist = torch.full((1024,), 12345, dtype=torch.int64, device="cuda")
        desc = contract.to_c()
        torch.cuda.synchronize()
        rc = lib.rd_render_device_noalloc(d_base.data_ptr(), w, h, ctypes.byref(desc), d_out.data_ptr(),
                                          d_hist.data_ptr(), stream.cuda_stream)
        assert rc == 0, lib.rd_status_name(rc)
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        hist = d_hist.cpu().numpy().view(np.uint64)
        assert np.array_equal(out, ref_out)
        assert np.array_equal(hist, ref_hist)
        c = contract
        x = oracle.adjust(rgb, c.exposure_ev, c.base_lut, c.tone_lut, c.saturation, c.vibrance, c.hsl, c.grading)
        diff = np.abs(out.astype(np.int32) - oracle.display_srgb8(x).astype(np.int32))
        assert diff.max() <= 1 and (diff > 0).mean() <= 1e-3  # the sRGB8 bar: 1 code on at most 0.1%
        assert np.array_equal(hist, oracle.histogram(out)[0])


def test_noalloc_render_rejects_bad_arguments(device):
    torch = pytest.importorskip("torch")
    lib = device.lib
    from rohditor_gb300 import ColorContract

    desc = ColorContract(wb_gains=(1.0, 1.0, 1.0), camera_to_rec2020=IDENTITY).to_c()
    buf = torch.zeros(4096, dtype=torch.float32, device="cuda")
    ptr = buf.data_ptr()
    assert lib.rd_render_device_noalloc(None, 4, 4, ctypes.byref(desc), ptr, ptr, None) != 0
    assert lib.rd_render_device_noalloc(ptr, 0, 4, ctypes.byref(desc), ptr, ptr, None) != 0
    assert lib.rd_render_device_noalloc(ptr, 4, 4, None, ptr, ptr, None) != 0


def test_noalloc_render_refuses_a_capturing_stream(device):
    # The LUT copies come from the caller's descriptor on every call, which a
    # graph cannot record: the call is refused and enqueues nothing.
    torch = pytest.importorskip("torch")
    lib = device.lib
    from rohditor_gb300 import ColorContract

    desc = ColorContract(wb_gains=(1.0, 1.0, 1.0), camera_to_rec2020=IDENTITY).to_c()
    buf = torch.zeros(4096, dtype=torch.float32, device="cuda")
    ptr = buf.data_ptr()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        graph.capture_begin()
        rc = lib.rd_render_device_noalloc(ptr, 4, 4, ctypes.byref(desc), ptr, ptr, side.cuda_stream)
        buf.add_(1.0)
        graph.capture_end()
    assert rc == 8  # RD_INVALID_INPUT
    graph.replay()
    torch.cuda.synchronize()
    assert float(buf[0]) == 1.0
    assert lib.rd_render_device_noalloc(ptr, 4, 4, ctypes.byref(desc), ptr, ptr, side.cuda_stream) == 0
    torch.cuda.synchronize()
