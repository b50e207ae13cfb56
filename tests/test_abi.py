"""The C-ABI library on the CPU: it loads, exports every entry point that
include/rd_gpu.h declares, and its host-side contract helpers (status
routing, descriptor validation, optics plan, base rendering LUT) agree with
the oracle. No device compute runs here."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "rd_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rd_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from rohditor_gb300 import _ffi

    return _ffi.load()


def test_library_exports_every_declared_symbol(lib):
    from rohditor_gb300 import _ffi

    names = declared_symbols()
    assert len(names) >= 30
    raw = ctypes.CDLL(_ffi.library_path())
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing
    assert set(names) == set(_ffi.SIGNATURES), set(names) ^ set(_ffi.SIGNATURES)


def test_status_routing_mirrors_gpu_preview_error(lib):
    # GpuPreviewError::is_routing: only UnsupportedEdits and OverBudget keep the device.
    routing = {c for c in range(10) if lib.rd_status_is_routing(c)}
    assert routing == {3, 6}
    assert lib.rd_status_name(0) == b"Ok" and lib.rd_status_name(9) == b"Readback"


def test_supports_validates_contracts(lib):
    from rohditor_gb300 import SensorDescription

    ok = SensorDescription(100, 80, black=(64.0,), white=(4095.0,), highlight="clip")
    assert SensorDescription.__name__ and lib.rd_supports(ctypes.byref(ok.to_c())) == 1
    bad_levels = SensorDescription(100, 80, black=(5000.0,), white=(4095.0,))
    assert lib.rd_supports(ctypes.byref(bad_levels.to_c())) == 0
    bad_crop = SensorDescription(100, 80, crop=(90, 0, 20, 10))
    assert lib.rd_supports(ctypes.byref(bad_crop.to_c())) == 0
    d = ok.to_c()
    d.demosaic = 7
    assert lib.rd_supports(ctypes.byref(d)) == 0


@pytest.mark.parametrize("size", [(6048, 4024), (3008, 2008), (640, 427)])
def test_optics_plan_matches_oracle(lib, oracle, size):
    from rohditor_gb300 import OpticsExecution

    ex = OpticsExecution(size[0], size[1], distortion="poly5", distortion_k=(-0.02, 0.005, 0.0), tca="linear",
                         tca_red=(1.0003, 0, 0), tca_blue=(0.9997, 0, 0))
    c = ex.to_c()
    o = oracle.optics_plan(size[0], size[1], 2, (-0.02, 0.005, 0.0), 1, (1.0003, 0, 0), (0.9997, 0, 0))
    assert (c.norm_scale, c.norm_unscale, c.center_x, c.center_y) == (o.norm_scale, o.norm_unscale, o.center_x,
                                                                      o.center_y)
    assert np.float32(c.scale) == np.float32(o.scale)


def test_base_lut_matches_oracle(lib, oracle):
    from rohditor_gb300 import standard_base_lut

    assert np.array_equal(standard_base_lut(), oracle.standard_base_lut())


def test_highlight_levels_follow_the_reference_formulas():
    from rohditor_gb300 import clip_levels, opposed_levels

    # sensor.rs:836-865: Opposed ceilings use the as-shot gains, exact f32 arithmetic.
    det, ceiling = opposed_levels(1.2, (2.0, 1.0, 1.55))
    level = np.float32(np.float32(1.2) * np.float32(0.987))
    assert det == (float(level),) * 3
    common = np.float32(level * np.float32(1.0))
    assert ceiling == (float(common / np.float32(2.0)), float(common), float(common / np.float32(1.55)))
    cl = clip_levels(1.0, (2.0, 1.0, 1.6))
    assert cl[1] == float(np.float32(0.987))
