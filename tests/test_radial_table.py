"""The library's host build of the radial multiplier table against the oracle's,
bit for bit, on the CPU (rd_optics_radial_table is host-only code).

rd_spatial remaps through this table whenever the build accepts it
(crates/optics/src/correction.rs:110-181), so its knots, step, pinned freeze
boundaries and refusal decision must be the reference's. The lens models and
sizes are those of the oracle tests plus the 24 MP workload's frame.
"""

import ctypes

import numpy as np
import pytest

from test_oracle import RADIAL_LENSES

GUARDS = {-1: "no table", 0: "accepted", 1: "non-finite", 2: "tripwire", 3: "break collision",
          4: "freeze ambiguity", 5: "unexplained jump"}
MODELS = {0: "none", 1: "poly3", 2: "poly5", 3: "ptlens"}
TCA = {0: "none", 1: "linear", 2: "poly3"}


def product_table(desc):
    from rohditor_gb300 import _ffi

    knots = np.zeros((1024, 4), dtype=np.float32)
    step = ctypes.c_float(0.0)
    guard = ctypes.c_int32(0)
    rc = _ffi.load().rd_optics_radial_table(ctypes.byref(desc), knots.ctypes.data_as(_ffi.F32P),
                                            ctypes.byref(step), ctypes.byref(guard))
    assert rc == 0
    return GUARDS[guard.value], step.value, knots


@pytest.mark.parametrize("size", [(97, 61), (320, 213), (1536, 1024), (6048, 4024)])
@pytest.mark.parametrize("name", sorted(RADIAL_LENSES))
def test_library_table_build_equals_the_oracle(oracle, name, size):
    from rohditor_gb300 import OpticsExecution

    (dm, dk, tm, red, blue), _ = RADIAL_LENSES[name]
    ex = OpticsExecution(size[0], size[1], distortion=MODELS[dm], distortion_k=dk, tca=TCA[tm], tca_red=red,
                         tca_blue=blue)
    desc = ex.to_c()
    guard, step, knots = product_table(desc)
    ref_guard, ref_step, ref_table, ref_pins = oracle.optics_radial(oracle.optics_desc_from(desc))
    assert guard == ref_guard
    assert np.float32(step) == np.float32(ref_step)
    assert np.array_equal(knots[:, :3].view(np.uint32), ref_table.view(np.uint32))
    pinned = [(i, float(knots[i, 3])) for i in range(1024) if not np.isnan(knots[i, 3])]
    assert pinned == ref_pins  # a collision keeps the first flip of its segment in both builds
