"""The allocation-free RHS entry point (mfg_compute_dsdt_flow_noalloc).

It exists for callers that may not allocate device memory while they run --
an AMReX application whose arena has reserved most of the GPU, or a code with
a fixed device-memory budget.  Its scratch is a static array inside the
library.  The test calls it through the C ABI twice in a row (the second call
finds the first call's leftovers in the shared array) and compares both
results with the regular entry point's, at the tolerance of the other parity
tests; it also checks that a box too large for the array is refused.  This
file sorts last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12


def _setup(case):
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = len(case.boxes)
    abi.check("mfg_fill_patch", lib.mfg_fill_patch(lev.descriptors(), n, C.byref(case.geom), 1, 0.0, st))
    return lib, lev, st, n


@pytest.mark.parametrize("make", [
    lambda: perturb(cases.taylor_green_mix(n=32, order=5, max_grid=32), 11, vel_amp=1e-2),
    lambda: perturb(cases.porous_ib(n=32, order=2, max_grid=16), 12, vel_amp=1e-2),
])
def test_noalloc_matches_regular_entry_point_twice(make):
    case = make()
    lib, lev, st, n = _setup(case)
    g = C.byref(case.geom)
    abi.check("mfg_compute_dsdt_flow", lib.mfg_compute_dsdt_flow(lev.descriptors(), n, g, 0.0, 1e-7, st))
    torch.cuda.synchronize()
    ref = lev.get_state(case.shape_zyx, which="dsdt")
    for call in range(2):
        for x in lev.dsdt:
            x.fill_(float("nan"))
        abi.check("mfg_compute_dsdt_flow_noalloc",
                  lib.mfg_compute_dsdt_flow_noalloc(lev.descriptors(), n, g, 0.0, 1e-7, st))
        torch.cuda.synchronize()
        got = lev.get_state(case.shape_zyx, which="dsdt")
        assert np.all(np.isfinite(got)), call
        e, comp = rel_err(got, ref)
        assert e < TOL_STEP, (call, comp, e)


def test_noalloc_rejects_box_larger_than_static_scratch():
    case = cases.taylor_green_mix(n=40, order=5, max_grid=40)
    lib, lev, st, n = _setup(case)
    rc = lib.mfg_compute_dsdt_flow_noalloc(lev.descriptors(), n, C.byref(case.geom), 0.0, 1e-7, st)
    assert rc == abi.ERR_SIZE
