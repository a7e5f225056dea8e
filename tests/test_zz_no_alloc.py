"""The allocation-free RHS entry point (mfg_compute_dsdt_flow_noalloc).

It exists for callers that may not allocate device memory while they run --
an AMReX application whose arena has reserved most of the GPU, or a code with
a fixed device-memory budget.  Its scratch is a static array inside the
library.  The tests call it through the C ABI:

* on one level, then on another box layout and state (so the shared array
  holds another call's data), then on the first level again: every result
  equals the regular entry point's at the tolerance of the other parity tests;
* in a fresh process with every module loaded at context creation, before
  any regular entry point has run (so the library's scratch pool does not
  exist yet): the device's free memory is the same before and after the call;
* a box too large for the array is refused.

This file sorts last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))


def _setup(case, lib):
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = len(case.boxes)
    abi.check("mfg_fill_patch", lib.mfg_fill_patch(lev.descriptors(), n, C.byref(case.geom), 1, 0.0, st))
    return lev, st, n


def _regular(lib, case, lev, st, n):
    g = C.byref(case.geom)
    abi.check("mfg_compute_dsdt_flow", lib.mfg_compute_dsdt_flow(lev.descriptors(), n, g, 0.0, 1e-7, st))
    torch.cuda.synchronize()
    return lev.get_state(case.shape_zyx, which="dsdt")


def _noalloc(lib, case, lev, st, n):
    for x in lev.dsdt:
        x.fill_(float("nan"))
    abi.check("mfg_compute_dsdt_flow_noalloc",
              lib.mfg_compute_dsdt_flow_noalloc(lev.descriptors(), n, C.byref(case.geom), 0.0, 1e-7, st))
    torch.cuda.synchronize()
    return lev.get_state(case.shape_zyx, which="dsdt")


@pytest.mark.parametrize("kind", ["tg5", "porous2"])
def test_noalloc_matches_regular_entry_point_across_calls(kind):
    if kind == "tg5":
        a = perturb(cases.taylor_green_mix(n=32, order=5, max_grid=32), 11, vel_amp=1e-2)
        b = perturb(cases.taylor_green_mix(n=32, order=5, max_grid=16), 13, vel_amp=2e-2)
    else:
        a = perturb(cases.porous_ib(n=32, order=2, max_grid=16), 12, vel_amp=1e-2)
        b = perturb(cases.porous_ib(n=32, order=2, max_grid=32, seed=9), 14, vel_amp=2e-2)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(a.params)))  # a and b share their parameter tables
    la, lb = _setup(a, lib), _setup(b, lib)
    ref_a, ref_b = _regular(lib, a, *la), _regular(lib, b, *lb)
    for case, lev, ref in ((a, la, ref_a), (b, lb, ref_b), (a, la, ref_a)):
        got = _noalloc(lib, case, *lev, )
        assert np.all(np.isfinite(got))
        e, comp = rel_err(got, ref)
        assert e < TOL_STEP, (case.name, comp, e)


FRESH = r"""
import ctypes as C, sys
sys.path[:0] = [{root!r}, {here!r}]
import numpy as np, torch
from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb
import ref_lib
torch.cuda.init()
case = perturb(cases.taylor_green_mix(n=32, order=5, max_grid=16), 15, vel_amp=1e-2)
lib = abi.load()
assert lib.mfg_init(C.byref(case.params)) == 0
lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
lev.set_state(case.state)
ref_lib.wrap_sborder(case, lev)
st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
rc = lib.mfg_compute_dsdt_flow_noalloc(lev.descriptors(), len(case.boxes), C.byref(case.geom), 0.0, 1e-7, st)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
d = lev.get_state(case.shape_zyx, which="dsdt")
print("RESULT", rc, free0, free1, int(np.isfinite(d).all()), float(np.abs(d).max()))
"""


def test_noalloc_allocates_nothing_in_a_fresh_process():
    """CUDA_MODULE_LOADING=EAGER loads the library's modules (and its static
    array) when the context is created, so the call itself may change the
    device's free memory only by allocating -- which it must not."""
    root = os.path.dirname(HERE)
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    r = subprocess.run([sys.executable, "-c", FRESH.format(root=root, here=HERE)], capture_output=True, text=True,
                       env=env, timeout=600)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT")]
    assert r.returncode == 0 and line, r.stdout + r.stderr
    _, rc, free0, free1, finite, mx = line[0].split()
    assert int(rc) == abi.OK
    assert int(free0) == int(free1), (free0, free1)
    assert int(finite) == 1 and float(mx) > 0


def test_noalloc_rejects_box_larger_than_static_scratch():
    case = cases.taylor_green_mix(n=40, order=5, max_grid=40)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev, st, n = _setup(case, lib)
    rc = lib.mfg_compute_dsdt_flow_noalloc(lev.descriptors(), n, C.byref(case.geom), 0.0, 1e-7, st)
    assert rc == abi.ERR_SIZE
