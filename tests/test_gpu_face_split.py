"""Face pass of orders 1 and 2 with Navier-Stokes terms (mfg_set_face_compaction):
writing the solid-side faces in one pass and running the flux branch over a
compacted list of the other faces gives bitwise the states of the single
face kernel, on immersed-boundary and catalyst configurations, through the
level step and through the stand-alone right-hand side."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(case, split, nsteps=2, dt=5e-10):
    lib = abi.load()
    abi.check("mfg_set_face_compaction", lib.mfg_set_face_compaction(int(split)))
    try:
        abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
        lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
        lev.set_state(case.state)
        desc = lev.descriptors()
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for i in range(nsteps):
            abi.check("mfg_advance_level", lib.mfg_advance_level(desc, len(case.boxes), C.byref(case.geom), i * dt,
                                                                 dt, 0, 1, None, st))
        abi.check("mfg_compute_dsdt_flow", lib.mfg_compute_dsdt_flow(desc, len(case.boxes), C.byref(case.geom),
                                                                     nsteps * dt, dt, st))
        torch.cuda.synchronize()
        return lev.get_state(case.shape_zyx), lev.get_state(case.shape_zyx, which="dsdt")
    finally:
        abi.check("mfg_set_face_compaction", lib.mfg_set_face_compaction(1))


@pytest.mark.parametrize("name", ["porous2", "porous1", "cat2", "porous2_uneven"])
def test_face_compaction_is_bitwise_invisible(name):
    if name == "porous2":
        c = perturb(cases.porous_ib(n=32, order=2, max_grid=16), 41, vel_amp=1e-2)
    elif name == "porous1":
        c = perturb(cases.porous_ib(n=24, order=1, max_grid=12), 42, vel_amp=1e-2)
    elif name == "cat2":
        c = perturb(cases.catalyst(n=16, order=2, max_grid=8), 43, vel_amp=1e-2)
    else:
        c = perturb(cases.porous_ib(n=28, order=2, max_grid=12), 44, vel_amp=1e-2)
    on_s, on_d = _run(c, True)
    off_s, off_d = _run(c, False)
    assert np.array_equal(on_s, off_s)
    assert np.array_equal(on_d, off_d)
