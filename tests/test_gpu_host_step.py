"""mfg_advance_level_host: the level step with the state in host memory (each
box copied in, the step, each box copied back on the copy stream as soon as
its last kernels are done) gives bitwise the states and residual norms of
copying in, mfg_advance_level and copying out; a host view whose layout
differs from phi_new's is refused."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def setup(case):
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib, lev, lev.descriptors(), st


@pytest.mark.parametrize("name,pinned", [("porous2", True), ("cat5", True), ("porous2", False)])
def test_host_step_equals_device_step(name, pinned):
    if name == "porous2":
        c = perturb(cases.porous_ib(n=32, order=2, max_grid=16), 11, vel_amp=1e-2)
    else:
        c = perturb(cases.catalyst(n=16, order=5, max_grid=8), 12, vel_amp=1e-2)
    nb = len(c.boxes)
    g = C.byref(c.geom)

    lib, lev, desc, st = setup(c)
    out = C.c_double()
    abi.check("mfg_est_timestep", lib.mfg_est_timestep(desc, nb, g, 0.0, C.byref(out), st))
    dt = out.value
    ref_states, ref_norms = [], []
    for i in range(3):
        rn = (C.c_double * c.ncomp)()
        abi.check("mfg_advance_level", lib.mfg_advance_level(desc, nb, g, i * dt, dt, 0, 1, rn, st))
        ref_states.append([x.cpu().numpy().copy() for x in lev.s_new])
        ref_norms.append(np.array(rn[:]))
    del lev

    lib, lev, desc, st = setup(c)
    host = [torch.empty_like(x, device="cpu") for x in lev.s_new]
    if pinned:
        host = [h.pin_memory() for h in host]
    for h, x in zip(host, lev.s_new):
        h.copy_(x)
        x.zero_()  # the step must take its input from the host arrays
    views = lev.host_views(host)
    for i in range(3):
        rn = (C.c_double * c.ncomp)()
        abi.check("mfg_advance_level_host", lib.mfg_advance_level_host(desc, nb, g, i * dt, dt, 0, 1, views, rn, st))
        for b in range(nb):
            assert np.array_equal(host[b].numpy(), ref_states[i][b]), (i, b)
            assert np.array_equal(lev.s_new[b].cpu().numpy(), ref_states[i][b]), (i, b)
        assert np.array_equal(np.array(rn[:]), ref_norms[i]), i


def test_host_view_layout_mismatch_is_refused():
    c = cases.porous_ib(n=16, order=2, max_grid=8)
    lib, lev, desc, st = setup(c)
    host = [torch.empty_like(x, device="cpu") for x in lev.s_new]
    views = lev.host_views(host)
    views[1].jstride += 1
    rc = lib.mfg_advance_level_host(desc, len(c.boxes), C.byref(c.geom), 0.0, 1e-12, 0, 1, views, None, st)
    assert rc == abi.ERR_ARG
    views = lev.host_views(host)
    views[0].p = None
    rc = lib.mfg_advance_level_host(desc, len(c.boxes), C.byref(c.geom), 0.0, 1e-12, 0, 1, views, None, st)
    assert rc == abi.ERR_ARG
