"""Cut-cell cache (mfg_set_cutcell_cache): stored lists and weights give
bitwise the same steps as recomputing them every stage, and a volume
fraction changed between calls is detected on the device (the changed call
recomputes, later calls rebuild the cache) with results equal to the
uncached run."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def run(case, cache, nsteps=3, dt=None, edit=None):
    lib = abi.load()
    abi.check("mfg_set_cutcell_cache", lib.mfg_set_cutcell_cache(int(cache)))
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    desc = lev.descriptors()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if dt is None:
        out = C.c_double()
        abi.check("mfg_est_timestep", lib.mfg_est_timestep(desc, len(case.boxes), C.byref(case.geom), 0.0,
                                                           C.byref(out), st))
        dt = out.value
    for i in range(nsteps):
        if edit is not None and i == edit[0]:
            edit[1](lev)
        abi.check("mfg_advance_level", lib.mfg_advance_level(desc, len(case.boxes), C.byref(case.geom), i * dt, dt,
                                                             0, 1, None, st))
    torch.cuda.synchronize()
    s = lev.get_state(case.shape_zyx)
    abi.check("mfg_set_cutcell_cache", lib.mfg_set_cutcell_cache(1))
    return s, dt


@pytest.mark.parametrize("name", ["porous2", "porous5", "cat5"])
def test_cache_is_bitwise_invisible(name):
    if name == "porous2":
        c = perturb(cases.porous_ib(n=24, order=2, max_grid=12), 6, vel_amp=1e-2)
    elif name == "porous5":
        c = perturb(cases.porous_ib(n=24, order=5, max_grid=12), 7, vel_amp=1e-2)
    else:
        c = perturb(cases.catalyst(n=16, order=5, max_grid=8), 8, vel_amp=1e-2)
    off, dt = run(c, False)
    on, _ = run(c, True, dt=dt)
    again, _ = run(c, True, dt=dt)  # entries built by the previous run are checked and reused
    assert np.array_equal(on, off)
    assert np.array_equal(again, off)


def test_changed_volume_fraction_is_detected():
    c = perturb(cases.porous_ib(n=24, order=2, max_grid=12), 6, vel_amp=1e-2)

    def carve(lev):
        # a new solid sphere in box 0 between steps (s_new's vfrac and its derived cut cells)
        s = lev.s_new[0]
        nz, ny, nx = s.shape[1:]
        z, y, x = torch.meshgrid(torch.arange(nz), torch.arange(ny), torch.arange(nx), indexing="ij")
        r2 = ((x - nx / 2.0) ** 2 + (y - ny / 2.0) ** 2 + (z - nz / 2.0) ** 2).to(s.device, torch.float64)
        v = torch.clamp((r2.sqrt() - 3.0) / 2.0, 0.0, 1.0)
        s[abi.VFRAC] = torch.minimum(s[abi.VFRAC], v)
        torch.cuda.synchronize()

    off, dt = run(c, False, nsteps=4, edit=(2, carve))
    on, _ = run(c, True, nsteps=4, dt=dt, edit=(2, carve))
    assert np.array_equal(on, off)
