"""Split-chemistry driver pieces (mflo::Evolve_split, Source/mflo_splitchem.cpp):
the midpoint chemistry step with the reference's phi_old/phi_new swap, the
background-gas store, the post-chemistry variable update, and the whole
split loop, against the oracle on the catalyst case (molar and
background-gas thermo)."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.driver import Mflo
from mesoflow_gb300.level import Level
from helpers import perturb, rel_err
from oracle_run import OracleLevel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bg", [False, True])
def test_split_pieces_match_oracle(bg):
    c = perturb(cases.catalyst(n=16, order=5, max_grid=8, bg_gas=bg), 11, vel_amp=1e-2)
    o = OracleLevel(c)
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(c.params)))
    lev = Level(c.boxes, c.ncomp, backend="torch", device="cuda")
    lev.set_state(c.state)
    desc, n = lev.descriptors(), len(c.boxes)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = C.byref(c.params)
    dt = o.est_timestep()
    o.advance(dt, only_flow=True)  # s_old = the state before this flow step
    abi.check("adv", lib.mfg_advance_level(desc, n, C.byref(c.geom), 0.0, dt, 1, 1, None, st))
    if bg:
        assert o.lib.oracle_store_inertgas_conc(P, o.desc, n) == 0
        abi.check("store", lib.mfg_store_inertgas_conc(desc, n, st))
    for q in range(3):
        assert o.lib.oracle_chem_advance_rk2(P, o.desc, n, 1e-7) == 0
        abi.check("rk2", lib.mfg_chem_advance_rk2(desc, n, q * 1e-7, 1e-7, st))
    torch.cuda.synchronize()
    for which in ("new", "old"):
        e, comp = rel_err(lev.get_state(c.shape_zyx, which=which), o.level.get_state(c.shape_zyx, which=which))
        assert e <= 1e-12, (which, comp, e)
    # the chemistry changed the species
    assert not np.array_equal(lev.get_state(c.shape_zyx)[abi.FLO_NVARS:], c.state[abi.FLO_NVARS:])
    assert o.lib.oracle_update_vars_after_chemsolve(P, o.desc, n, int(bg)) == 0
    abi.check("vars", lib.mfg_update_vars_after_chemsolve(desc, n, int(bg), st))
    e, comp = rel_err(lev.get_state(c.shape_zyx), o.state())
    assert e <= 1e-12, (comp, e)


@pytest.mark.parametrize("bg", [False, True])
def test_evolve_split_matches_oracle(bg):
    """The whole split loop (flow to steady state, chemistry sub-steps on the
    frozen flow, variable update, flow again), both sides on the same dt."""
    c = perturb(cases.catalyst(n=16, order=5, max_grid=8, bg_gas=bg), 12, vel_amp=1e-2)
    o = OracleLevel(c)
    dt = o.est_timestep()
    g = Mflo(c, device="cuda")
    o.compute_dt = lambda stop_time=1e300: dt
    g.compute_dt = lambda stop_time=1e300: dt
    args = (3 * dt, 4e-7, 2e-7, 1e-7, 2 * dt)
    o.evolve_split(*args, bg_inertgas=bg)
    g.evolve_split(*args, bg_inertgas=bg)
    assert g.istep == 7 and abs(g.time - o.time) <= 1e-12 * o.time
    so, sg = o.state(), g.state()
    for comp in range(c.ncomp):
        den = np.linalg.norm(so[comp])
        if den > 0:
            assert np.linalg.norm(sg[comp] - so[comp]) / den < 1e-10, comp
