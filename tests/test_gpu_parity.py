"""GPU parity: the CUDA library (through its C ABI) against the oracle on the
same seeded inputs.  Tolerances (per cell and component, relative to the
component's domain maximum): 1e-12 for one RHS / one RK3 step, 1e-10 (L2)
after several steps; ghost fill and pure copies are bit-exact."""
import ctypes as C

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
from mesoflow_gb300.level import Level
from helpers import perturb, rel_err
from oracle_run import OracleLevel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12
TOL_L2 = 1e-10


def small(name):
    if name == "sod5":
        return perturb(cases.sod(n_cell=(48, 8, 8), order=5, max_grid=16), 1)
    if name == "sod2":
        return perturb(cases.sod(n_cell=(48, 8, 8), order=2, max_grid=16), 2)
    if name == "sod1":
        return perturb(cases.sod(n_cell=(48, 8, 8), order=1, max_grid=16), 3)
    if name == "sod4":
        return perturb(cases.sod(n_cell=(48, 8, 8), order=4, max_grid=16), 4)
    if name == "tg5":
        return perturb(cases.taylor_green_mix(n=16, order=5, max_grid=8), 5, vel_amp=1e-2)
    if name == "porous2":
        return perturb(cases.porous_ib(n=24, order=2, max_grid=12), 6, vel_amp=1e-2)
    if name == "porous5":
        return perturb(cases.porous_ib(n=24, order=5, max_grid=12), 7, vel_amp=1e-2)
    if name == "cat5":
        return perturb(cases.catalyst(n=16, order=5, max_grid=8), 8, vel_amp=1e-2)
    if name == "cat2":
        return perturb(cases.catalyst(n=16, order=2, max_grid=8), 9, vel_amp=1e-2)
    if name == "speq":  # frozen flow (no Navier-Stokes terms), species Dirichlet ends, a constant source
        c = cases.species_eq(n=32, max_grid=8)
        rng = np.random.default_rng(11)
        c.state[abi.FLO_NVARS:abi.FLO_NVARS + 2] = rng.uniform(0.0, 1.0, size=(2,) + c.state.shape[1:])
        return c
    if name == "bcat1d":  # immersed block, surface reaction, species boundary values, no Navier-Stokes terms
        c = cases.block_catalyst_1d(n=32, max_grid=8)
        rng = np.random.default_rng(12)
        c.state[abi.FLO_NVARS:abi.FLO_NVARS + 2] = rng.uniform(0.0, 1.0, size=(2,) + c.state.shape[1:])
        return c
    if name == "catbg5":
        return perturb(cases.catalyst(n=16, order=5, max_grid=8, bg_gas=True), 10, vel_amp=1e-2)
    raise KeyError(name)


NAMES = ["sod5", "sod2", "sod1", "sod4", "tg5", "porous2", "porous5", "cat5", "cat2", "catbg5", "speq", "bcat1d"]


class Gpu:
    def __init__(self, case):
        self.lib = abi.load()
        self.case = case
        abi.check("mfg_init", self.lib.mfg_init(C.byref(case.params)))
        self.level = Level(case.boxes, case.ncomp, backend="torch", device="cuda", with_flux=True)
        self.level.set_state(case.state)
        self.desc = self.level.descriptors()
        self.st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.n = len(case.boxes)
        self.g = C.byref(case.geom)

    def sync(self):
        torch.cuda.synchronize()


def oracle_for(case):
    return OracleLevel(case, with_flux=True)


def fill_both(o, g, src=1):
    lib = o.lib
    assert lib.oracle_fill_patch(C.byref(o.case.params), C.byref(o.case.geom), o.desc, len(o.case.boxes), src, 0.0) == 0
    abi.check("mfg_fill_patch", g.lib.mfg_fill_patch(g.desc, g.n, g.g, src, 0.0, g.st))
    g.sync()


@pytest.mark.parametrize("name", NAMES)
def test_fill_patch_bitwise(name):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    fill_both(o, g)
    for b in range(len(c.boxes)):
        ob = o.level.sborder_host(b)
        gb = g.level.sborder_host(b)
        assert np.array_equal(np.nan_to_num(ob), np.nan_to_num(gb)) or rel_err(gb, ob)[0] < 1e-15, b


@pytest.mark.parametrize("name", ["porous2", "porous5", "cat5", "catbg5"])
def test_cutcells(name):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    fill_both(o, g)
    assert o.lib.oracle_cutcells(C.byref(c.params), C.byref(c.geom), o.desc, len(c.boxes)) == 0
    abi.check("mfg_cutcells", g.lib.mfg_cutcells(g.desc, g.n, g.g, 0.0, g.st))
    g.sync()
    for b in range(len(c.boxes)):
        e, comp = rel_err(g.level.sborder_host(b), o.level.sborder_host(b))
        assert e < TOL_STEP, (b, comp, e)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("fast", [1, 0])
def test_dsdt_parity(name, fast):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    g.lib.mfg_set_weno_mode(fast)
    fill_both(o, g)
    # the GPU works on the oracle's ghost-filled state
    for b in range(len(c.boxes)):
        g.level.set_sborder(b, o.level.sborder_host(b))
    assert o.lib.oracle_compute_dsdt(C.byref(c.params), C.byref(c.geom), o.desc, len(c.boxes)) == 0
    abi.check("mfg_compute_dsdt_flow", g.lib.mfg_compute_dsdt_flow(g.desc, g.n, g.g, 0.0, 1e-6, g.st))
    g.sync()
    g.lib.mfg_set_weno_mode(1)
    od = o.level.get_state(c.shape_zyx, which="dsdt")
    gd = g.level.get_state(c.shape_zyx, which="dsdt")
    e, comp = rel_err(gd, od)
    assert e < TOL_STEP, (comp, e)
    # face fluxes for reflux
    for b in range(len(c.boxes)):
        for d in range(3):
            of = o.level.flux[b][d]
            gf = g.level.flux[b][d].cpu().numpy()
            e, comp = rel_err(gf, of)
            assert e < TOL_STEP, (b, d, comp, e)


@pytest.mark.parametrize("name", NAMES)
def test_one_step_parity(name):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    dt = o.est_timestep()
    ro = o.advance(dt)
    rg = (C.c_double * c.ncomp)()
    abi.check("mfg_advance_level", g.lib.mfg_advance_level(g.desc, g.n, g.g, 0.0, dt, 0, 1, rg, g.st))
    so, sg = o.state(), g.level.get_state(c.shape_zyx)
    e, comp = rel_err(sg, so)
    assert e < TOL_STEP, (comp, e)
    # residual norms measure (S_new - S_old)/dt: the state tolerance, carried
    # through that difference, bounds them
    rg = np.array(rg[:])
    scale = np.array([np.linalg.norm(so[q]) for q in range(c.ncomp)]) / dt
    assert np.all(np.abs(rg - ro) <= 1e-9 * np.abs(ro) + TOL_STEP * scale)


@pytest.mark.parametrize("name", ["sod5", "tg5", "porous2", "cat5", "catbg5", "speq", "bcat1d"])
def test_multistep_l2(name):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    for step in range(8):
        dt = o.est_timestep()
        o.advance(dt)
        abi.check("mfg_advance_level", g.lib.mfg_advance_level(g.desc, g.n, g.g, o.time - dt, dt, 0, 1, None, g.st))
    so, sg = o.state(), g.level.get_state(c.shape_zyx)
    for comp in range(c.ncomp):
        den = np.linalg.norm(so[comp])
        if den > 0:
            assert np.linalg.norm(sg[comp] - so[comp]) / den < TOL_L2, comp


@pytest.mark.parametrize("name", ["cat5", "catbg5"])
def test_chemistry_parity(name):
    c = small(name)
    o, g = oracle_for(c), Gpu(c)
    # chemistry sub-step alone: s_old -> s_new
    o.level.set_state(c.state, which="old")
    g.level.set_state(c.state, which="old")
    dt = 1e-7
    assert o.lib.oracle_chem_substep(C.byref(c.params), o.desc, len(c.boxes), dt) == 0
    abi.check("mfg_chem_substep", g.lib.mfg_chem_substep(g.desc, g.n, g.g, 0.0, dt, g.st))
    g.sync()
    e, comp = rel_err(g.level.get_state(c.shape_zyx), o.state())
    assert e < TOL_STEP, (comp, e)


def test_est_timestep_and_prims():
    c = small("tg5")
    o, g = oracle_for(c), Gpu(c)
    out = C.c_double()
    abi.check("mfg_est_timestep", g.lib.mfg_est_timestep(g.desc, g.n, g.g, 0.0, C.byref(out), g.st))
    assert abs(out.value - o.est_timestep()) <= 1e-14 * o.est_timestep()
    assert o.lib.oracle_update_primitive_vars(C.byref(c.params), o.desc, len(c.boxes)) == 0
    abi.check("prims", g.lib.mfg_update_primitive_vars(g.desc, g.n, g.g, g.st))
    e, comp = rel_err(g.level.get_state(c.shape_zyx), o.state())
    assert e < TOL_STEP, (comp, e)


def test_nan_sets_status_and_error():
    c = cases.sod(n_cell=(32, 4, 4), order=5, max_grid=32)
    c.state[abi.RHOE, 0, 0, 5] = np.nan
    g = Gpu(c)
    v = C.c_uint32()
    g.lib.mfg_status(C.byref(v), 1)
    rc = g.lib.mfg_advance_level(g.desc, g.n, g.g, 0.0, 1e-4, 0, 1, None, g.st)
    assert rc == abi.ERR_NAN
    g.lib.mfg_status(C.byref(v), 1)
    assert v.value & abi.STATUS_NAN


def test_bad_box_rejected():
    c = cases.sod(n_cell=(32, 4, 4), order=5, max_grid=32)
    g = Gpu(c)
    d = (abi.Box * 1)()
    d[0] = g.desc[0]
    d[0].sborder.begin[0] += 1  # ghost region no longer covered
    assert g.lib.mfg_compute_dsdt_flow(d, 1, g.g, 0.0, 1e-6, g.st) == abi.ERR_ARG


def test_species_equations_reach_the_analytic_steady_state():
    """The GPU on tests/Cartesian/SpeciesEqTests run to t = 1 (its own dt
    sequence): the same bounds as the oracle's run against x(1-x)/2 and the
    upwind scheme's steady state (tests/test_cpu_oracle.py)."""
    from mesoflow_gb300.driver import Mflo
    c = cases.species_eq(n=32)
    g = Mflo(c, device="cuda")
    while g.time < 1.0 - 1e-12:
        g.advance(g.compute_dt(stop_time=1.0), norms=False)
    s = g.state()
    x = (np.arange(32) + 0.5) / 32
    e2 = 0.5 * (x - x * x)
    deff = 0.1 + 0.5 / 32
    e1m = (np.exp(x / deff) - 1) / (np.exp(1 / deff) - 1)
    assert np.abs(s[abi.FLO_NVARS + 1][2, 2, :] - e2).max() < 2e-3 * e2.max()
    assert np.abs(s[abi.FLO_NVARS][2, 2, :] - e1m).max() < 1e-2


def test_block_catalyst_reaches_the_analytic_steady_state():
    """The GPU on models/blockCatalyst1d run to t = 1.35: S1 within 0.025 of
    the piecewise analytic solution, as the oracle (tests/test_cpu_oracle.py)."""
    from mesoflow_gb300.driver import Mflo
    from test_cpu_oracle import _block_catalyst_exact
    c = cases.block_catalyst_1d(n=32)
    g = Mflo(c, device="cuda")
    while g.time < 1.35 - 1e-12:
        g.advance(g.compute_dt(stop_time=1.35), norms=False)
    x = (np.arange(32) + 0.5) / 32
    assert np.abs(g.state()[abi.FLO_NVARS][2, 2, :] - _block_catalyst_exact(x)).max() < 0.025
