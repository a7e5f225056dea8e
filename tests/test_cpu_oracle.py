"""CPU suite: the oracle pinned to the reference's fixtures and analytic
solutions, the C ABI layout, and the CUDA library's exported symbols."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mesoflow_gb300 import abi, cases
import oracle_lib
import riemann
from oracle_run import OracleLevel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SOD = os.path.join(os.environ.get("MFLO_REFERENCE", "/root/reference"), "tests", "Cartesian", "ShockTube_N2",
                       "exact_soln")


def test_abi_layout_matches_c():
    lib = oracle_lib.load()
    buf = (C.c_int64 * 32)()
    m = lib.oracle_abi_layout(buf, 32)
    want = [C.sizeof(abi.Array4), C.sizeof(abi.Box), C.sizeof(abi.Geom), C.sizeof(abi.ExtBC),
            C.sizeof(abi.Params), abi.Box.flux.offset, abi.Box.level.offset, abi.Params.order_hyp.offset,
            abi.Params.nu.offset, abi.Params.bc_lo.offset, abi.Params.ext_hi.offset, abi.ExtBC.state.offset,
            abi.Params.cfl.offset]
    assert list(buf[:m]) == want


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "mflo_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mfg_[a-z0-9_]+)\s*\(", txt)))


def test_library_builds_loads_and_exports_header_symbols():
    from mesoflow_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    names = header_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    # every binding in abi.SIGNATURES is declared in the header
    assert {s[0] for s in abi.SIGNATURES} <= set(names)


@pytest.mark.skipif(not os.path.exists(REF_SOD), reason="reference fixture not mounted")
def test_exact_riemann_solver_matches_reference_fixture():
    ref = np.loadtxt(REF_SOD, skiprows=1)  # x, p, rho, T, u at t = 0.1, diaphragm at 0
    mine = riemann.sample(ref[:, 0], 0.1, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1)
    # the fixture samples the discontinuities at finite resolution: compare away from them
    for col, row in ((2, 0), (4, 1), (1, 2)):
        d = np.abs(mine[row] - ref[:, col])
        assert np.median(d) < 1e-6
        assert np.mean(d < 1e-3) > 0.99


@pytest.mark.parametrize("order,tol", [(5, 0.008), (2, 0.012)])
def test_oracle_sod_converges_to_exact(order, tol):
    c = cases.sod(n_cell=(128, 4, 4), order=order, max_grid=32)
    o = OracleLevel(c)
    while o.time < 0.1 - 1e-12:
        o.advance(o.compute_dt(stop_time=0.1))
    rho = o.state()[abi.RHO][0, 0, :]
    x = (np.arange(128) + 0.5) / 128 - 0.5
    ex = riemann.sample(x, 0.1, 1, 0, 1, 0.125, 0, 0.1)
    assert np.abs(rho - ex[0]).mean() < tol
    # uniform across the periodic directions
    S = o.state()
    assert np.all(S[abi.RHO] == S[abi.RHO][:1, :1, :])


def test_oracle_sod_orientation_invariance():
    """x, y and z tubes give the same profile (the reference runs inputs_x/y/z)."""
    prof = []
    for axis in range(3):
        c = cases.sod(n_cell=(64, 4, 4), order=5, max_grid=32, axis=axis)
        o = OracleLevel(c)
        for _ in range(10):
            o.advance(2e-3)
        r = o.state()[abi.RHO]
        prof.append(r[0, 0, :] if axis == 0 else (r[0, :, 0] if axis == 1 else r[:, 0, 0]))
    assert np.max(np.abs(prof[0] - prof[1])) < 1e-13
    assert np.max(np.abs(prof[0] - prof[2])) < 1e-13


def test_oracle_conserves_mass_periodic():
    c = cases.taylor_green_mix(n=12, order=5, max_grid=6)
    o = OracleLevel(c)
    m0 = c.state[abi.RHO].sum()
    for _ in range(2):
        o.advance(2e-6)
    m1 = o.state()[abi.RHO].sum()
    assert abs(m1 - m0) / m0 < 1e-13


def test_oracle_box_decomposition_invariance():
    """Fluxes are computed once per face from the ghost-filled state, so the
    result does not depend on how the domain is chopped into boxes."""
    a = cases.taylor_green_mix(n=12, order=5, max_grid=12)
    b = cases.taylor_green_mix(n=12, order=5, max_grid=4)
    oa, ob = OracleLevel(a), OracleLevel(b)
    oa.advance(2e-6)
    ob.advance(2e-6)
    assert np.array_equal(oa.state(), ob.state())


def test_oracle_nan_reports_status():
    c = cases.sod(n_cell=(32, 4, 4), order=5, max_grid=32)
    c.state[abi.RHOE, 0, 0, 5] = np.nan
    o = OracleLevel(c)
    with pytest.raises(abi.MfloError) as e:
        o.advance(1e-3)
    assert e.value.code == abi.ERR_NAN


def test_oracle_two_level_step_conserves_composite_totals():
    """Subcycled two-level step on a periodic box (no immersed boundary, no
    chemistry): with the flux registers, reflux and average-down, the
    composite totals of mass, momentum, energy and species are conserved to
    rounding, although the fine level takes two substeps and its ghost cells
    come from time-interpolated conservative interpolation."""
    from oracle_run import OracleAmr
    c = cases.taylor_green_mix(n=12, order=5, max_grid=6)
    amr = cases.two_level(c, [((4, 4, 4), (11, 15, 15)), ((12, 4, 4), (19, 11, 11))])
    o = OracleAmr(amr)
    comps = [abi.RHO, abi.RHOU, abi.RHOV, abi.RHOW, abi.RHOE] + [abi.FLO_NVARS + s for s in range(c.params.nspec)]
    t0, a0 = o.composite_totals(comps)
    for _ in range(2):
        o.advance(2e-6, only_flow=True, clip=False)
    t1, _ = o.composite_totals(comps)
    assert np.all(np.abs(t1 - t0) <= 1e-13 * a0), (t1 - t0) / a0
    # the covered coarse cells hold the average of the fine cells
    fine = o.box_state(len(c.boxes))
    avg = fine.reshape(fine.shape[0], 6, 2, 6, 2, 4, 2).mean(axis=(2, 4, 6))  # coarse z, y 2..7, x 2..5
    crse = o.box_state(0)  # coarse box 0 holds coarse cells 0..5 in each direction
    # (conserved components: the primitive refresh after the step recomputes the others)
    assert np.allclose(crse[comps, 2:6, 2:6, 2:6], avg[comps, 0:4, 0:4, 0:4], rtol=1e-14, atol=0)


def _stiff_decay_case(k=1e10):
    """Catalyst layout with one reaction A -> B, first order in A, rate k."""
    c = cases.catalyst(n=8, order=5, max_grid=8)
    P = c.params
    P.nreact = 1
    for s in range(abi.MAX_SPECIES):
        P.nu[0][s] = 0.0
        P.order[0][s] = 0.0
    P.nu[0][0], P.nu[0][1], P.order[0][0] = -1.0, 1.0, 1.0
    P.A[0], P.Ea[0] = k, 0.0
    return c


def test_oracle_ros2_stiff_decay():
    """The implicit (ROS2) chemistry of the oracle on A -> B with k dt = 1e4
    (explicit RK3 is unstable beyond k dt ~ 2.5): A decays to nothing (the
    method is L-stable), A + B is conserved to rounding (Rosenbrock stages
    keep linear invariants), and the adaptive steps resolve the transient."""
    c = _stiff_decay_case()
    o = OracleLevel(c)
    lev = o.level
    lev.s_old[0][...] = lev.s_new[0]
    a0, b0 = lev.s_new[0][abi.FLO_NVARS].copy(), lev.s_new[0][abi.FLO_NVARS + 1].copy()
    rc = o.lib.oracle_chem_substep_ros2(C.byref(c.params), o.desc, 1, 1e-6, 1e-3, 1e-6, 2000)
    assert rc == 0
    a1, b1 = lev.s_new[0][abi.FLO_NVARS], lev.s_new[0][abi.FLO_NVARS + 1]
    assert np.all(np.abs(a1) <= 1e-6 * a0.max())
    assert np.allclose(a1 + b1, a0 + b0, rtol=1e-13, atol=0)
    # at k dt = 0.5 the result matches exp(-k dt) to the tolerance
    c = _stiff_decay_case(k=5e5)
    o = OracleLevel(c)
    o.level.s_old[0][...] = o.level.s_new[0]
    a0 = o.level.s_new[0][abi.FLO_NVARS].copy()
    assert o.lib.oracle_chem_substep_ros2(C.byref(c.params), o.desc, 1, 1e-6, 1e-6, 1e-12, 2000) == 0
    assert np.allclose(o.level.s_new[0][abi.FLO_NVARS], a0 * np.exp(-0.5), rtol=2e-5, atol=0)


def _species_eq_exact(n):
    x = (np.arange(n) + 0.5) / n
    return x, (np.exp(x / 0.1) - 1) / (np.exp(10.0) - 1), 0.5 * (x - x * x)


def test_oracle_species_equations_reach_the_analytic_steady_state():
    """tests/Cartesian/SpeciesEqTests (its inputs_x, externbc.H, chemistry.H,
    verify_spec.py): frozen flow, S1 advected (u = 1) and diffused (D = 0.1)
    between 0 and 1, S2 diffused (D = 1) with a unit source, run to t = 1 with
    CFL 0.8 on 32 cells.  S2 matches x(1-x)/2 to 0.2% of its maximum.  S1 is
    advected first-order upwind (the scalar MUSCL call takes its states by
    value, compute_flux_3d.H:403), so it matches the exact solution of that
    scheme's modified equation (D + u dx/2) to 1e-2 and the continuous one to
    5e-2."""
    c = cases.species_eq(n=32)
    o = OracleLevel(c)
    while o.time < 1.0 - 1e-12:
        o.advance(o.compute_dt(stop_time=1.0))
    s = o.state()
    x, e1, e2 = _species_eq_exact(32)
    s1 = s[abi.FLO_NVARS][2, 2, :]
    s2 = s[abi.FLO_NVARS + 1][2, 2, :]
    assert np.abs(s2 - e2).max() < 2e-3 * e2.max()
    deff = 0.1 + 0.5 / 32
    e1m = (np.exp(x / deff) - 1) / (np.exp(1 / deff) - 1)
    assert np.abs(s1 - e1m).max() < 1e-2
    assert np.abs(s1 - e1).max() < 5e-2
    # the frozen flow stays as initialised
    assert np.array_equal(s[abi.RHO], c.state[abi.RHO]) and np.array_equal(s[abi.RHOU], c.state[abi.RHOU])


def _block_catalyst_exact(x, v=1.0, D=0.5, k=5.0, l1=0.7, l=1.0):
    """The piecewise steady solution of models/blockCatalyst1d/verify_spec.py
    (advection-diffusion in the gas, diffusion-reaction in the catalyst, flux
    continuity at l1), restated."""
    w = np.sqrt(k / D)
    F = 1 / (np.exp(v * l1 / D) - 1)
    A = v * (1 + F) / (v * F * (np.exp(w * l1) - np.exp(w * (2 * l - l1))) -
                       D * w * (np.exp(w * l1) + np.exp(w * (2 * l - l1))))
    B = -A * np.exp(2 * w * l)
    c1 = (A * np.exp(w * l1) + B * np.exp(-w * l1) - 1) * F
    return np.where(x < l1, c1 * (np.exp(v * x / D) - 1) + 1, A * np.exp(w * x) + B * np.exp(-w * x))


def test_oracle_block_catalyst_reaches_the_analytic_steady_state():
    """models/blockCatalyst1d (inputs_x, Prob.H, chemistry.H, externbc.H,
    verify_spec.py): gas with unit velocity up to x = 0.7, a catalyst block
    beyond (cut cell at the interface), surface reaction S1 + site -> S2 +
    site, run to t = 1.35: S1 within 0.025 of the piecewise analytic solution
    on 32 cells (first-order upwind advection, one cut cell)."""
    c = cases.block_catalyst_1d(n=32)
    o = OracleLevel(c)
    while o.time < 1.35 - 1e-12:
        o.advance(o.compute_dt(stop_time=1.35))
    x = (np.arange(32) + 0.5) / 32
    s1 = o.state()[abi.FLO_NVARS][2, 2, :]
    assert np.abs(s1 - _block_catalyst_exact(x)).max() < 0.025
