"""Case set-ups: parameter tables (the reference's per-case plugin headers and
inputs files as mfg_params) and seeded synthetic initial states.

Cases
  sod               tests/Cartesian/ShockTube_N2 (single species N2, R_univ = 1)
  taylor_green_mix  3D Taylor-Green vortex (tests/Cartesian/TaylorGreen/Prob.H
                    velocity field) in a 5-species calorically perfect mixture
  porous_ib         pressure-driven flow through a seeded sphere pack, immersed
                    boundary (models/porousParticle pattern)
  catalyst          catalyst block with surface reactions (models/stagFlowCatalyst /
                    rxnscheme example pattern)
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .level import chop, geometry

RU = 8.31446261815324


def _base_params(nspec):
    p = abi.Params()
    C.memset(C.byref(p), 0, C.sizeof(p))
    p.nspec = nspec
    p.ngas = nspec
    p.R_univ = RU
    p.order_hyp = 2           # Source/mflo.H:241
    p.dissfactor = 0.5
    p.do_ns = 1
    p.species_in_solid = 1
    p.solid_temp = 300.0
    p.cfl = 0.7
    for s in range(nspec):
        p.advect_flag[s] = 1.0
    for d in range(3):
        p.bc_lo[d] = abi.BC_FOEXTRAP
        p.bc_hi[d] = abi.BC_FOEXTRAP
    return p


# ---------------------------------------------------------------------------
# host thermodynamics for building initial states (numpy, vectorised)
# ---------------------------------------------------------------------------
def temperature(P_, rho, pres, spec):
    """get_t_from_rpc of the case's thermo family."""
    if P_.thermo_kind == abi.THERMO_MASS_SINGLE:
        return pres / P_.gas_R / rho
    if P_.thermo_kind == abi.THERMO_BG_GAS:
        sum_ci = sum(spec[s] for s in range(P_.ngas))
        sum_cm = sum(spec[s] * P_.molwt[s] for s in range(P_.ngas))
        return pres / ((sum_ci + (rho - sum_cm) / P_.bg_molwt) * RU)
    sum_ci = sum(spec[s] for s in range(P_.ngas))
    return pres / (sum_ci * P_.R_univ)


def energy(P_, rho, pres, spec):
    """get_e_from_rpc of the case's thermo family (specific internal energy)."""
    if P_.thermo_kind == abi.THERMO_MASS_SINGLE:
        return pres / (P_.gamma_single - 1.0) / rho
    T = temperature(P_, rho, pres, spec)
    if P_.thermo_kind == abi.THERMO_BG_GAS:
        sum_cm = sum(spec[s] * P_.molwt[s] for s in range(P_.ngas))
        cbg = (rho - sum_cm) / P_.bg_molwt
        scv = sum(RU / (P_.gamma[s] - 1.0) * spec[s] for s in range(P_.ngas))
        scv = scv + RU / (P_.gamma[P_.ngas] - 1.0) * cbg
        return scv * T / rho
    if P_.energy_form == abi.EFORM_MASS_CV:
        sum_ci = sum(spec[s] for s in range(P_.ngas))
        cvbar = sum(P_.R_univ / (P_.gamma[s] - 1.0) / P_.molwt[s] * (spec[s] / sum_ci) for s in range(P_.ngas))
        return cvbar * T
    scv = sum(P_.R_univ / (P_.gamma[s] - 1.0) * spec[s] for s in range(P_.ngas))
    return scv * T / rho


def state_from_prim(P_, rho, u, v, w, pres, spec, vfrac):
    """Full state (ncomp, Z, Y, X) from primitive fields (as the cases' initdata)."""
    ns = P_.nspec
    shp = np.shape(rho)
    S = np.zeros((abi.FLO_NVARS + ns,) + shp)
    S[abi.DENS], S[abi.VELX], S[abi.VELY], S[abi.VELZ], S[abi.PRES] = rho, u, v, w, pres
    S[abi.VFRAC] = vfrac
    for s in range(ns):
        S[abi.FLO_NVARS + s] = spec[s]
    S[abi.TEMP] = temperature(P_, rho, pres, spec)
    S[abi.RHO] = rho
    S[abi.RHOU], S[abi.RHOV], S[abi.RHOW] = rho * u, rho * v, rho * w
    S[abi.RHOE] = rho * energy(P_, rho, pres, spec) + 0.5 * rho * (u * u + v * v + w * w)
    return S


class Case:
    """Parameters, geometry, box layout and initial state of one configuration."""

    def __init__(self, name, params, n_cell, prob_lo, prob_hi, periodic, max_grid, state, meta=None):
        self.name = name
        self.params = params
        self.n_cell = tuple(n_cell)
        self.domain_lo = (0, 0, 0)
        self.domain_hi = tuple(n - 1 for n in n_cell)
        self.geom = geometry(self.domain_lo, self.domain_hi, prob_lo, prob_hi, periodic)
        self.boxes = chop(self.domain_lo, self.domain_hi, max_grid)
        self.state = state
        self.meta = meta or {}

    @property
    def ncomp(self):
        return abi.FLO_NVARS + self.params.nspec

    @property
    def shape_zyx(self):
        return (self.n_cell[2], self.n_cell[1], self.n_cell[0])


def _centers(n_cell, prob_lo, prob_hi):
    ax = []
    for d in range(3):
        dx = (prob_hi[d] - prob_lo[d]) / n_cell[d]
        ax.append(prob_lo[d] + (np.arange(n_cell[d]) + 0.5) * dx)
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return X, Y, Z


# ---------------------------------------------------------------------------
def sod(n_cell=(256, 4, 4), order=5, max_grid=64, axis=0):
    """Sod shock tube along `axis` (tests/Cartesian/ShockTube_N2: N2, gamma 1.4,
    R_univ = 1 because inputs_x sets prob.R_univ while userfuncs.cpp reads
    prob.univr).  Left rho=1, p=1; right rho=0.125, p=0.1.  Outflow (foextrap)
    along the tube, periodic across."""
    P = _base_params(1)
    P.thermo_kind = abi.THERMO_MOLAR
    P.energy_form = abi.EFORM_MASS_CV
    P.R_univ = 1.0
    P.molwt[0] = 0.028
    P.gamma[0] = 1.4
    P.order_hyp = order
    P.cfl = 0.5
    for d in range(3):
        P.bc_lo[d] = abi.BC_FOEXTRAP if d == axis else abi.BC_INT_DIR
        P.bc_hi[d] = abi.BC_FOEXTRAP if d == axis else abi.BC_INT_DIR
    n_cell = list(n_cell)
    if axis != 0:
        n_cell[0], n_cell[axis] = n_cell[axis], n_cell[0]
    prob_hi = [0.125, 0.125, 0.125]
    prob_hi[axis] = 1.0
    X, Y, Z = _centers(n_cell, (0, 0, 0), prob_hi)
    xa = (X, Y, Z)[axis]
    left = xa < 0.5
    rho = np.where(left, 1.0, 0.125)
    pres = np.where(left, 1.0, 0.1)
    spec = [rho / 0.028]
    zero = np.zeros_like(rho)
    S = state_from_prim(P, rho, zero, zero, zero, pres, spec, np.ones_like(rho))
    periodic = [d != axis for d in range(3)]
    return Case("sod", P, n_cell, (0, 0, 0), prob_hi, periodic, max_grid, S, {"axis": axis})


def species_eq(n=32, max_grid=16, axis=0):
    """tests/Cartesian/SpeciesEqTests: the flow is frozen (solve_navier_stokes
    = 0) at rho = p = 1 (mass-single thermo, R = 1, gamma 1.4) with unit
    velocity along `axis`; S1 is advected and diffused (D = 0.1) between the
    boundary values 0 and 1, S2 is only diffused (D = 1, advect flag 0) with a
    unit source and zero boundary values (ext_dir faces whose ghost species
    are reflected about the value, externbc.H; walls across).  Steady state:
    S1 = (exp(x/0.1) - 1)/(exp(10) - 1), S2 = x(1 - x)/2."""
    P = _base_params(2)
    P.thermo_kind = abi.THERMO_MASS_SINGLE
    P.gas_R = 1.0
    P.gamma_single = 1.4
    P.ngas = 2
    P.molwt[0], P.molwt[1] = 0.032, 0.028
    P.advect_flag[0], P.advect_flag[1] = 1.0, 0.0
    for s, D in enumerate((0.1, 1.0)):
        P.diff_mode[s] = abi.TRANSPORT_CONST
        P.diff_gas[s] = D
    P.visc_gas = 0.01
    P.cond_gas = 0.0
    P.do_ns = 0
    P.cfl = 0.8
    P.chem_on = 1
    P.nreact = 1
    P.nu[0][1] = 1.0       # S2 source 1: a reaction with no reactants and rate constant 1
    P.A[0] = 1.0
    for d in range(3):
        if d == axis:
            P.bc_lo[d] = P.bc_hi[d] = abi.BC_EXT_DIR
        else:
            P.bc_lo[d] = P.bc_hi[d] = abi.BC_WALL
    for e, (s1, s2) in ((P.ext_lo[axis], (0.0, 0.0)), (P.ext_hi[axis], (1.0, 0.0))):
        e.kind = abi.EXT_SPECIES_DIRICHLET
        e.spec[0], e.spec[1] = s1, s2
    n_cell = [4, 4, 4]
    n_cell[axis] = n
    prob_hi = [0.125, 0.125, 0.125]
    prob_hi[axis] = 1.0
    shape = (n_cell[2], n_cell[1], n_cell[0])
    one = np.ones(shape)
    zero = np.zeros(shape)
    vel = [zero, zero, zero]
    vel[axis] = one
    S = state_from_prim(P, one, vel[0], vel[1], vel[2], one, [zero, zero], one)
    return Case("species_eq", P, n_cell, (0, 0, 0), prob_hi, (0, 0, 0), max_grid, S, {"axis": axis})


def block_catalyst_1d(n=32, max_grid=16, l1=0.7):
    """models/blockCatalyst1d: frozen flow at rho = p = 1 (mass-single, R = 1,
    gamma 1.4); gas for x < l1 with unit velocity, a catalyst block beyond
    (vfrac by 8-corner sampling, velocity 0 where vfrac < 1, site
    concentration 1 - vfrac); S1 (D = 0.5) is 1 at x = 0 and 0 at x = 1, S2
    (D = 1) has zero gradient at both ends, site species not transported; the
    surface reaction S1 + site -> S2 + site with rate 5 [site][S1].  Steady S1:
    the piecewise analytic solution of verify_spec.py."""
    P = _base_params(3)
    P.thermo_kind = abi.THERMO_MASS_SINGLE
    P.gas_R = 1.0
    P.gamma_single = 1.4
    P.ngas = 2
    for s, (W, adv, D) in enumerate(((0.032, 1.0, 0.5), (0.028, 1.0, 1.0), (0.001, 0.0, 0.0))):
        P.molwt[s], P.advect_flag[s] = W, adv
        P.diff_mode[s] = abi.TRANSPORT_CONST
        P.diff_gas[s] = D
    P.visc_gas = 0.01
    P.cond_gas = 0.0
    P.do_ns = 0
    P.species_in_solid = 1
    P.cfl = 0.8
    P.chem_on = 1
    P.nreact = 1
    P.nu[0][0], P.nu[0][1] = -1.0, 1.0
    P.order[0][0], P.order[0][2] = 1.0, 1.0
    P.A[0] = 5.0
    P.bc_lo[0] = P.bc_hi[0] = abi.BC_EXT_DIR
    for d in (1, 2):
        P.bc_lo[d] = P.bc_hi[d] = abi.BC_WALL
    for e, s1 in ((P.ext_lo[0], 1.0), (P.ext_hi[0], 0.0)):
        e.kind = abi.EXT_SPECIES_DIRICHLET
        e.spec[0] = s1
        e.spec_zero_grad_mask = 0b010   # S2 zero gradient
        e.vfrac_interior = 1
    n_cell = (n, 4, 4)
    prob_hi = (1.0, 0.125, 0.125)
    dx = 1.0 / n
    xc = np.arange(n + 1) * dx                                  # cell corners along x
    frac = np.array([0.5 * (float(xc[i] < l1) + float(xc[i + 1] < l1)) for i in range(n)])
    shape = (4, 4, n)
    vf = np.broadcast_to(frac, shape).copy()
    one = np.ones(shape)
    zero = np.zeros(shape)
    u = np.where(vf < 1.0, 0.0, 1.0)
    spec = [zero, zero, 1.0 - vf]
    S = state_from_prim(P, one, u, zero, zero, one, spec, vf)
    return Case("block_catalyst_1d", P, n_cell, (0, 0, 0), prob_hi, (0, 0, 0), max_grid, S, {"l1": l1})


def taylor_green_mix(n=256, order=5, max_grid=64, seed=20261203, v0=10.0):
    """3D Taylor-Green vortex on [-1,1]^3 (velocity of tests/Cartesian/TaylorGreen/
    Prob.H) plus 1% Gaussian noise, in a 5-species calorically perfect molar
    mixture at p = 1e5 Pa, T = 300 K with mass fractions ~ Dirichlet(2) per cell.
    mu = rho0 v0 L / Re (Re = 1600, TaylorGreen/userfuncs.H), k = mu cp / Pr,
    D_k = 1e-5.  Periodic."""
    ns = 5
    P = _base_params(ns)
    P.thermo_kind = abi.THERMO_MOLAR
    P.energy_form = abi.EFORM_MOLAR_CV
    W = [0.028, 0.032, 0.044, 0.018, 0.040]
    G = [1.4, 1.4, 1.3, 1.33, 1.67]
    for s in range(ns):
        P.molwt[s], P.gamma[s] = W[s], G[s]
        P.diff_gas[s] = 1e-5
    mu = 1.0 * v0 * 1.0 / 1600.0
    P.visc_gas = mu
    P.cond_gas = mu * 1000.0 / 0.7
    P.order_hyp = order
    P.cfl = 0.4
    for d in range(3):
        P.bc_lo[d] = P.bc_hi[d] = abi.BC_INT_DIR
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    X, Y, Z = _centers((n, n, n), (-1, -1, -1), (1, 1, 1))
    pi = math.pi
    u = v0 * np.sin(pi * X) * np.cos(pi * Y) * np.cos(pi * Z)
    v = -v0 * np.cos(pi * X) * np.sin(pi * Y) * np.cos(pi * Z)
    w = np.zeros(shape)
    u = u + 0.01 * v0 * rng.standard_normal(shape)
    v = v + 0.01 * v0 * rng.standard_normal(shape)
    w = w + 0.01 * v0 * rng.standard_normal(shape)
    Yk = rng.dirichlet([2.0] * ns, size=shape)  # (Z,Y,X,ns)
    Yk = np.moveaxis(Yk, -1, 0)
    pres = np.full(shape, 1e5)
    T = 300.0
    sum_y_w = sum(Yk[s] / W[s] for s in range(ns))
    rho = pres / (RU * T * sum_y_w)
    spec = [rho * Yk[s] / W[s] for s in range(ns)]
    S = state_from_prim(P, rho, u, v, w, pres, spec, np.ones(shape))
    return Case("taylor_green_mix", P, (n, n, n), (-1, -1, -1), (1, 1, 1), (1, 1, 1), max_grid, S)


def sphere_pack_vfrac(n, seed, solid_frac, rmin=4.0, rmax=12.0, smooth=True):
    """Fluid volume fraction of a seeded random pack of overlapping spheres
    (radii uniform in [rmin, rmax] cells, centres uniform in the domain), grown
    until the solid fraction of the cell corners reaches solid_frac; 8-corner
    sampling as the reference's initdata (tests/ImmBoundary/subsonicCylinder/
    Prob.H:39-59), then a 2-cell box filter (one 3-point average per axis:
    the 8-corner ramp of one cell widens to about two) and snapping of values within 1e-3 of 0 or 1, so that pure cells
    stay exactly 0 or 1."""
    rng = np.random.default_rng(seed)
    nn = n + 1
    ax = np.arange(nn, dtype=np.float64)
    solid_c = np.zeros((nn, nn, nn), dtype=bool)  # corner (k, j, i) inside a sphere
    nsolid, target = 0, solid_frac * nn ** 3
    while nsolid < target:
        c = rng.uniform(0, n, size=3)
        r = rng.uniform(rmin, rmax)
        lo = np.maximum(np.floor(c - r).astype(int), 0)
        hi = np.minimum(np.ceil(c + r).astype(int) + 1, nn)
        if np.any(hi <= lo):
            continue
        dz = (ax[lo[2]:hi[2]] - c[2])[:, None, None] ** 2
        dy = (ax[lo[1]:hi[1]] - c[1])[None, :, None] ** 2
        dx = (ax[lo[0]:hi[0]] - c[0])[None, None, :] ** 2
        inside = (dz + dy + dx) <= r * r
        sl = (slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0]))
        nsolid += int(np.count_nonzero(inside & ~solid_c[sl]))
        solid_c[sl] |= inside
    fluid = (~solid_c).astype(np.float64)
    vf = 0.125 * sum(fluid[kk:kk + n, jj:jj + n, ii:ii + n] for kk in (0, 1) for jj in (0, 1) for ii in (0, 1))
    if smooth:
        for axis in range(3):
            pad = [(0, 0)] * 3
            pad[axis] = (1, 1)
            q = np.pad(vf, pad, mode="edge")
            sl = [slice(None)] * 3
            acc = 0.0
            for o in range(3):
                sl[axis] = slice(o, o + n)
                acc = acc + q[tuple(sl)]
            vf = acc / 3.0
        vf[vf >= 0.999] = 1.0
        vf[vf <= 0.001] = 0.0
    return vf


def porous_ib(n=256, order=2, max_grid=64, seed=3, solid_frac=0.4, dx=2e-6, p_out=1e5, dp_rel=1e-3):
    """Pressure-driven flow through a seeded sphere pack (models/porousParticle
    pattern): air (W = 0.0289, gamma 1.4, p = rho R_air T), mu = 1e-5,
    k = 0.014, D = 1e-5, species_in_solid = 0, cfl 0.1; x: pressure inlet
    p_in = (1 + dp_rel) p_out / pressure outlet p_out (ext_dir), y/z: walls."""
    P = _base_params(1)
    P.thermo_kind = abi.THERMO_MASS_SINGLE
    W = 0.0289
    P.molwt[0] = W
    P.gamma[0] = 1.4
    P.gamma_single = 1.4
    P.gas_R = RU / W
    P.visc_gas = 1e-5
    P.cond_gas = 0.014
    P.diff_gas[0] = 1e-5
    P.species_in_solid = 0
    P.order_hyp = order
    P.cfl = 0.1  # models/porousParticle/inputs (mflo.cfl); 0.4 per direction is unstable in 3D
    T = 300.0
    p_in = p_out * (1.0 + dp_rel)
    rho_in = p_in / (P.gas_R * T)
    P.bc_lo[0] = P.bc_hi[0] = abi.BC_EXT_DIR
    for d in (1, 2):
        P.bc_lo[d] = P.bc_hi[d] = abi.BC_WALL
    P.ext_lo[0].kind = abi.EXT_PRESSURE_INLET
    P.ext_lo[0].dens = rho_in
    P.ext_lo[0].pres = p_in
    P.ext_lo[0].spec[0] = rho_in / W
    P.ext_hi[0].kind = abi.EXT_PRESSURE_OUTLET
    P.ext_hi[0].pres = p_out
    vf = sphere_pack_vfrac(n, seed, solid_frac)
    shape = (n, n, n)
    rho = np.full(shape, p_out / (P.gas_R * T))
    zero = np.zeros(shape)
    S = state_from_prim(P, rho, zero, zero, zero, np.full(shape, p_out), [rho / W], vf)
    L = n * dx
    return Case("porous_ib", P, shape, (0, 0, 0), (L, L, L), (0, 0, 0), max_grid, S,
                {"p_in": p_in, "p_out": p_out, "mu": 1e-5})


def permeability(case, state):
    """Darcy permeability k = mu <u_x>_superficial L_x / dp (superficial
    velocity: the volume average of rho u_x / rho over all cells, solid = 0)."""
    m = case.meta
    rho = state[abi.RHO]
    ux = np.where(state[abi.VFRAC] > 0, state[abi.RHOU] / np.where(rho > 0, rho, 1.0), 0.0) * state[abi.VFRAC]
    Lx = case.n_cell[0] * case.geom.dx[0]
    return m["mu"] * float(ux.mean()) * Lx / (m["p_in"] - m["p_out"])


def catalyst(n=128, order=5, max_grid=32, seed=4, nreact=8, solid_frac=0.3, block=True, u_in=1.0, dx=1e-5,
             arrhenius=True, bg_gas=False):
    """Catalyst block with explicit surface chemistry (models/stagFlowCatalyst /
    rxnscheme example pattern): 8 gas species + 2 non-advected site species
    (molar mixture, R = RU); mass-action surface reactions gas_a + site_b ->
    gas_c + site_d with log10 A ~ U[3, 8] and Ea ~ U[40, 120] kJ/mol (seeded),
    or the reference's table form (Ea = 0) when arrhenius is False.
    Diffusivities blend gas/solid with vfrac; species_in_solid = 1.
    x: velocity inlet u_in / outflow (foextrap); y, z: walls.  The immersed
    solid is a block in the middle third plus a seeded sphere pack.
    bg_gas: the background-gas thermo family (rxnscheme example thermo.H): an
    untracked inert gas (W = 0.028, gamma 1.4) holds 70% of the moles and the
    tracked gases share the rest."""
    ng, nsite = 8, 2
    ns = ng + nsite
    P = _base_params(ns)
    P.thermo_kind = abi.THERMO_MOLAR
    P.energy_form = abi.EFORM_MOLAR_CV
    P.ngas = ng
    rng = np.random.default_rng(seed)
    W = [0.028, 0.032, 0.044, 0.018, 0.002, 0.016, 0.030, 0.026]
    G = [1.4, 1.4, 1.3, 1.33, 1.41, 1.31, 1.4, 1.3]
    for s in range(ng):
        P.molwt[s], P.gamma[s] = W[s], G[s]
        P.diff_mode[s] = abi.TRANSPORT_VFRAC_BLEND
        P.diff_gas[s] = 1e-5 * (1.0 + s / ng)
        P.diff_solid[s] = 1e-6 * (1.0 + s / ng)
    for s in range(ng, ns):
        P.molwt[s] = 0.001
        P.advect_flag[s] = 0.0
        P.diff_mode[s] = abi.TRANSPORT_CONST
        P.diff_gas[s] = 0.0
    P.visc_gas = 2.15e-5
    P.cond_gas = 8.25e-2
    P.species_in_solid = 1
    P.order_hyp = order
    P.cfl = 0.4
    P.chem_on = 1
    P.nreact = nreact
    for r in range(nreact):
        a, c = rng.choice(ng, size=2, replace=False)
        b = ng + r % nsite
        d = ng + (r + 1) % nsite
        P.nu[r][a] = -1.0
        P.nu[r][b] += -1.0
        P.nu[r][c] += 1.0
        P.nu[r][d] += 1.0
        P.order[r][a] = 1.0
        P.order[r][b] = 1.0
        P.A[r] = 10.0 ** rng.uniform(3.0, 8.0)
        P.Ea[r] = rng.uniform(40e3, 120e3) if arrhenius else 0.0
    T, pres = 500.0, 1e5
    x = np.array([0.7, 0.1, 0.05, 0.05, 0.04, 0.03, 0.02, 0.01])
    ctot = pres / (RU * T)
    cbg = 0.0
    if bg_gas:
        P.thermo_kind = abi.THERMO_BG_GAS
        P.bg_molwt = 0.028
        P.gamma[ng] = 1.4
        cbg = 0.7 * ctot
        x = 0.3 * x
    cg = x * ctot
    rho_in = float(sum(cg[s] * W[s] for s in range(ng))) + cbg * P.bg_molwt
    P.bc_lo[0] = abi.BC_EXT_DIR
    P.bc_hi[0] = abi.BC_FOEXTRAP
    for d in (1, 2):
        P.bc_lo[d] = P.bc_hi[d] = abi.BC_WALL
    e = P.ext_lo[0]
    e.kind = abi.EXT_VELOCITY_INLET
    e.dens = rho_in
    e.pres = pres
    e.vel[0] = u_in
    for s in range(ng):
        e.spec[s] = cg[s]
    shape = (n, n, n)
    vf = sphere_pack_vfrac(n, seed + 1, solid_frac * 0.5, rmin=max(2.0, n / 64), rmax=max(4.0, n / 20))
    if block:
        X, Y, Z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        inb = (Z >= n // 3) & (Z < 2 * n // 3) & (Y >= n // 4) & (Y < 3 * n // 4) & (X >= n // 4) & (X < 3 * n // 4)
        vf = np.where(inb.transpose(0, 1, 2), np.minimum(vf, 0.0), vf)  # (z, y, x) indexing == (X, Y, Z) names here
        vf = np.clip(vf, 0.0, 1.0)
    spec = [np.full(shape, cg[s]) for s in range(ng)]
    site = np.where(vf < 1.0, 50.0, 0.0)
    spec += [site * 0.6, site * 0.4]
    rho = sum(spec[s] * W[s] for s in range(ng)) + cbg * P.bg_molwt
    u = np.where(vf == 1.0, u_in, 0.0)
    zero = np.zeros(shape)
    S = state_from_prim(P, rho, u, zero, zero, np.full(shape, pres), spec, vf)
    L = n * dx
    return Case("catalyst", P, shape, (0, 0, 0), (L, L, L), (0, 0, 0), max_grid, S, {"u_in": u_in})


# ---------------------------------------------------------------------------
# multi-level catalyst hierarchy (batched AMR form)
# ---------------------------------------------------------------------------
class Geometry:
    """Analytic catalyst geometry in physical units: one axis-aligned solid block
    plus seeded spheres; fluid volume fraction by 8-corner sampling of any cell
    box at any resolution (as the reference's initdata, Prob.H:39-59)."""

    def __init__(self, L, seed, nspheres=24, block=(0.35, 0.65, 0.3, 0.7, 0.3, 0.7), rmin=0.03, rmax=0.07):
        rng = np.random.default_rng(seed)
        self.L = L
        self.block = np.array(block) * L
        self.c = rng.uniform(0.15, 0.85, size=(nspheres, 3)) * L
        self.r = rng.uniform(rmin, rmax, size=nspheres) * L

    def vfrac(self, lo, hi, dx):
        """vfrac of cells lo..hi (inclusive) on a grid of spacing dx, shape (z, y, x)."""
        ax = [np.arange(lo[d], hi[d] + 2) * dx for d in range(3)]  # corner coordinates
        Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        b = self.block
        solid = (X >= b[0]) & (X <= b[1]) & (Y >= b[2]) & (Y <= b[3]) & (Z >= b[4]) & (Z <= b[5])
        bl = np.array([lo[d] * dx for d in range(3)])
        bh = np.array([(hi[d] + 1) * dx for d in range(3)])
        for c, r in zip(self.c, self.r):
            if np.any(c + r < bl) or np.any(c - r > bh):
                continue
            solid |= (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r
        f = (~solid).astype(np.float64)
        return 0.125 * sum(f[kk:kk + f.shape[0] - 1, jj:jj + f.shape[1] - 1, ii:ii + f.shape[2] - 1]
                           for kk in (0, 1) for jj in (0, 1) for ii in (0, 1))


def _merge_blocks(tag, blk, max_blocks):
    """Greedy merge of tagged blocks (bool array over block indices (z, y, x))
    into boxes of at most max_blocks blocks per side; returns block-index boxes."""
    used = np.zeros_like(tag)
    out = []
    nz, ny, nx = tag.shape
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if not tag[z, y, x] or used[z, y, x]:
                    continue
                x1 = x
                while x1 + 1 < nx and x1 + 1 - x < max_blocks and tag[z, y, x1 + 1] and not used[z, y, x1 + 1]:
                    x1 += 1
                y1 = y
                while (y1 + 1 < ny and y1 + 1 - y < max_blocks and tag[z, y1 + 1, x:x1 + 1].all()
                       and not used[z, y1 + 1, x:x1 + 1].any()):
                    y1 += 1
                z1 = z
                while (z1 + 1 < nz and z1 + 1 - z < max_blocks and tag[z1 + 1, y:y1 + 1, x:x1 + 1].all()
                       and not used[z1 + 1, y:y1 + 1, x:x1 + 1].any()):
                    z1 += 1
                used[z:z1 + 1, y:y1 + 1, x:x1 + 1] = True
                out.append(((x * blk, y * blk, z * blk), ((x1 + 1) * blk - 1, (y1 + 1) * blk - 1, (z1 + 1) * blk - 1)))
    return out


class AmrCase:
    """Levels of boxes (uneven sizes), per-level geometry and per-box initial states."""

    def __init__(self, params, geoms, boxes, states, meta):
        self.params = params
        self.geoms = geoms            # list of abi.Geom, one per level
        self.boxes = boxes            # list of (lo, hi, level)
        self.states = states          # per box (ncomp, nz, ny, nx)
        self.meta = meta

    @property
    def ncomp(self):
        return abi.FLO_NVARS + self.params.nspec

    def cells(self):
        return sum(int(np.prod([h[d] - l[d] + 1 for d in range(3)])) for l, h, _ in self.boxes)


def catalyst_amr(n0=128, nlev=3, order=5, seed=4, blocking=16, max_grid=64, base_grid=32, u_in=1.0, dx0=1e-5,
                 nspheres=80, nreact=8, nested=True):
    """Catalyst block + spheres on 3 levels (ratio 2, base n0^3): level l+1
    covers the level-l cells within 2 cells of the immersed surface (cut cells
    and their neighbours), clustered into blocks of `blocking` cells and merged
    into uneven boxes of up to max_grid cells per side (a stand-in for AMReX's
    regrid, which is not vendored).  Chemistry, species and boundaries as
    catalyst(): 8 gas + 2 site species, 8 Arrhenius surface reactions.
    nested: level l+1 keeps one block of level-l cells around it (inside the
    domain), so that its ghost cells and their interpolation stencils lie on
    level l (proper nesting, which the multi-level step needs when
    blocking/2 >= 3)."""
    base = catalyst(n=8, order=order, seed=seed, nreact=nreact, u_in=u_in, dx=dx0)  # parameter tables only
    P = base.params
    L = n0 * dx0
    geo = Geometry(L, seed, nspheres=nspheres)
    geoms, boxes = [], []
    # level 0: the whole domain in base_grid boxes
    lev_boxes = [((lo[0], lo[1], lo[2]), (hi[0], hi[1], hi[2])) for lo, hi in
                 chop((0, 0, 0), (n0 - 1, n0 - 1, n0 - 1), base_grid)]
    for l in range(nlev):
        n = n0 * 2 ** l
        geoms.append(geometry((0, 0, 0), (n - 1,) * 3, (0, 0, 0), (L, L, L), (0, 0, 0)))
        boxes += [(lo, hi, l) for lo, hi in lev_boxes]
        if l + 1 == nlev:
            break
        dx = L / n
        # tag cells of this level near the surface, in fine-block units
        nb = (2 * n) // blocking
        tag = np.zeros((nb, nb, nb), dtype=bool)
        inside = np.zeros((nb, nb, nb), dtype=bool)
        for lo, hi in lev_boxes:
            vf = geo.vfrac(lo, hi, dx)
            cut = (vf > 0) & (vf < 1)
            g = np.zeros_like(cut)
            for ax in range(3):  # grow the cut band by 2 cells
                for s in (-2, -1, 1, 2):
                    g |= np.roll(cut, s, axis=ax)
            g |= cut
            zz, yy, xx = np.nonzero(g)
            fz = ((zz + lo[2]) * 2) // blocking
            fy = ((yy + lo[1]) * 2) // blocking
            fx = ((xx + lo[0]) * 2) // blocking
            tag[fz, fy, fx] = True
            # fine blocks that lie inside this coarse box (proper nesting)
            bz0, by0, bx0 = (2 * lo[2]) // blocking, (2 * lo[1]) // blocking, (2 * lo[0]) // blocking
            bz1, by1, bx1 = (2 * (hi[2] + 1)) // blocking, (2 * (hi[1] + 1)) // blocking, (2 * (hi[0] + 1)) // blocking
            inside[bz0:bz1, by0:by1, bx0:bx1] = True
        if nested:  # erode the covered region by one block; outside the domain counts as covered
            pad = np.pad(inside, 1, constant_values=True)
            er = np.ones_like(inside)
            for dz in (0, 1, 2):
                for dy in (0, 1, 2):
                    for dx_ in (0, 1, 2):
                        er &= pad[dz:dz + nb, dy:dy + nb, dx_:dx_ + nb]
            inside = er
        tag &= inside
        lev_boxes = _merge_blocks(tag, blocking, max_grid // blocking)
    # initial states: gas at rest except the inlet velocity in fluid cells, sites in solid cells
    W = [P.molwt[s] for s in range(P.ngas)]
    T, pres = 500.0, 1e5
    x = np.array([0.7, 0.1, 0.05, 0.05, 0.04, 0.03, 0.02, 0.01])
    cg = x * pres / (RU * T)
    states = []
    for lo, hi, l in boxes:
        dx = L / (n0 * 2 ** l)
        vf = geo.vfrac(lo, hi, dx)
        shape = vf.shape
        spec = [np.full(shape, cg[s]) for s in range(P.ngas)]
        site = np.where(vf < 1.0, 50.0, 0.0)
        spec += [site * 0.6, site * 0.4]
        rho = sum(spec[s] * W[s] for s in range(P.ngas))
        u = np.where(vf == 1.0, u_in, 0.0)
        zero = np.zeros(shape)
        states.append(state_from_prim(P, rho, u, zero, zero, np.full(shape, pres), spec, vf))
    meta = {"nlev": nlev, "per_level_boxes": [sum(1 for b in boxes if b[2] == l) for l in range(nlev)]}
    return AmrCase(P, geoms, boxes, states, meta)


def two_level(case, fine_boxes, ratio=2):
    """Two-level hierarchy over a single-level case: level 0 is the case's
    boxes, level 1 the given boxes (inclusive fine-index corners, aligned to
    the ratio), initialised by piecewise-constant injection of the coarse
    state."""
    g0 = case.geom
    n = [g0.domain_hi[d] - g0.domain_lo[d] + 1 for d in range(3)]
    prob_lo = [g0.prob_lo[d] for d in range(3)]
    prob_hi = [g0.prob_lo[d] + n[d] * g0.dx[d] for d in range(3)]
    per = [g0.is_periodic[d] for d in range(3)]
    g1 = geometry((0, 0, 0), tuple(ratio * n[d] - 1 for d in range(3)), prob_lo, prob_hi, per)
    boxes, states = [], []
    for lo, hi in case.boxes:
        boxes.append((tuple(lo), tuple(hi), 0))
        states.append(np.ascontiguousarray(case.state[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]))
    for lo, hi in fine_boxes:
        assert all(lo[d] % ratio == 0 and (hi[d] + 1) % ratio == 0 for d in range(3))
        c = case.state[:, lo[2] // ratio:(hi[2] + 1) // ratio, lo[1] // ratio:(hi[1] + 1) // ratio,
                       lo[0] // ratio:(hi[0] + 1) // ratio]
        f = c.repeat(ratio, axis=1).repeat(ratio, axis=2).repeat(ratio, axis=3)
        boxes.append((tuple(lo), tuple(hi), 1))
        states.append(np.ascontiguousarray(f))
    meta = dict(case.meta)
    meta.update({"nlev": 2, "per_level_boxes": [len(case.boxes), len(fine_boxes)]})
    return AmrCase(case.params, [g0, g1], boxes, states, meta)
