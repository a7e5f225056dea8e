"""The reference's own per-cell numerics, built per case plugin by
oracle/ref.mk into oracle/_ref/libref_<case>.so (test infrastructure only),
and the oracle parameter tables that mirror each of those plugins.

A pin case pairs one plugin library with the mfg_params the oracle needs to
compute the same thing: the constants below are the plugin's own values
(species.cpp init(), thermo.H, transport.H, userfuncs.H/.cpp, chemistry.H of
the named case directory), written out as the oracle's tables."""
import ctypes as C
import math
import os
import subprocess

import numpy as np

from mesoflow_gb300 import abi, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ODIR = os.path.join(ROOT, "oracle")
REF_ROOT = os.environ.get("MFLO_REFERENCE", "/root/reference")
RU = cases.RU
PI = 3.14159265358979323846264338327950288  # Source/mflo_constants.H


def available():
    return os.path.isfile(os.path.join(REF_ROOT, "Source", "Src_3d", "compute_flux_3d.H"))


def build():
    r = subprocess.run(["make", "-s", "-j8", "-C", ODIR, "-f", "ref.mk", "REF=" + REF_ROOT],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)


_LIBS = {}


def load(name):
    if name in _LIBS:
        return _LIBS[name]
    build()
    lib = C.CDLL(os.path.join(ODIR, "_ref", f"libref_{name}.so"))
    GP, BP = C.POINTER(abi.Geom), C.POINTER(abi.Box)
    sig = {
        "ref_num_species": [],
        "ref_init": [],
        "ref_compute_dsdt": [GP, BP, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int],
        "ref_cutcells": [GP, BP, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int],
        "ref_chem_source": [GP, BP, C.c_int, C.c_double],
    }
    for k, v in sig.items():
        f = getattr(lib, k)
        f.argtypes = v
        f.restype = C.c_int
    for k in ("ref_molwt", "ref_advect_flag"):
        getattr(lib, k).argtypes = [C.c_int]
        getattr(lib, k).restype = C.c_double
    assert lib.ref_init() == 0
    _LIBS[name] = lib
    return lib


def set_chemistry_on(lib, on):
    """mflo_user_funcs::chemistry_on of the rxnscheme example (userfuncs.cpp:27,
    default 0, read from the inputs file by the reference)."""
    C.c_int.in_dll(lib, "_ZN15mflo_user_funcs12chemistry_onE").value = int(on)


# ---------------------------------------------------------------------------
# oracle tables of each plugin
# ---------------------------------------------------------------------------
def _params(nspec, ngas):
    P = cases._base_params(nspec)
    P.ngas = ngas
    for d in range(3):
        P.bc_lo[d] = P.bc_hi[d] = abi.BC_INT_DIR
    return P


def _set_species(P, W, adv=None):
    for s, w in enumerate(W):
        P.molwt[s] = w
        P.advect_flag[s] = 1.0 if adv is None else adv[s]


def _transport(P, visc, cond, diff, cond_solid=None, diff_solid=None):
    P.visc_mode = abi.TRANSPORT_CONST
    P.visc_gas = visc
    if cond_solid is None:
        P.cond_mode, P.cond_gas = abi.TRANSPORT_CONST, cond
    else:
        P.cond_mode, P.cond_gas, P.cond_solid = abi.TRANSPORT_VFRAC_BLEND, cond, cond_solid
    for s, dv in enumerate(diff):
        if diff_solid is None or diff_solid[s] is None:
            P.diff_mode[s], P.diff_gas[s] = abi.TRANSPORT_CONST, dv
        else:
            P.diff_mode[s], P.diff_gas[s], P.diff_solid[s] = abi.TRANSPORT_VFRAC_BLEND, dv, diff_solid[s]


def plugin_params(name):
    """(params, scales) for a plugin; scales = (rho0, p0, vmag) of the seeded
    states, chosen for the plugin's units."""
    if name == "stube":  # tests/Cartesian/ShockTube_N2
        P = _params(1, 1)
        P.thermo_kind, P.energy_form, P.R_univ = abi.THERMO_MOLAR, abi.EFORM_MASS_CV, 1.0  # userfuncs.cpp:3
        _set_species(P, [0.028])
        P.gamma[0] = 1.4
        _transport(P, 0.0, 0.0, [0.0])
        return P, (1.0, 1.0, 0.3)
    if name == "stubehe":  # tests/Cartesian/ShockTube_N2He
        P = _params(2, 2)
        P.thermo_kind, P.energy_form, P.R_univ = abi.THERMO_MOLAR, abi.EFORM_MASS_CV, RU
        _set_species(P, [0.004, 0.028])
        P.gamma[0], P.gamma[1] = 1.6, 1.4
        _transport(P, 0.0, 0.0, [0.0, 0.0])
        return P, (1.0, 1e5, 50.0)
    if name == "tg":  # tests/Cartesian/TaylorGreen
        P = _params(1, 1)
        P.thermo_kind, P.gas_R, P.gamma_single = abi.THERMO_MASS_SINGLE, 1.0, 1.4
        _set_species(P, [0.0289])
        rho0, v0, L, Re = 1.0, 0.1, 1.0 / PI, 1600.0  # userfuncs.cpp:5-8
        mu = rho0 * v0 * L / Re
        cp = 1.0 * 1.4 / (1.4 - 1.0)
        _transport(P, mu, mu * cp / 0.7, [0.0])
        return P, (1.0, 1.0 / 1.4, 0.1)
    if name == "speq":  # tests/Cartesian/SpeciesEqTests
        P = _params(2, 2)
        P.thermo_kind, P.gas_R, P.gamma_single = abi.THERMO_MASS_SINGLE, 1.0, 1.4
        _set_species(P, [0.032, 0.028], [1.0, 0.0])
        _transport(P, 0.01, 0.0, [0.1, 1.0])
        return P, (1.0, 1.0, 0.5)
    if name == "bcat":  # models/blockCatalyst1d
        P = _params(3, 2)
        P.thermo_kind, P.gas_R, P.gamma_single = abi.THERMO_MASS_SINGLE, 1.0, 1.4
        _set_species(P, [0.032, 0.028, 0.001], [1.0, 1.0, 0.0])
        _transport(P, 0.01, 0.0, [0.5, 1.0, 0.0])
        return P, (1.0, 1.0, 0.5)
    if name == "porous":  # models/porousParticle
        P = _params(1, 1)
        P.thermo_kind, P.gas_R, P.gamma_single = abi.THERMO_MASS_SINGLE, RU / 0.0289, 1.4
        _set_species(P, [0.0289])
        _transport(P, 1e-5, 0.014, [1e-5])
        return P, (1.16, 1e5, 1.0)
    if name == "cht":  # models/conjHtransferTest
        P = _params(2, 1)
        P.thermo_kind, P.gas_R, P.gamma_single = abi.THERMO_MASS_SINGLE, RU / 0.028, 1.4
        _set_species(P, [0.028, 0.07], [0.0, 0.0])
        _transport(P, 0.01, 500.0, [1e-6, 0.0], cond_solid=5000.0)
        return P, (1.16, 1e5, 1.0)
    if name == "catcyl":  # models/catalystCylinder
        P = _params(4, 3)
        P.thermo_kind, P.energy_form, P.R_univ = abi.THERMO_MOLAR, abi.EFORM_MOLAR_CV, RU
        # species.cpp:6 initialises advect_flags[NUM_SPECIES] = {one}: only the
        # first species is advected (init() then zeroes the site species)
        _set_species(P, [0.0289, 0.044, 0.044, 0.001], [1.0, 0.0, 0.0, 0.0])
        for s, g in enumerate([1.4, 1.2, 1.2]):
            P.gamma[s] = g
        _transport(P, 1e-5, 0.01, [1e-5, 1e-5, 1e-4, 0.0], diff_solid=[1e-6, 1e-6, 1e-5, None])
        # chemistry.H: rate = 20 c_S c_A, A -> B on the sites
        P.chem_on, P.nreact = 1, 1
        P.A[0] = 20.0
        P.nu[0][1], P.nu[0][2] = -1.0, 1.0
        P.order[0][1], P.order[0][3] = 1.0, 1.0
        return P, (1.2, 1e5, 1.0)
    if name == "stag":  # models/stagFlowCatalyst
        P = _params(6, 5)
        P.thermo_kind, P.energy_form, P.R_univ = abi.THERMO_MOLAR, abi.EFORM_MOLAR_CV, RU
        # species.cpp:6: advect_flags = {one}, only the first species advected
        _set_species(P, [0.016, 0.032, 0.028, 0.028, 0.018, 0.001], [1.0] + [0.0] * 5)
        for s, g in enumerate([1.2, 1.4, 1.4, 1.2, 1.2]):
            P.gamma[s] = g
        _transport(P, 1e-5, 0.01, [1e-5, 1e-5, 1e-5, 1e-3, 1e-3, 0.0], cond_solid=50.0,
                   diff_solid=[1e-8, 1e-8, 1e-8, 1e-8, 1e-8, None])
        # chemistry.H: 2CH4 + O2 + S -> C2H4 + 2H2O + S, rate = 5 c_S c_CH4 c_O2
        P.chem_on, P.nreact = 1, 1
        P.A[0] = 5.0
        for s, v in ((0, -2.0), (1, -1.0), (3, 1.0), (4, 2.0)):
            P.nu[0][s] = v
        P.order[0][0], P.order[0][1], P.order[0][5] = 1.0, 1.0, 1.0
        return P, (1.0, 1e5, 1.0)
    if name == "rxn":  # py_utils/rxnscheme_writer/example
        P = _params(3, 1)
        P.thermo_kind, P.R_univ, P.bg_molwt = abi.THERMO_BG_GAS, RU, 0.04
        _set_species(P, [0.002, 0.044, 0.0], [1.0, 0.0, 0.0])
        P.gamma[0], P.gamma[1] = 1.4, 1.67
        _transport(P, 2.15e-05, 8.25e-2, [4.27e-5, 0.0, 0.0], diff_solid=[1e-10, None, None])
        P.chem_on, P.nreact = 1, 2  # species.cpp:39-53
        for s, v in enumerate([-1.0, 1.0, -1.0]):
            P.nu[0][s] = v
        for s, v in enumerate([1.0, -1.0, 1.0]):
            P.nu[1][s] = v
        P.order[0][0], P.order[0][2] = 1.0, 1.0
        P.order[1][1] = 1.0
        P.A[0], P.A[1] = 165675000000.0, 16567452390.0
        return P, (1.5, 1e5, 1.0)
    raise KeyError(name)


PLUGINS = ["stube", "stubehe", "tg", "speq", "bcat", "porous", "cht", "catcyl", "stag", "rxn"]


# ---------------------------------------------------------------------------
# seeded states
# ---------------------------------------------------------------------------
def seeded_case(name, seed, vfrac="mixed", n_cell=(12, 10, 8), max_grid=(6, 10, 8)):
    """A periodic case of the plugin with a seeded, non-uniform state:
    densities, pressures and velocities with 20% variations, mass fractions
    from a Dirichlet(2), site species of order one, and the lagged primitive
    components perturbed independently of the conserved ones.  vfrac "ones":
    all gas; "mixed": 55% gas, 15% solid and 30% cut cells in a seeded
    pattern (every immersed-boundary branch of the face and cut-cell code)."""
    P, (rho0, p0, vmag) = plugin_params(name)
    rng = np.random.default_rng(seed)
    nx, ny, nz = n_cell
    shp = (nz, ny, nx)
    u = lambda a=1.0: 1.0 + a * rng.uniform(-1.0, 1.0, size=shp)
    rho = rho0 * u(0.2)
    pres = p0 * u(0.2)
    vel = [vmag * rng.standard_normal(shp) for _ in range(3)]
    ns, ng = P.nspec, P.ngas
    spec = [None] * ns
    Y = np.moveaxis(rng.dirichlet([2.0] * max(ng, 1), size=shp), -1, 0)
    if P.thermo_kind == abi.THERMO_MASS_SINGLE:
        for s in range(ns):
            spec[s] = rho * Y[s % max(ng, 1)] / P.molwt[s]
    elif P.thermo_kind == abi.THERMO_BG_GAS:
        T = 300.0 * u(0.2)
        ctot = pres / (RU * T)
        cgas = 0.3 * ctot
        for s in range(ng):
            spec[s] = cgas * Y[s]
        rho = sum(spec[s] * P.molwt[s] for s in range(ng)) + (ctot - cgas) * P.bg_molwt
    else:
        W = np.array([P.molwt[s] for s in range(ng)])
        for s in range(ng):
            spec[s] = rho * Y[s] / W[s]
    for s in range(ns):
        if spec[s] is None:
            spec[s] = 100.0 * u(0.5)
    if vfrac == "ones":
        vf = np.ones(shp)
    else:
        r = rng.uniform(size=shp)
        vf = np.where(r < 0.55, 1.0, np.where(r < 0.70, 0.0, rng.uniform(0.05, 0.95, size=shp)))
    S = cases.state_from_prim(P, rho, vel[0], vel[1], vel[2], pres, spec, vf)
    for c in (abi.DENS, abi.PRES, abi.TEMP):
        S[c] *= u(0.05)
    for c in (abi.VELX, abi.VELY, abi.VELZ):
        S[c] += 0.1 * vmag * rng.standard_normal(shp)
    return cases.Case("pin_" + name, P, n_cell, (0.0, 0.0, 0.0), (nx * 1e-2, ny * 1.1e-2, nz * 0.9e-2),
                      (1, 1, 1), max_grid, S)


def wrap_sborder(case, level):
    """Every box's Sborder from the periodic domain (np.pad wrap)."""
    g = abi.NGROW
    full = np.pad(case.state, ((0, 0), (g, g), (g, g), (g, g)), mode="wrap")
    for b, (lo, hi) in enumerate(case.boxes):
        sl = tuple(slice(lo[q], hi[q] + 2 * g + 1) for q in (2, 1, 0))
        level.set_sborder(b, full[(slice(None),) + sl])
