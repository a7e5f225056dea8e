"""The oracle pinned to the reference's own code, bit for bit.

oracle/ref.mk compiles the reference's per-cell numerics
(Source/Src_3d/compute_flux_3d.H, flux_schemes.H, consprim_funcs.H, div_3d.H,
ib_utils.H) and each case's plugin sources unmodified against a small AMReX
stand-in; oracle/ref_driver.cpp runs the box bodies of compute_dsdt_flow,
update_cutcell_data and compute_dsdt_chemistry over the same mfg_box
descriptors the oracle takes.  Every test below runs both on the same seeded
state and requires equal bits: every face flux and every dsdt value
(compute_flux + update_residual), every Sborder value after update_cutcells,
and the reaction source of the table-form chemistry.

Coverage: orders 1, 2, 4 (the truncated twelveth, Q9) and 5; Navier-Stokes
and the species-only branch (the by-value scalar limiter, Q2, the
spec_in_solid face velocity weights that both read the left cell, Q3, the
4-cell species stencil against the 6-cell immersed-boundary fallback, Q10);
the immersed-boundary fallback and solid-side faces (mixed volume fractions);
volume-fraction-blended conductivity, whose harmonic mean reads cell i-1 in
every sweep direction (Q1); multi-species eigenvalues with the left state's
species in the right pressure (Q4); the conjugate-heat-transfer residual mask
and the in-place 26-neighbour temperature of cut cells (Q7); all three
thermo families (molar with the mass- or molar-cv energy, single gas,
background gas) in every plugin of the reference that defines one.

The tests that build the libraries need the reference checkout
(the MFLO_REFERENCE variable, else ref_lib's default) and are skipped without it; the
golden-fixture test needs only the oracle.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from mesoflow_gb300 import abi
from mesoflow_gb300.level import Level
import oracle_lib
import ref_lib

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

needs_ref = pytest.mark.skipif(not ref_lib.available(), reason="reference checkout not present")


def _pair(name, seed, vfrac, with_flux=True):
    case = ref_lib.seeded_case(name, seed, vfrac=vfrac)
    levels = []
    for _ in range(2):
        lev = Level(case.boxes, case.ncomp, backend="numpy", with_flux=with_flux)
        lev.set_state(case.state)
        ref_lib.wrap_sborder(case, lev)
        levels.append(lev)
    return case, levels[0], levels[1]


def _bitwise(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        idx = np.argwhere(~same)[0]
        raise AssertionError(f"{what}: {int((~same).sum())} values differ, first at {tuple(idx)}: "
                             f"oracle {a[tuple(idx)]!r} reference {b[tuple(idx)]!r}")


def _dsdt_case(name, seed, vfrac, order, ns, sis, cht=0, dissfactor=0.5):
    case, lo, lr = _pair(name, seed, vfrac)
    P = case.params
    P.order_hyp, P.do_ns, P.species_in_solid, P.conj_ht, P.dissfactor = order, ns, sis, cht, dissfactor
    ref = ref_lib.load(name)
    assert ref.ref_num_species() == P.nspec
    for s in range(P.nspec):  # the plugin's species.cpp values are the oracle's tables
        assert ref.ref_molwt(s) == P.molwt[s] and ref.ref_advect_flag(s) == P.advect_flag[s], s
    orc = oracle_lib.load()
    n = len(case.boxes)
    rc_o = orc.oracle_compute_dsdt(C.byref(P), C.byref(case.geom), lo.descriptors(), n)
    rc_r = ref.ref_compute_dsdt(C.byref(case.geom), lr.descriptors(), n, 0.0, order, dissfactor, ns, sis, cht)
    assert rc_o == rc_r == abi.OK, (rc_o, rc_r)
    for b in range(n):
        for d in range(3):
            _bitwise(lo.flux[b][d], lr.flux[b][d], f"{name} box {b} flux {d}")
        _bitwise(lo.dsdt[b], lr.dsdt[b], f"{name} box {b} dsdt")
    assert max(np.abs(lr.dsdt[b]).max() for b in range(n)) > 0
    return lo, lr


DSDT = [
    # plugin, seed, vfrac, order, do_ns, species_in_solid, conj_ht
    ("stube", 1, "ones", 1, 1, 1, 0),
    ("stube", 2, "ones", 2, 1, 1, 0),
    ("stube", 3, "ones", 4, 1, 1, 0),
    ("stube", 4, "ones", 5, 1, 1, 0),
    ("stube", 5, "mixed", 5, 1, 0, 0),
    ("stube", 6, "mixed", 2, 0, 0, 0),
    ("stubehe", 7, "ones", 5, 1, 1, 0),
    ("stubehe", 8, "mixed", 2, 1, 1, 0),
    ("tg", 9, "ones", 4, 1, 1, 0),
    ("tg", 10, "ones", 5, 1, 1, 0),
    ("speq", 11, "mixed", 2, 0, 0, 0),
    ("speq", 12, "mixed", 2, 0, 1, 0),
    ("bcat", 13, "mixed", 2, 0, 1, 0),
    ("bcat", 14, "mixed", 5, 0, 0, 0),
    ("porous", 15, "mixed", 2, 1, 0, 0),
    ("porous", 16, "mixed", 5, 1, 0, 0),
    ("porous", 17, "mixed", 1, 1, 0, 0),
    ("porous", 18, "mixed", 4, 1, 0, 0),
    ("cht", 19, "mixed", 2, 1, 1, 1),
    ("cht", 20, "mixed", 5, 1, 0, 1),
    ("catcyl", 21, "mixed", 5, 1, 1, 0),
    ("catcyl", 22, "mixed", 2, 1, 1, 0),
    ("catcyl", 23, "ones", 4, 1, 1, 0),
    ("stag", 24, "mixed", 5, 1, 1, 0),
    ("stag", 25, "mixed", 2, 1, 0, 0),
    ("rxn", 26, "mixed", 5, 1, 1, 0),
    ("rxn", 27, "mixed", 2, 1, 0, 0),
    ("rxn", 28, "ones", 1, 1, 1, 0),
]


@needs_ref
@pytest.mark.parametrize("name,seed,vfrac,order,ns,sis,cht", DSDT)
def test_compute_dsdt_bitwise(name, seed, vfrac, order, ns, sis, cht):
    _dsdt_case(name, seed, vfrac, order, ns, sis, cht)


@needs_ref
def test_pin_sees_the_advection_flag_quirk():
    """Negative control: the oracle given the advection flags one would read off
    catalystCylinder's species list (all gases advected) differs from the
    reference, whose species.cpp:6 initialiser {one} advects the first species
    only; the pin resolves such differences to the bit."""
    case, lo, lr = _pair("catcyl", 21, "mixed")
    P = case.params
    P.order_hyp = 5
    for s in range(3):
        P.advect_flag[s] = 1.0
    assert oracle_lib.load().oracle_compute_dsdt(C.byref(P), C.byref(case.geom), lo.descriptors(), 2) == abi.OK
    assert ref_lib.load("catcyl").ref_compute_dsdt(C.byref(case.geom), lr.descriptors(), 2, 0.0, 5, 0.5, 1, 1,
                                                   0) == abi.OK
    with pytest.raises(AssertionError):
        _bitwise(lo.dsdt[0], lr.dsdt[0], "catcyl dsdt")


@needs_ref
def test_unknown_scheme_both_refuse():
    """order_hyp 3 is "unknown hyperbolics scheme" (compute_flux_3d.H:271-274)
    in both; the mixed pattern keeps gas faces in the box."""
    case, lo, lr = _pair("porous", 29, "mixed")
    P = case.params
    P.order_hyp = 3
    rc_o = oracle_lib.load().oracle_compute_dsdt(C.byref(P), C.byref(case.geom), lo.descriptors(), 2)
    rc_r = ref_lib.load("porous").ref_compute_dsdt(C.byref(case.geom), lr.descriptors(), 2, 0.0, 3, 0.5, 1, 0, 0)
    assert rc_o == rc_r == abi.ERR_SCHEME


CUT = [
    # plugin, seed, species_in_solid, use_bg_gas, cht
    ("porous", 31, 0, 0, 0),
    ("catcyl", 32, 1, 0, 0),
    ("stag", 33, 1, 0, 0),
    ("stag", 34, 0, 0, 0),
    ("rxn", 35, 1, 1, 0),
    ("cht", 36, 0, 0, 1),
    ("bcat", 37, 1, 0, 0),
    ("stubehe", 38, 0, 0, 0),
]


@needs_ref
@pytest.mark.parametrize("name,seed,sis,bg,cht", CUT)
def test_cutcells_bitwise(name, seed, sis, bg, cht):
    case, lo, lr = _pair(name, seed, "mixed", with_flux=False)
    P = case.params
    P.species_in_solid, P.conj_ht = sis, cht
    n = len(case.boxes)
    assert oracle_lib.load().oracle_cutcells(C.byref(P), C.byref(case.geom), lo.descriptors(), n) == abi.OK
    assert ref_lib.load(name).ref_cutcells(C.byref(case.geom), lr.descriptors(), n, 0.0, sis, bg, cht) == abi.OK
    changed = 0
    for b in range(n):
        _bitwise(lo.sborder_host(b), lr.sborder_host(b), f"{name} box {b} sborder")
        changed += int((lo.sborder_host(b) != ref_lib_wrap(case, b)).sum())
    assert changed > 0  # the pattern has cut cells, so the pass did change the state


def ref_lib_wrap(case, b):
    lev = Level([case.boxes[b]], case.ncomp, backend="numpy")
    g = abi.NGROW
    full = np.pad(case.state, ((0, 0), (g, g), (g, g), (g, g)), mode="wrap")
    lo, hi = case.boxes[b]
    sl = tuple(slice(lo[q], hi[q] + 2 * g + 1) for q in (2, 1, 0))
    lev.set_sborder(0, full[(slice(None),) + sl])
    return lev.sborder_host(0)


def _chem(name, seed):
    case, lo, lr = _pair(name, seed, "mixed", with_flux=False)
    P = case.params
    ref = ref_lib.load(name)
    if name == "rxn":
        ref_lib.set_chemistry_on(ref, 1)
    n = len(case.boxes)
    assert oracle_lib.load().oracle_chem_source(C.byref(P), lo.descriptors(), n) == abi.OK
    assert ref.ref_chem_source(C.byref(case.geom), lr.descriptors(), n, 0.0) == abi.OK
    ns = P.nspec
    return [(lo.dsdt[b][abi.FLO_NVARS:abi.FLO_NVARS + ns], lr.dsdt[b][abi.FLO_NVARS:abi.FLO_NVARS + ns])
            for b in range(n)]


@needs_ref
def test_chem_source_table_form_bitwise():
    """py_utils/rxnscheme_writer/example/chemistry.H (the table form the oracle
    restates): equal bits, both reactions of the example's table."""
    for o, r in _chem("rxn", 41):
        assert np.abs(r).max() > 0
        _bitwise(o, r, "rxn chemistry source")


@needs_ref
@pytest.mark.parametrize("name", ["catcyl", "stag"])
def test_chem_source_hand_written_plugins(name):
    """catalystCylinder and stagFlowCatalyst write their single surface
    reaction by hand as k * c_S * c_A (* c_B): the table form multiplies the
    concentrations first, (k * ((1 * c_A) * c_S)), so the two may differ in
    the last bits; they agree to 4 ulp."""
    for o, r in _chem(name, 42):
        assert np.abs(r).max() > 0
        np.testing.assert_array_max_ulp(o, r, maxulp=4)


def test_golden_fixture_matches_oracle():
    """tests/golden/ref_pin.npz holds the reference's own outputs (made by
    tests/golden/make_ref_pin.py from oracle/_ref); the oracle reproduces every
    value bit for bit.  Needs no reference checkout."""
    import make_ref_pin as M
    gold = np.load(M.os.path.join(M.HERE, "ref_pin.npz"))
    orc = oracle_lib.load()
    for e in M.DSDT:
        name, seed, vfrac, order, ns, sis, cht = e
        case = ref_lib.seeded_case(name, seed, vfrac=vfrac, n_cell=M.N_CELL, max_grid=M.MAX_GRID)
        P = case.params
        P.order_hyp, P.do_ns, P.species_in_solid, P.conj_ht = order, ns, sis, cht
        lev = M.level_of(case)
        assert orc.oracle_compute_dsdt(C.byref(P), C.byref(case.geom), lev.descriptors(), len(case.boxes)) == 0
        _bitwise(lev.get_state(case.shape_zyx, which="dsdt"), gold[M.key("dsdt", e)], M.key("dsdt", e))
    for e in M.CUT:
        name, seed, sis, bg = e
        case = ref_lib.seeded_case(name, seed, vfrac="mixed", n_cell=M.N_CELL, max_grid=M.MAX_GRID)
        case.params.species_in_solid = sis
        lev = M.level_of(case)
        assert orc.oracle_cutcells(C.byref(case.params), C.byref(case.geom), lev.descriptors(), len(case.boxes)) == 0
        g = abi.NGROW
        for b, (lo, hi) in enumerate(case.boxes):
            want = gold[M.key("cut", e)][:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
            _bitwise(lev.sborder_host(b)[:, g:-g, g:-g, g:-g], want, M.key("cut", e))
