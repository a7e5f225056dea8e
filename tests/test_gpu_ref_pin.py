"""The CUDA path against the reference's own per-cell code.

tests/golden/ref_pin.npz holds outputs of the reference's compute_flux +
update_residual (the box body of compute_dsdt_flow) and update_cutcells,
compiled unmodified from the reference checkout with its case plugins
(oracle/ref.mk, tests/golden/make_ref_pin.py), on seeded states of the
plugins ShockTube_N2 (orders 1, 2, 4, 5), porousParticle (orders 2 and 5 with
immersed boundaries), SpeciesEqTests (no Navier-Stokes terms),
conjHtransferTest, catalystCylinder, stagFlowCatalyst and the rxnscheme
example (background-gas thermo).  The library, given the same plugin tables
through mfg_init, must match every cell and component to 1e-12 of the
component's domain maximum, in both WENO5 normalisations.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from mesoflow_gb300 import abi
from mesoflow_gb300.level import Level
from helpers import rel_err
import ref_lib

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_ref_pin as M  # noqa: E402

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
GOLD = np.load(os.path.join(M.HERE, "ref_pin.npz"))


def _gpu_level(case, lib):
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    ref_lib.wrap_sborder(case, lev)
    return lev


@pytest.mark.parametrize("entry", M.DSDT, ids=[M.key("dsdt", e) for e in M.DSDT])
@pytest.mark.parametrize("fast", [1, 0])
def test_dsdt_matches_reference(entry, fast):
    name, seed, vfrac, order, ns, sis, cht = entry
    case = ref_lib.seeded_case(name, seed, vfrac=vfrac, n_cell=M.N_CELL, max_grid=M.MAX_GRID)
    P = case.params
    P.order_hyp, P.do_ns, P.species_in_solid, P.conj_ht = order, ns, sis, cht
    lib = abi.load()
    lib.mfg_set_weno_mode(fast)
    lev = _gpu_level(case, lib)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    abi.check("mfg_compute_dsdt_flow",
              lib.mfg_compute_dsdt_flow(lev.descriptors(), len(case.boxes), C.byref(case.geom), 0.0, 1e-9, st))
    torch.cuda.synchronize()
    lib.mfg_set_weno_mode(1)
    err, comp = rel_err(lev.get_state(case.shape_zyx, which="dsdt"), GOLD[M.key("dsdt", entry)])
    assert err <= TOL, (err, comp)


@pytest.mark.parametrize("entry", M.CUT, ids=[M.key("cut", e) for e in M.CUT])
def test_cutcells_match_reference(entry):
    name, seed, sis, bg = entry
    case = ref_lib.seeded_case(name, seed, vfrac="mixed", n_cell=M.N_CELL, max_grid=M.MAX_GRID)
    case.params.species_in_solid = sis
    lib = abi.load()
    lev = _gpu_level(case, lib)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    abi.check("mfg_cutcells", lib.mfg_cutcells(lev.descriptors(), len(case.boxes), C.byref(case.geom), 0.0, st))
    torch.cuda.synchronize()
    g = abi.NGROW
    got = np.zeros_like(case.state)
    for b, (lo, hi) in enumerate(case.boxes):
        got[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = lev.sborder_host(b)[:, g:-g, g:-g, g:-g]
    want = GOLD[M.key("cut", entry)]
    assert not np.array_equal(want, case.state)  # the pattern has cut cells
    err, comp = rel_err(got, want)
    assert err <= TOL, (err, comp)
