"""The AMReX-side adapter on the GPU: a level's boxes handed over as
amrex::Array4<Real> views (compiled against the AMReX stand-in) through
mflo_gpu::BoxSet into mfg_compute_dsdt_flow and mfg_cutcells give the
reference's own per-cell results (tests/golden/ref_pin.npz: compute_flux +
update_residual and update_cutcells compiled from the reference checkout) to
1e-12 of each component's domain maximum."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from mesoflow_gb300 import abi
from mesoflow_gb300.level import Level
from helpers import rel_err
import adapter_build
import ref_lib

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_ref_pin as M  # noqa: E402

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(M.HERE, "ref_pin.npz"))


def _args(case, lev):
    n = len(case.boxes)
    lohi = (C.c_int * (6 * n))(*[v for lo, hi in case.boxes for v in (*lo, *hi)])
    ptrs = [(C.c_void_p * n)(*[t.data_ptr() for t in arrs]) for arrs in (lev.sborder, lev.dsdt, lev.s_old, lev.s_new)]
    G = case.geom
    return (n, lohi, *ptrs, case.ncomp, (C.c_double * 3)(*G.dx), (C.c_double * 3)(*G.prob_lo),
            (C.c_int * 3)(*G.domain_lo), (C.c_int * 3)(*G.domain_hi), (C.c_int * 3)(*G.is_periodic))


def _level(case):
    lib = abi.load()
    abi.check("mfg_init", lib.mfg_init(C.byref(case.params)))
    lev = Level(case.boxes, case.ncomp, backend="torch", device="cuda")
    lev.set_state(case.state)
    ref_lib.wrap_sborder(case, lev)
    return lev


@pytest.mark.parametrize("entry", M.DSDT, ids=[M.key("dsdt", e) for e in M.DSDT])
def test_adapter_dsdt_matches_reference(entry):
    name, seed, vfrac, order, ns, sis, cht = entry
    case = ref_lib.seeded_case(name, seed, vfrac=vfrac, n_cell=M.N_CELL, max_grid=M.MAX_GRID)
    P = case.params
    P.order_hyp, P.do_ns, P.species_in_solid, P.conj_ht = order, ns, sis, cht
    lev = _level(case)
    ad = adapter_build.build(with_lib=True)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert ad.adapter_dsdt(*_args(case, lev), 0.0, 1e-9, st) == abi.OK
    torch.cuda.synchronize()
    err, comp = rel_err(lev.get_state(case.shape_zyx, which="dsdt"), GOLD[M.key("dsdt", entry)])
    assert err <= 1e-12, (err, comp)


@pytest.mark.parametrize("entry", M.CUT, ids=[M.key("cut", e) for e in M.CUT])
def test_adapter_cutcells_match_reference(entry):
    name, seed, sis, bg = entry
    case = ref_lib.seeded_case(name, seed, vfrac="mixed", n_cell=M.N_CELL, max_grid=M.MAX_GRID)
    case.params.species_in_solid = sis
    lev = _level(case)
    ad = adapter_build.build(with_lib=True)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert ad.adapter_cutcells(*_args(case, lev), 0.0, st) == abi.OK
    torch.cuda.synchronize()
    g = abi.NGROW
    got = np.zeros_like(case.state)
    for b, (lo, hi) in enumerate(case.boxes):
        got[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = lev.sborder_host(b)[:, g:-g, g:-g, g:-g]
    err, comp = rel_err(got, GOLD[M.key("cut", entry)])
    assert err <= 1e-12, (err, comp)
