"""Writes tests/golden/flops_per_cell_update.json: the algorithmic FP64
operation count of one cell-update of the benchmark workload, counted on the
reference's own per-cell code.

The counting build (oracle/ref.mk, libref_count_porous.so) compiles the
reference's Source/Src_3d numerics and the models/porousParticle plugin with
amrex::Real = a double that counts every add/sub, mul, div, sqrt and other
call (oracle/ref_shim/count_double.H).  It runs the box bodies of
compute_dsdt_flow (compute_flux over the faces of the three directions,
update_residual over every component) and update_cutcell_data on the eight
central 64^3 boxes of the 256^3 sphere-pack workload (order_hyp 2,
species_in_solid 0, its initial state: a quiescent gas, so every face takes
the subsonic branch it takes in the run), whose ghost cells lie inside the
domain.  Per cell-update = 3 x (flux + residual + cut cells) / cell, plus
the stage algebra of Advance_coupled_strang (Source/mflo_evolve.cpp:283-311:
LinComb 3, Saxpy 2 + Saxpy 2 + mult 1, Saxpy 2 + Xpay 2 + mult 1 = 13 ops per
component) and compute_residual_norms (:91-112: LinComb 3 and norm2 2 per
component, vfrac scaling 1 per flow component).  The primitive refresh and
the (inactive) chemistry sub-step are left out (< 1%).

    python tests/golden/make_flop_counts.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from mesoflow_gb300 import abi, cases  # noqa: E402
from mesoflow_gb300.level import Level  # noqa: E402
import ref_lib  # noqa: E402

KINDS = ["add", "mul", "div", "sqrt", "other"]


def counting_lib(name):
    ref_lib.build()
    lib = C.CDLL(os.path.join(ref_lib.ODIR, "_ref", f"libref_count_{name}.so"))
    lib.ref_init()
    GP, BP = C.POINTER(abi.Geom), C.POINTER(abi.Box)
    lib.ref_compute_dsdt.argtypes = [GP, BP, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
    lib.ref_cutcells.argtypes = [GP, BP, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
    lib.ref_flop_counts.argtypes = [C.POINTER(C.c_uint64), C.c_int]
    return lib


def read(lib):
    out = (C.c_uint64 * 5)()
    lib.ref_flop_counts(out, 1)
    return dict(zip(KINDS, [int(x) for x in out]))


def main():
    n, mg, order = 256, 64, 2
    case = cases.porous_ib(n=n, order=order, max_grid=mg)
    g = abi.NGROW
    central = [(lo, hi) for lo, hi in case.boxes if all(mg <= lo[d] and hi[d] < n - mg for d in range(3))]
    lev = Level(central, case.ncomp, backend="numpy")
    for b, (lo, hi) in enumerate(central):
        sl = tuple(slice(lo[q] - g, hi[q] + g + 1) for q in (2, 1, 0))
        lev.set_sborder(b, case.state[(slice(None),) + sl])
    lib = counting_lib("porous")
    desc = lev.descriptors()
    cells = sum(int(np.prod([hi[d] - lo[d] + 1 for d in range(3)])) for lo, hi in central)
    read(lib)
    assert lib.ref_cutcells(C.byref(case.geom), desc, len(central), 0.0, 0, 0, 0) == 0
    cut = read(lib)
    assert lib.ref_compute_dsdt(C.byref(case.geom), desc, len(central), 0.0, order, 0.5, 1, 0, 0) == 0
    rhs = read(lib)
    N = case.ncomp
    per_rhs = {k: (cut[k] + rhs[k]) / cells for k in KINDS}
    algebra = 13 * N + (3 + 2) * N + (abi.VFRAC - abi.RHO)
    total = 3 * sum(per_rhs.values()) + algebra
    out = {"porous_ib_256_order2": {
        "flop_per_cell_update": total,
        "per_rhs_per_cell": per_rhs,
        "cutcells_per_cell": {k: cut[k] / cells for k in KINDS},
        "flux_and_residual_per_cell": {k: rhs[k] / cells for k in KINDS},
        "stage_algebra_and_norms_per_cell": algebra,
        "divisions_per_cell_update": 3 * per_rhs["div"],
        "sqrt_per_cell_update": 3 * per_rhs["sqrt"],
        "sample": f"{len(central)} central {mg}^3 boxes of the {n}^3 sphere pack (order_hyp {order}), "
                  "initial state, counting build of the reference's own Source/Src_3d code with the "
                  "models/porousParticle plugin",
        "ncomp": N}}
    path = os.path.join(HERE, "flops_per_cell_update.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
