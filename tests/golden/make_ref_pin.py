"""Writes tests/golden/ref_pin.npz: outputs of the reference's own per-cell
numerics (oracle/_ref, built by oracle/ref.mk from the reference checkout) on
seeded states of its case plugins, so that the GPU can be compared with the
reference itself on a machine without the checkout
(tests/test_gpu_ref_pin.py).

For each entry of DSDT: the valid-box dsdt of ref_compute_dsdt (the box body
of compute_dsdt_flow: compute_flux + update_residual).  For each entry of CUT:
the valid cells of Sborder after ref_cutcells (update_cutcell_data).  The
inputs are regenerated from the seeds by tests/ref_lib.seeded_case.

    python tests/golden/make_ref_pin.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from mesoflow_gb300 import abi  # noqa: E402
from mesoflow_gb300.level import Level  # noqa: E402
import ref_lib  # noqa: E402

N_CELL, MAX_GRID = (8, 8, 6), (4, 8, 6)

# plugin, seed, vfrac, order, do_ns, species_in_solid, conj_ht
DSDT = [
    ("stube", 101, "ones", 1, 1, 1, 0),
    ("stube", 102, "ones", 2, 1, 1, 0),
    ("stube", 103, "ones", 4, 1, 1, 0),
    ("stube", 104, "ones", 5, 1, 1, 0),
    ("porous", 105, "mixed", 2, 1, 0, 0),
    ("porous", 106, "mixed", 5, 1, 0, 0),
    ("speq", 107, "mixed", 2, 0, 1, 0),
    ("cht", 108, "mixed", 2, 1, 1, 1),
    ("catcyl", 109, "mixed", 5, 1, 1, 0),
    ("stag", 110, "mixed", 2, 1, 0, 0),
    ("rxn", 111, "mixed", 5, 1, 1, 0),
]
# plugin, seed, species_in_solid, use_bg_gas
CUT = [
    ("porous", 121, 0, 0),
    ("catcyl", 122, 1, 0),
    ("rxn", 123, 1, 1),
]


def key(kind, entry):
    return f"{kind}_{entry[0]}_{entry[1]}"


def level_of(case, with_flux=False):
    lev = Level(case.boxes, case.ncomp, backend="numpy", with_flux=with_flux)
    lev.set_state(case.state)
    ref_lib.wrap_sborder(case, lev)
    return lev


def main():
    out = {}
    for e in DSDT:
        name, seed, vfrac, order, ns, sis, cht = e
        case = ref_lib.seeded_case(name, seed, vfrac=vfrac, n_cell=N_CELL, max_grid=MAX_GRID)
        lev = level_of(case)
        lib = ref_lib.load(name)
        rc = lib.ref_compute_dsdt(C.byref(case.geom), lev.descriptors(), len(case.boxes), 0.0, order, 0.5, ns, sis, cht)
        assert rc == abi.OK, rc
        out[key("dsdt", e)] = lev.get_state(case.shape_zyx, which="dsdt")
    for e in CUT:
        name, seed, sis, bg = e
        case = ref_lib.seeded_case(name, seed, vfrac="mixed", n_cell=N_CELL, max_grid=MAX_GRID)
        lev = level_of(case)
        assert ref_lib.load(name).ref_cutcells(C.byref(case.geom), lev.descriptors(), len(case.boxes), 0.0, sis, bg,
                                               0) == abi.OK
        g = abi.NGROW
        valid = np.zeros_like(case.state)
        for b, (lo, hi) in enumerate(case.boxes):
            sb = lev.sborder_host(b)[:, g:-g, g:-g, g:-g]
            valid[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = sb
        out[key("cut", e)] = valid
    path = os.path.join(HERE, "ref_pin.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
