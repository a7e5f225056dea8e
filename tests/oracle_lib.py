"""Loader of the oracle (oracle/_build/liboracle.so): the CPU restatement of
the reference's numerics used as the checker.  Test infrastructure only."""
import ctypes as C
import os
import subprocess

from mesoflow_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ODIR = os.path.join(ROOT, "oracle")


def build():
    r = subprocess.run(["make", "-s", "-C", ODIR], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load(variant="strict"):
    build()
    name = "liboracle.so" if variant == "strict" else "liboracle_omp.so"
    lib = C.CDLL(os.path.join(ODIR, "_build", name))
    BP, GP, PP = C.POINTER(abi.Box), C.POINTER(abi.Geom), C.POINTER(abi.Params)
    sig = {
        "oracle_compute_dsdt": [PP, GP, BP, C.c_int],
        "oracle_cutcells": [PP, GP, BP, C.c_int],
        "oracle_stage_algebra": [PP, BP, C.c_int, C.c_int, C.c_double],
        "oracle_fill_patch": [PP, GP, BP, C.c_int, C.c_int, C.c_double],
        "oracle_chem_source": [PP, BP, C.c_int],
        "oracle_chem_substep": [PP, BP, C.c_int, C.c_double],
        "oracle_update_primitive_vars": [PP, BP, C.c_int],
        "oracle_clip_species": [PP, BP, C.c_int],
        "oracle_residual_norms": [PP, BP, C.c_int, C.c_double, C.POINTER(C.c_double)],
        "oracle_est_timestep": [PP, GP, BP, C.c_int, C.POINTER(C.c_double)],
        "oracle_advance": [PP, GP, BP, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)],
        "oracle_advance_amr": [PP, GP, BP, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int],
        "oracle_chem_advance_rk2": [PP, BP, C.c_int, C.c_double],
        "oracle_chem_substep_ros2": [PP, BP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int],
        "oracle_store_inertgas_conc": [PP, BP, C.c_int],
        "oracle_update_vars_after_chemsolve": [PP, BP, C.c_int, C.c_int],
        "oracle_abi_layout": [C.POINTER(C.c_int64), C.c_int],
        "oracle_objective": [PP, GP, BP, C.c_int, C.POINTER(C.c_double)],
    }
    for k, v in sig.items():
        f = getattr(lib, k)
        f.argtypes = v
        f.restype = C.c_int
    return lib
