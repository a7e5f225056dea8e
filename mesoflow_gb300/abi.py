"""ctypes mirror of include/mflo_gpu.h and the loader of the CUDA library.

The structures below must match the C header field for field; the CPU test
suite checks their sizes and offsets against the C compiler's.
"""
import ctypes as C
import os

MAX_SPECIES = 16
MAX_REACTIONS = 16
FLO_NVARS = 12
NCVARS = 5
NGROW = 3

RHO, RHOU, RHOV, RHOW, RHOE = 0, 1, 2, 3, 4
DENS, VELX, VELY, VELZ, PRES, TEMP, VFRAC = 5, 6, 7, 8, 9, 10, 11

OK, ERR_ARG, ERR_NAN, ERR_NEG_PRESSURE, ERR_SCHEME, ERR_TIMEOUT, ERR_CUDA, ERR_STATE, ERR_SIZE = range(9)
NOALLOC_SCRATCH_DOUBLES = 4194304
STATUS_NAN, STATUS_NEG_PRESSURE, STATUS_TIMEOUT, STATUS_BAD_BOX, STATUS_CHEM_STEPS = 0x1, 0x2, 0x4, 0x8, 0x10

THERMO_MOLAR, THERMO_MASS_SINGLE, THERMO_BG_GAS = 0, 1, 2
EFORM_MOLAR_CV, EFORM_MASS_CV = 0, 1
TRANSPORT_CONST, TRANSPORT_VFRAC_BLEND = 0, 1
BC_INT_DIR, BC_FOEXTRAP, BC_EXT_DIR, BC_WALL = 0, 2, 3, 6
EXT_FIXED_STATE, EXT_PRESSURE_INLET, EXT_PRESSURE_OUTLET, EXT_VELOCITY_INLET, EXT_SPECIES_DIRICHLET = 0, 1, 2, 3, 4

ERROR_NAMES = {
    OK: "ok", ERR_ARG: "bad argument", ERR_NAN: "NaN detected in dsdt",
    ERR_NEG_PRESSURE: "Pressure has gone negative", ERR_SCHEME: "unknown hyperbolics scheme",
    ERR_TIMEOUT: "device wait timed out", ERR_CUDA: "CUDA error", ERR_STATE: "library not initialised or configuration not supported",
    ERR_SIZE: "box needs more scratch than the static array of the allocation-free entry point",
}


class Array4(C.Structure):
    _fields_ = [("p", C.c_void_p), ("jstride", C.c_int64), ("kstride", C.c_int64), ("nstride", C.c_int64),
                ("begin", C.c_int * 3), ("end", C.c_int * 3), ("ncomp", C.c_int)]


class Box(C.Structure):
    _fields_ = [("lo", C.c_int * 3), ("hi", C.c_int * 3), ("sborder", Array4), ("dsdt", Array4),
                ("s_old", Array4), ("s_new", Array4), ("flux", Array4 * 3), ("level", C.c_int), ("pad_", C.c_int)]


class Geom(C.Structure):
    _fields_ = [("dx", C.c_double * 3), ("prob_lo", C.c_double * 3), ("domain_lo", C.c_int * 3),
                ("domain_hi", C.c_int * 3), ("is_periodic", C.c_int * 3), ("pad_", C.c_int)]


class ExtBC(C.Structure):
    _fields_ = [("kind", C.c_int), ("keep_interior_pres", C.c_int), ("spec_zero_grad_mask", C.c_int),
                ("vfrac_interior", C.c_int), ("dens", C.c_double), ("pres", C.c_double),
                ("vel", C.c_double * 3), ("spec", C.c_double * MAX_SPECIES),
                ("state", C.c_double * (FLO_NVARS + MAX_SPECIES))]


class Params(C.Structure):
    _fields_ = [
        ("nspec", C.c_int), ("ngas", C.c_int), ("thermo_kind", C.c_int), ("energy_form", C.c_int),
        ("R_univ", C.c_double), ("gas_R", C.c_double), ("gamma_single", C.c_double), ("bg_molwt", C.c_double),
        ("molwt", C.c_double * MAX_SPECIES), ("gamma", C.c_double * (MAX_SPECIES + 1)),
        ("advect_flag", C.c_double * MAX_SPECIES),
        ("visc_mode", C.c_int), ("cond_mode", C.c_int),
        ("visc_gas", C.c_double), ("visc_solid", C.c_double), ("cond_gas", C.c_double), ("cond_solid", C.c_double),
        ("diff_mode", C.c_int * MAX_SPECIES), ("diff_gas", C.c_double * MAX_SPECIES),
        ("diff_solid", C.c_double * MAX_SPECIES),
        ("order_hyp", C.c_int), ("do_ns", C.c_int), ("species_in_solid", C.c_int), ("conj_ht", C.c_int),
        ("dissfactor", C.c_double), ("solid_temp", C.c_double), ("cfl", C.c_double),
        ("chem_on", C.c_int), ("nreact", C.c_int),
        ("nu", (C.c_double * MAX_SPECIES) * MAX_REACTIONS), ("order", (C.c_double * MAX_SPECIES) * MAX_REACTIONS),
        ("A", C.c_double * MAX_REACTIONS), ("Ea", C.c_double * MAX_REACTIONS),
        ("bc_lo", C.c_int * 3), ("bc_hi", C.c_int * 3),
        ("ext_lo", ExtBC * 3), ("ext_hi", ExtBC * 3),
    ]


HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmflo_gpu.so")

# (name, restype, argtypes) of every exported entry point
_VP = C.c_void_p
_BP = C.POINTER(Box)
_GP = C.POINTER(Geom)
SIGNATURES = [
    ("mfg_init", C.c_int, [C.POINTER(Params)]),
    ("mfg_finalize", C.c_int, []),
    ("mfg_status", C.c_int, [C.POINTER(C.c_uint32), C.c_int]),
    ("mfg_version", C.c_char_p, []),
    ("mfg_fill_patch", C.c_int, [_BP, C.c_int, _GP, C.c_int, C.c_double, _VP]),
    ("mfg_cutcells", C.c_int, [_BP, C.c_int, _GP, C.c_double, _VP]),
    ("mfg_compute_dsdt_flow", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.c_double, _VP]),
    ("mfg_rk3_stage", C.c_int, [_BP, C.c_int, _GP, C.c_int, C.c_double, C.c_double, _VP]),
    ("mfg_chem_source", C.c_int, [_BP, C.c_int, _GP, C.c_double, _VP]),
    ("mfg_chem_substep", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.c_double, _VP]),
    ("mfg_update_primitive_vars", C.c_int, [_BP, C.c_int, _GP, _VP]),
    ("mfg_clip_species", C.c_int, [_BP, C.c_int, _VP]),
    ("mfg_residual_norms", C.c_int, [_BP, C.c_int, C.c_double, C.POINTER(C.c_double), _VP]),
    ("mfg_est_timestep", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.POINTER(C.c_double), _VP]),
    ("mfg_advance_level", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.POINTER(C.c_double), _VP]),
    ("mfg_advance_level_host", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.POINTER(Array4), C.POINTER(C.c_double), _VP]),
    ("mfg_set_weno_mode", C.c_int, [C.c_int]),
    ("mfg_set_cutcell_cache", C.c_int, [C.c_int]),
    ("mfg_set_face_compaction", C.c_int, [C.c_int]),
    ("mfg_profile", C.c_int, [C.c_int]),
    ("mfg_profile_read", C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.c_int]),
    ("mfg_profile_name", C.c_char_p, [C.c_int]),
    ("mfg_launch_count", C.c_ulonglong, []),
    ("mfg_compute_dsdt_flow_noalloc", C.c_int, [_BP, C.c_int, _GP, C.c_double, C.c_double, _VP]),
    ("mfg_measure_fp64_peak", C.c_int, [C.POINTER(C.c_double), _VP]),
    ("mfg_selftest_exact_ops", C.c_int, [C.c_ulonglong, C.POINTER(C.c_uint)]),
    ("mfg_boxlist_create", C.c_int, [_BP, C.c_int, _GP, C.c_int, C.POINTER(C.c_void_p)]),
    ("mfg_boxlist_destroy", C.c_int, [C.c_void_p]),
    ("mfg_boxlist_step", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _VP]),
    ("mfg_boxlist_step_amr", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _VP]),
    ("mfg_boxlist_evolve", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_int), _VP]),
    ("mfg_boxlist_evolve_amr", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_int), _VP]),
    ("mfg_chem_advance_rk2", C.c_int, [_BP, C.c_int, C.c_double, C.c_double, _VP]),
    ("mfg_set_chem_integrator", C.c_int, [C.c_int, C.c_double, C.c_double, C.c_int]),
    ("mfg_set_adjoint_flux_form", C.c_int, [C.c_int]),
    ("mfg_store_inertgas_conc", C.c_int, [_BP, C.c_int, _VP]),
    ("mfg_update_vars_after_chemsolve", C.c_int, [_BP, C.c_int, C.c_int, _VP]),
    ("mfg_boxlist_autotune", C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_double), _VP]),
    ("mfg_boxlist_cells", C.c_longlong, [C.c_void_p]),
    ("mfg_last_error", C.c_char_p, []),
    ("mfg_reaction_objective", C.c_int, [_BP, C.c_int, _GP, C.POINTER(C.c_double), _VP]),
    ("mfg_adjoint_objective", C.c_int, [_BP, C.c_int, _GP, C.c_int, C.c_double, C.c_int,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), _VP]),
]

_lib = None


def load(path=None):
    """Loads libmflo_gpu.so (built by mesoflow_gb300.build).  Raises if absent:
    there is no CPU fallback for the GPU path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library {p} is missing; run mesoflow_gb300.build.build() first")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MfloError(RuntimeError):
    def __init__(self, call, code):
        msg = f"{call} failed: {ERROR_NAMES.get(code, code)} (status {code})"
        if code == ERR_CUDA and _lib is not None:
            detail = _lib.mfg_last_error()
            if detail:
                msg += f" [{detail.decode()}]"
        super().__init__(msg)
        self.code = code


def check(call, code):
    if code != OK:
        raise MfloError(call, code)
    return code
