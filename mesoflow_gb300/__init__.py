"""mesoflow_gb300 — GB300 (sm_103a) FP64 implementation of NREL/mesoflow's
per-box explicit right-hand side and SSP-RK3 stage update, behind the C ABI
of include/mflo_gpu.h.

Python here is plumbing: ctypes bindings (abi), per-box storage (level),
case set-ups (cases) and a single-level driver (driver).  The computation is
the CUDA library mesoflow_gb300/_lib/libmflo_gpu.so; nothing falls back to
the CPU.
"""
from . import abi  # noqa: F401

__version__ = "0.1.0"
