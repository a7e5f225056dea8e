// Forwards to the AMReX stand-in (see amrex_shim.H).
#include "amrex_shim.H"
