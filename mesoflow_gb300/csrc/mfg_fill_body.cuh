// Physical-boundary device code of the ghost fill (wall parity, ext_dir ghost
// state), shared by the single-level fill (mfg_fill.cu) and the multi-level
// batched fill (mfg_batch.cu).
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {
namespace {

__device__ __forceinline__ bool odd_at_wall(int n) {  // Source/mflo.cpp:98-110
    return (n >= RHOU && n <= RHOW) || (n >= VELX && n <= VELZ);
}

// ext_dir ghost state (the case's externalbc functor as a parameterised template)
template <int NS>
__device__ void external_state(const mfg_extbc& E, int idir, const double* s_int, double* s_ext, int nc) {
    const int ns = c_P.nspec;
    for (int n = 0; n < nc; ++n) s_ext[n] = 0.0;
    if (E.kind == MFG_EXT_FIXED_STATE) {
        for (int n = 0; n < nc; ++n) s_ext[n] = E.state[n];
        if (E.keep_interior_pres) s_ext[PRES] = s_int[PRES];
        return;
    }
    if (E.kind == MFG_EXT_SPECIES_DIRICHLET) {
        for (int n = 0; n < NFLO && n < nc; ++n) s_ext[n] = s_int[n];
        if (!E.vfrac_interior) s_ext[VFRAC] = 1.0;
        for (int s = 0; s < ns; ++s)
            s_ext[NFLO + s] = ((E.spec_zero_grad_mask >> s) & 1)
                                  ? s_int[NFLO + s]
                                  : __dsub_rn(__dmul_rn(2.0, E.spec[s]), s_int[NFLO + s]);
        return;
    }
    double spec[NS];
    double dens, pres, vel[3];
    if (E.kind == MFG_EXT_PRESSURE_INLET) {
        dens = E.dens;
        pres = E.pres;
        const double vm = sqrt((s_int[VELX] * s_int[VELX] + s_int[VELY] * s_int[VELY]) + s_int[VELZ] * s_int[VELZ]);
        vel[0] = vel[1] = vel[2] = 0.0;
        vel[idir] = vm;
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? E.spec[s] : 0.0;
    } else if (E.kind == MFG_EXT_PRESSURE_OUTLET) {
        dens = s_int[DENS];
        pres = E.pres;
        vel[0] = s_int[VELX];
        vel[1] = s_int[VELY];
        vel[2] = s_int[VELZ];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? s_int[NFLO + s] : 0.0;
    } else {
        dens = E.dens;
        pres = E.pres;
        vel[0] = E.vel[0];
        vel[1] = E.vel[1];
        vel[2] = E.vel[2];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? E.spec[s] : 0.0;
    }
    s_ext[DENS] = dens;
    s_ext[PRES] = pres;
    s_ext[VELX] = vel[0];
    s_ext[VELY] = vel[1];
    s_ext[VELZ] = vel[2];
    s_ext[TEMP] = thermo_t<NS>(dens, pres, spec);
    s_ext[RHO] = dens;
    s_ext[RHOU] = mul(dens, vel[0]);
    s_ext[RHOV] = mul(dens, vel[1]);
    s_ext[RHOW] = mul(dens, vel[2]);
    const double ke = add(add(mul(vel[0], vel[0]), mul(vel[1], vel[1])), mul(vel[2], vel[2]));
    s_ext[RHOE] = add(mul(dens, thermo_e<NS>(dens, pres, spec)), mul(mul(0.5, dens), ke));
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < ns) s_ext[NFLO + s] = spec[s];
    s_ext[VFRAC] = s_int[VFRAC];
}

}  // namespace
}  // namespace mfg
