// Device thermodynamics and transport for the three thermo families of the
// reference's case plugins, evaluated from the parameter tables in constant
// memory.  Operand order follows the plugins (sums over gas species in
// ascending order, divisions where the plugins divide) so the FP64 results
// track the reference's rounding.
#pragma once
#include "mfg_common.cuh"

namespace mfg {

extern __constant__ DevParams c_P;

// Temperature from (rho, p, species).  Molar: ShockTube_N2/thermo.H:58-67,
// catalystCylinder/thermo.H:54-63; mass-single: porousParticle/thermo.H:54-59;
// background gas: rxnscheme example thermo.H:61-76.
template <int NS>
__device__ __forceinline__ double thermo_t(double rho, double pres, const double* spec) {
    const DevParams& P = c_P;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return pres / P.gas_R / rho;
    double sum_ci = 0.0;
    if (P.thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) {
                sum_ci += spec[s];
                sum_ciMi += spec[s] * P.molwt[s];
            }
        double c_bg = (rho - sum_ciMi) / P.bg_molwt;
        sum_ci += c_bg;
        return pres / (sum_ci * kRU);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) sum_ci += spec[s];
    return pres / (sum_ci * P.R_univ);
}

// Mixture density from the species concentrations (thermo.H get_r_from_c):
// molar, catalystCylinder/thermo.H:37-45 (gas species); mass-single,
// TaylorGreen/thermo.H:37-45 (every species); background gas, rxnscheme
// example thermo.H:20-31 (gas species + bgasconc W_bg).
template <int NS>
__device__ __forceinline__ double thermo_r_from_c(const double* spec, double bgasconc) {
    const DevParams& P = c_P;
    const int n = (P.thermo_kind == MFG_THERMO_MASS_SINGLE) ? P.nspec : P.ngas;
    double rho = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < n) rho = add(rho, mul(spec[s], P.molwt[s]));
    if (P.thermo_kind == MFG_THERMO_BG_GAS) rho = add(rho, mul(bgasconc, P.bg_molwt));
    return rho;
}

// Untracked background-gas concentration (thermo.H get_bgasconc_from_rc):
// molar 0 (catalystCylinder/thermo.H:47-52), mass-single the first species
// (TaylorGreen/thermo.H:46-53), background gas (rho - sum c W) / W_bg
// (rxnscheme example thermo.H:32-42).
template <int NS>
__device__ __forceinline__ double thermo_bgasconc(double rho, const double* spec) {
    const DevParams& P = c_P;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return spec[0];
    if (P.thermo_kind != MFG_THERMO_BG_GAS) return 0.0;
    double sum_ciMi = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) sum_ciMi = add(sum_ciMi, mul(spec[s], P.molwt[s]));
    return __ddiv_rn(__dsub_rn(rho, sum_ciMi), P.bg_molwt);
}

// Pressure from (rho e, rho, species).
template <int NS>
__device__ __forceinline__ double thermo_p(double rhoe, double rho, const double* spec) {
    const DevParams& P = c_P;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return rhoe * P.gm1_single;
    if (P.thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) sum_ciMi += spec[s] * P.molwt[s];
        double c_bg = (rho - sum_ciMi) / P.bg_molwt;
        double cvs = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) cvs += P.cv[s] * spec[s];
        cvs += P.cv[P.ngas] * c_bg;
        double T = rhoe / cvs;
        double p = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) p += spec[s] * kRU * T;
        p += c_bg * kRU * T;
        return p;
    }
    double cvs = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) cvs += P.cv[s] * spec[s];
    double T = rhoe / cvs;
    double p = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) p += spec[s] * P.R_univ * T;
    return p;
}

// Mixture gamma (depends on composition only).
template <int NS>
__device__ __forceinline__ double thermo_gamma(double rho, const double* spec) {
    const DevParams& P = c_P;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return P.gamma_single;
    double sum_ci = 0.0, term2 = 0.0;
    if (P.thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) sum_ciMi += spec[s] * P.molwt[s];
        double c_bg = (rho - sum_ciMi) / P.bg_molwt;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) sum_ci += spec[s];
        sum_ci += c_bg;
        const double isum = 1.0 / sum_ci;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) term2 += (spec[s] * isum) * P.igm1[s];
        term2 += (c_bg * isum) * P.igm1[P.ngas];
        return 1.0 + 1.0 / term2;
    }
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) sum_ci += spec[s];
    // mole fractions x_s = c_s / sum c and 1/(gamma_s - 1) as products: one
    // division instead of two per species
    const double isum = 1.0 / sum_ci;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) term2 += (spec[s] * isum) * P.igm1[s];
    return 1.0 + 1.0 / term2;
}

// Specific internal energy from (rho, p, species).
template <int NS>
__device__ __forceinline__ double thermo_e(double rho, double pres, const double* spec) {
    const DevParams& P = c_P;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return pres / (P.gamma_single - 1.0) / rho;
    if (P.thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) sum_ciMi += spec[s] * P.molwt[s];
        double c_bg = (rho - sum_ciMi) / P.bg_molwt;
        double temp = thermo_t<NS>(rho, pres, spec);
        double scv = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) scv += P.cv[s] * spec[s];
        scv += P.cv[P.ngas] * c_bg;
        return scv * temp / rho;
    }
    if (P.energy_form == MFG_EFORM_MASS_CV) {
        double sum_ci = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) sum_ci += spec[s];
        double temp = thermo_t<NS>(rho, pres, spec);
        double cvbar = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) cvbar += P.cvmass[s] * (spec[s] / sum_ci);
        return cvbar * temp;
    }
    double temp = thermo_t<NS>(rho, pres, spec);
    double scv = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) scv += P.cv[s] * spec[s];
    return scv * temp / rho;
}

// Transport coefficient: constant, or gas*vfrac + solid*(1-vfrac).
__device__ __forceinline__ double blend(int mode, double g, double s, double vf) {
    return (mode == MFG_TRANSPORT_VFRAC_BLEND) ? (g * vf + s * (1.0 - vf)) : g;
}

// 2 d1 d2 / (d1 + d2 + 1e-30)  (compute_flux_3d.H:18-22)
__device__ __forceinline__ double harmonic_mean(double d1, double d2) {
    return 2.0 * d1 * d2 / (d1 + d2 + 1e-30);
}

}  // namespace mfg
