// ORACLE — test infrastructure only.  A CPU restatement of NREL/mesoflow's
// per-cell numerics for the per-box RHS + RK3 path, used by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline leg as the checker.
// It is never linked into, imported by, or called from the product library.
//
// Every function follows the reference statement by statement (same operand
// order, same constants) so that, built with -ffp-contract=off, it reproduces
// the reference's FP64 rounding.  Citations are file:line in NREL/mesoflow.
// Parity anchor: tests pin this restatement against the reference's Sod
// exact-solution fixture (tests/Cartesian/ShockTube_N2/exact_soln) and
// analytic cases; AMReX-side semantics (ghost fill corners, TimeIntegrator
// tableau, norm2 summation order) are restated from AMReX's documented
// behaviour and are unpinned (AMReX is not vendored in the reference).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mflo_gpu.h"

namespace oracle {

// Source/globalDefines.H:5-32
constexpr int RHO_IND = 0, RHOU_IND = 1, RHOV_IND = 2, RHOW_IND = 3, RHOE_IND = 4;
constexpr int DENS_IND = 0, VELX_IND = 1, VELY_IND = 2, VELZ_IND = 3, PRES_IND = 4;
constexpr int NCVARS = 5;
constexpr int RHO_INDX = 0, RHOU_INDX = 1, RHOV_INDX = 2, RHOW_INDX = 3, RHOE_INDX = 4;
constexpr int DENS_INDX = 5, VELX_INDX = 6, VELY_INDX = 7, VELZ_INDX = 8, PRES_INDX = 9;
constexpr int TEMP_INDX = 10, VFRAC_INDX = 11, FLO_NVARS = 12;
constexpr int VISC_INDX = 0, THCOND_INDX = 1;
constexpr int XDIR = 0, YDIR = 1, ZDIR = 2;
constexpr int MAXS = MFG_MAX_SPECIES;
constexpr int MAXC = NCVARS + MAXS;

// Source/mflo_constants.H:4-27 (values exactly as the macros)
constexpr double zeroval = 0.0, one = 1.0, two = 2.0, three = 3.0, four = 4.0, five = 5.0;
constexpr double two3rd = 0.6666666666666666667, half = 0.5;
constexpr double third = (two3rd * half);
constexpr double sixth = (two3rd * half * half);
constexpr double eighth = 0.125, sixteenth = 0.0625, twelveth = 0.08333333333, fourth = 0.25;
constexpr double tenth = 0.1, threetenth = 0.3, threefourth = 0.75;
constexpr double RU = 8.31446261815324;
constexpr double TINYVAL = 1e-20, TINYVAL2 = 1e-40;

// Source/globalDefines.H:49-51
inline int GET_XDIR(int a) { return (a * (a - 1) / 2 - 2 * a * (a - 2)); }
inline int GET_YDIR(int a) { return ((a - 1) * (a - 2) / 2 + a * (a - 1)); }
inline int GET_ZDIR(int a) { return ((a - 1) * (a - 2) - a * (a - 2)); }

// amrex::Array4<Real> indexing
struct A4 {
    double* p = nullptr;
    int64_t js = 0, ks = 0, ns = 0;
    int b0 = 0, b1 = 0, b2 = 0;
    A4() = default;
    explicit A4(const mfg_array4& a)
        : p(a.p), js(a.jstride), ks(a.kstride), ns(a.nstride),
          b0(a.begin[0]), b1(a.begin[1]), b2(a.begin[2]) {}
    double& operator()(int i, int j, int k, int n) const {
        return p[(int64_t)(i - b0) + (int64_t)(j - b1) * js + (int64_t)(k - b2) * ks + (int64_t)n * ns];
    }
    double& at(const int iv[3], int n) const { return (*this)(iv[0], iv[1], iv[2], n); }
};

struct Ctx {
    const mfg_params* P;
    int nspec;
};

// ---------------------------------------------------------------------------
// Thermo plugins
// ---------------------------------------------------------------------------
// MFG_THERMO_MOLAR: models/catalystCylinder/thermo.H:54-156 (sums over the gas
// species), tests/Cartesian/ShockTube_N2/thermo.H:58-132 (R_univ variable).
// MFG_THERMO_MASS_SINGLE: tests/Cartesian/TaylorGreen/thermo.H:54-80,
// models/porousParticle/thermo.H:54-80 (R_air = RU/W).
// MFG_THERMO_BG_GAS: py_utils/rxnscheme_writer/example/thermo.H:61-190.
inline double cv_molar(const mfg_params* P, int sp) { return P->R_univ / (P->gamma[sp] - one); }

inline double get_t_from_rpc(const Ctx& c, double rho, double pres, const double* spec) {
    const mfg_params* P = c.P;
    if (P->thermo_kind == MFG_THERMO_MASS_SINGLE) {
        return (pres / P->gas_R / rho);
    } else if (P->thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ci = zeroval, sum_ciMi = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) {
            sum_ci += spec[sp];
            sum_ciMi += spec[sp] * P->molwt[sp];
        }
        double c_bg_gas = (rho - sum_ciMi) / P->bg_molwt;
        sum_ci += c_bg_gas;
        return (pres / (sum_ci * RU));
    }
    double sum_ci = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) sum_ci += spec[sp];
    return (pres / (sum_ci * P->R_univ));
}

// get_r_from_c: catalystCylinder/thermo.H:37-45 (molar, gas species),
// TaylorGreen/thermo.H:37-45 (mass-single, every species), rxnscheme example
// thermo.H:20-31 (background gas, + bgasconc W_bg).
inline double get_r_from_c(const Ctx& c, const double* spec, double bgasconc) {
    const mfg_params* P = c.P;
    const int n = (P->thermo_kind == MFG_THERMO_MASS_SINGLE) ? P->nspec : P->ngas;
    double rho = zeroval;
    for (int sp = 0; sp < n; sp++) rho += spec[sp] * P->molwt[sp];
    if (P->thermo_kind == MFG_THERMO_BG_GAS) rho += bgasconc * P->bg_molwt;
    return rho;
}

// get_bgasconc_from_rc: catalystCylinder/thermo.H:47-52 (0), TaylorGreen/
// thermo.H:46-53 (spec[AIR_ID]), rxnscheme example thermo.H:32-42.
inline double get_bgasconc_from_rc(const Ctx& c, double rho, const double* spec) {
    const mfg_params* P = c.P;
    if (P->thermo_kind == MFG_THERMO_MASS_SINGLE) return spec[0];
    if (P->thermo_kind != MFG_THERMO_BG_GAS) return 0.0;
    double sum_ciMi = 0.0;
    for (int sp = 0; sp < P->ngas; sp++) sum_ciMi += spec[sp] * P->molwt[sp];
    return (rho - sum_ciMi) / P->bg_molwt;
}

inline double get_p_from_rec(const Ctx& c, double rhoe, double rho, const double* spec) {
    const mfg_params* P = c.P;
    if (P->thermo_kind == MFG_THERMO_MASS_SINGLE) {
        return (rhoe * (P->gamma_single - one));
    } else if (P->thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_ciMi += spec[sp] * P->molwt[sp];
        double c_bg_gas = (rho - sum_ciMi) / P->bg_molwt;
        double cv_spec[MAXS + 1];
        for (int sp = 0; sp < P->ngas + 1; sp++) cv_spec[sp] = RU / (P->gamma[sp] - one);
        double cv_times_spec = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) cv_times_spec += cv_spec[sp] * spec[sp];
        cv_times_spec += cv_spec[P->ngas] * c_bg_gas;
        double T = rhoe / cv_times_spec;
        double p = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) p += spec[sp] * RU * T;
        p += c_bg_gas * RU * T;
        return p;
    }
    double cv_times_spec = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) cv_times_spec += cv_molar(P, sp) * spec[sp];
    double T = rhoe / cv_times_spec;
    double p = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) p += spec[sp] * P->R_univ * T;
    return p;
}

inline double get_gama_from_rpc(const Ctx& c, double rho, double pres, const double* spec) {
    const mfg_params* P = c.P;
    (void)pres;
    if (P->thermo_kind == MFG_THERMO_MASS_SINGLE) {
        return P->gamma_single;
    } else if (P->thermo_kind == MFG_THERMO_BG_GAS) {
        double x_i[MAXS + 1];
        double sum_ciMi = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_ciMi += spec[sp] * P->molwt[sp];
        double c_bg_gas = (rho - sum_ciMi) / P->bg_molwt;
        double sum_ci = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_ci += spec[sp];
        sum_ci += c_bg_gas;
        for (int sp = 0; sp < P->ngas; sp++) x_i[sp] = spec[sp] / sum_ci;
        x_i[P->ngas] = c_bg_gas / sum_ci;
        double term2 = zeroval;
        for (int sp = 0; sp < P->ngas + 1; sp++) term2 += x_i[sp] / (P->gamma[sp] - one);
        return one + std::pow(term2, -one);
    }
    double x_i[MAXS];
    double sum_ci = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) sum_ci += spec[sp];
    for (int sp = 0; sp < P->ngas; sp++) x_i[sp] = spec[sp] / sum_ci;
    double term2 = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) term2 += x_i[sp] / (P->gamma[sp] - one);
    return one + std::pow(term2, -one);
}

inline double get_e_from_rpc(const Ctx& c, double rho, double pres, const double* spec) {
    const mfg_params* P = c.P;
    if (P->thermo_kind == MFG_THERMO_MASS_SINGLE) {
        return (pres / (P->gamma_single - one) / rho);
    } else if (P->thermo_kind == MFG_THERMO_BG_GAS) {
        double sum_ciMi = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_ciMi += spec[sp] * P->molwt[sp];
        double c_bg_gas = (rho - sum_ciMi) / P->bg_molwt;
        double cv_spec[MAXS + 1];
        for (int sp = 0; sp < P->ngas + 1; sp++) cv_spec[sp] = RU / (P->gamma[sp] - one);
        double temp = get_t_from_rpc(c, rho, pres, spec);
        double sum_cvi_ci = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_cvi_ci += cv_spec[sp] * spec[sp];
        sum_cvi_ci += cv_spec[P->ngas] * c_bg_gas;
        return (sum_cvi_ci * temp / rho);
    }
    if (P->energy_form == MFG_EFORM_MASS_CV) {
        double x_i[MAXS];
        double sum_ci = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) sum_ci += spec[sp];
        for (int sp = 0; sp < P->ngas; sp++) x_i[sp] = spec[sp] / sum_ci;
        double temp = get_t_from_rpc(c, rho, pres, spec);
        double cvbar = zeroval;
        for (int sp = 0; sp < P->ngas; sp++) cvbar += (P->R_univ / (P->gamma[sp] - one) / P->molwt[sp]) * x_i[sp];
        return (cvbar * temp);
    }
    double temp = get_t_from_rpc(c, rho, pres, spec);
    double sum_cvi_ci = zeroval;
    for (int sp = 0; sp < P->ngas; sp++) sum_cvi_ci += cv_molar(P, sp) * spec[sp];
    return (sum_cvi_ci * temp / rho);
}

// ---------------------------------------------------------------------------
// Transport plugins (transport.H compute_spec_dcoeff, userfuncs.H
// compute_fluid_transport); models/catalystCylinder/transport.H:10-28 blend.
// ---------------------------------------------------------------------------
inline double blend(int mode, double g, double s, double vfrac) {
    if (mode == MFG_TRANSPORT_VFRAC_BLEND) return g * vfrac + s * (one - vfrac);
    return g;
}
inline double visc_at(const Ctx& c, const A4& phi, int i, int j, int k) {
    return blend(c.P->visc_mode, c.P->visc_gas, c.P->visc_solid, phi(i, j, k, VFRAC_INDX));
}
inline double cond_at(const Ctx& c, const A4& phi, int i, int j, int k) {
    return blend(c.P->cond_mode, c.P->cond_gas, c.P->cond_solid, phi(i, j, k, VFRAC_INDX));
}
inline double diff_at(const Ctx& c, const A4& phi, const int iv[3], int sp) {
    return blend(c.P->diff_mode[sp], c.P->diff_gas[sp], c.P->diff_solid[sp], phi.at(iv, VFRAC_INDX));
}

// ---------------------------------------------------------------------------
// Source/Src_3d/consprim_funcs.H
// ---------------------------------------------------------------------------
inline void cons_to_prim(const Ctx& c, const double* u, double* p) {  // :9-23
    p[DENS_IND] = u[RHO_IND];
    p[VELX_IND] = u[RHOU_IND] / u[RHO_IND];
    p[VELY_IND] = u[RHOV_IND] / u[RHO_IND];
    p[VELZ_IND] = u[RHOW_IND] / u[RHO_IND];
    double rhoe = u[RHOE_IND] - half * u[RHO_IND] *
                  (p[VELX_IND] * p[VELX_IND] + p[VELY_IND] * p[VELY_IND] + p[VELZ_IND] * p[VELZ_IND]);
    p[PRES_IND] = get_p_from_rec(c, rhoe, u[RHO_IND], u + NCVARS);
}

inline void prim_to_cons(const Ctx& c, double* u, const double* p) {  // :26-44
    u[RHO_IND] = p[DENS_IND];
    u[RHOU_IND] = p[DENS_IND] * p[VELX_IND];
    u[RHOV_IND] = p[DENS_IND] * p[VELY_IND];
    u[RHOW_IND] = p[DENS_IND] * p[VELZ_IND];
    u[RHOE_IND] = u[RHO_IND] * get_e_from_rpc(c, p[DENS_IND], p[PRES_IND], u + NCVARS);
    u[RHOE_IND] += half * u[RHO_IND] *
                   (p[VELX_IND] * p[VELX_IND] + p[VELY_IND] * p[VELY_IND] + p[VELZ_IND] * p[VELZ_IND]);
}

inline void geteulerflux(const Ctx& c, const double* u, double* f, const double* n) {  // :48-81
    double nx = n[XDIR], ny = n[YDIR], nz = n[ZDIR];
    double rho = u[RHO_IND];
    double vx = u[RHOU_IND] / rho;
    double vy = u[RHOV_IND] / rho;
    double vz = u[RHOW_IND] / rho;
    double rhoe = u[RHOE_IND] - half * u[RHO_IND] * (vx * vx + vy * vy + vz * vz);
    double p = get_p_from_rec(c, rhoe, u[RHO_IND], u + NCVARS);
    f[RHO_IND] = rho * vx * nx + rho * vy * ny + rho * vz * nz;
    f[RHOU_IND] = (rho * vx * vx + p) * nx + rho * vx * vy * ny + rho * vx * vz * nz;
    f[RHOV_IND] = rho * vy * vx * nx + (rho * vy * vy + p) * ny + rho * vy * vz * nz;
    f[RHOW_IND] = rho * vz * vx * nx + rho * vz * vy * ny + (rho * vz * vz + p) * nz;
    f[RHOE_IND] = (u[RHOE_IND] + p) * (vx * nx + vy * ny + vz * nz);
    for (int sp = 0; sp < c.nspec; sp++) f[NCVARS + sp] = u[NCVARS + sp] * (vx * nx + vy * ny + vz * nz);
}

// ---------------------------------------------------------------------------
// Source/Src_3d/flux_schemes.H
// ---------------------------------------------------------------------------
inline double get_max_eigenvalue(const Ctx& c, const double* ul, const double* ur, const double* n) {  // :12-46
    double rhoL = ul[RHO_IND], rhoR = ur[RHO_IND];
    double rhoeL = ul[RHOE_IND] - half * (ul[RHOU_IND] * ul[RHOU_IND] + ul[RHOV_IND] * ul[RHOV_IND] +
                                          ul[RHOW_IND] * ul[RHOW_IND]) / ul[RHO_IND];
    double rhoeR = ur[RHOE_IND] - half * (ur[RHOU_IND] * ur[RHOU_IND] + ur[RHOV_IND] * ur[RHOV_IND] +
                                          ur[RHOW_IND] * ur[RHOW_IND]) / ur[RHO_IND];
    double presL = get_p_from_rec(c, rhoeL, ul[RHO_IND], ul + NCVARS);
    double presR = get_p_from_rec(c, rhoeR, ur[RHO_IND], ul + NCVARS);  // (sic) ul species, :33
    double veln_L = (ul[RHOU_IND] * n[0] + ul[RHOV_IND] * n[1] + ul[RHOW_IND] * n[2]) / ul[RHO_IND];
    double veln_R = (ur[RHOU_IND] * n[0] + ur[RHOV_IND] * n[1] + ur[RHOW_IND] * n[2]) / ur[RHO_IND];
    double veln = std::max(std::fabs(veln_L), std::fabs(veln_R));
    double gamaL = get_gama_from_rpc(c, rhoL, presL, ul + NCVARS);
    double gamaR = get_gama_from_rpc(c, rhoR, presR, ur + NCVARS);
    double ahalf = std::max(std::sqrt(gamaL * presL / rhoL), std::sqrt(gamaR * presR / rhoR));
    return (ahalf + veln);
}

inline double split_Mach(double M, double beta, double plus_or_minus) {  // :107-141
    double Msplit;
    if (plus_or_minus < 0) {
        if (std::fabs(M) <= one)
            Msplit = -fourth * (M - one) * (M - one) - beta * (M * M - one) * (M * M - one);
        else
            Msplit = half * (M - std::fabs(M));
    } else {
        if (std::fabs(M) <= 1)
            Msplit = fourth * (M + one) * (M + one) + beta * (M * M - one) * (M * M - one);
        else
            Msplit = half * (M + std::fabs(M));
    }
    return Msplit;
}

inline double split_pres(double M, double alpha, double plus_or_minus) {  // :145-181
    double Psplit;
    if (plus_or_minus < 0) {
        if (std::fabs(M) <= one)
            Psplit = fourth * (M - one) * (M - one) * (two + M) - alpha * M * (M * M - one) * (M * M - one);
        else
            Psplit = half * (M - std::fabs(M)) / M;
    } else {
        if (std::fabs(M) <= one)
            Psplit = fourth * (M + one) * (M + one) * (two - M) + alpha * M * (M * M - one) * (M * M - one);
        else
            Psplit = half * (M + std::fabs(M)) / M;
    }
    return Psplit;
}

inline void ausmp_up_flux(const Ctx& c, const double* ul, const double* ur, double* fhalf,
                          const double* n, double Minf = threetenth) {  // :185-310
    double fluxL[MAXC], fluxR[MAXC], pl[NCVARS], pr[NCVARS];
    double delta = threetenth, beta = eighth, sigma = one, Kp = fourth, Ku = threefourth;
    double Minf2 = Minf * Minf;
    double nx = n[XDIR], ny = n[YDIR], nz = n[ZDIR];
    cons_to_prim(c, ul, pl);
    cons_to_prim(c, ur, pr);
    double gamaL = get_gama_from_rpc(c, pl[DENS_IND], pl[PRES_IND], ul + NCVARS);
    double gamaR = get_gama_from_rpc(c, pr[DENS_IND], pr[PRES_IND], ur + NCVARS);
    double vL = pl[VELX_IND] * nx + pl[VELY_IND] * ny + pl[VELZ_IND] * nz;
    double vR = pr[VELX_IND] * nx + pr[VELY_IND] * ny + pr[VELZ_IND] * nz;
    double HL = gamaL / (gamaL - one) * (pl[PRES_IND] / pl[DENS_IND]) +
                half * (pl[VELX_IND] * pl[VELX_IND] + pl[VELY_IND] * pl[VELY_IND] + pl[VELZ_IND] * pl[VELZ_IND]);
    double HR = gamaR / (gamaR - one) * (pr[PRES_IND] / pr[DENS_IND]) +
                half * (pr[VELX_IND] * pr[VELX_IND] + pr[VELY_IND] * pr[VELY_IND] + pr[VELZ_IND] * pr[VELZ_IND]);
    double rho_half = half * (pl[DENS_IND] + pr[DENS_IND]);
    double astar2 = two * (gamaL - one) / (gamaL + one) * HL;
    double ahatL = astar2 / std::max(std::sqrt(astar2), std::fabs(vL));
    astar2 = two * (gamaR - one) / (gamaR + one) * HR;
    double ahatR = astar2 / std::max(std::sqrt(astar2), std::fabs(vR));
    double a_half = std::min(ahatL, ahatR);
    double ML = vL / a_half, MR = vR / a_half;
    double MLplus = split_Mach(ML, beta, one);
    double MRminus = split_Mach(MR, beta, -one);
    double M_half = MLplus + MRminus;
    double M_bar2 = half * (vL * vL + vR * vR) / (a_half * a_half);
    double Mo2 = std::min(one, std::max(M_bar2, Minf2));
    double Mo = std::sqrt(Mo2);
    double fa_Mo = Mo * (two - Mo);
    M_half = M_half - (Kp / fa_Mo) * std::max(one - sigma * M_bar2, zeroval) *
                          (pr[PRES_IND] - pl[PRES_IND]) / (rho_half * a_half * a_half);
    fluxL[RHO_IND] = ul[RHO_IND];
    fluxL[RHOU_IND] = ul[RHOU_IND];
    fluxL[RHOV_IND] = ul[RHOV_IND];
    fluxL[RHOW_IND] = ul[RHOW_IND];
    fluxL[RHOE_IND] = ul[RHOE_IND] + pl[PRES_IND];
    fluxR[RHO_IND] = ur[RHO_IND];
    fluxR[RHOU_IND] = ur[RHOU_IND];
    fluxR[RHOV_IND] = ur[RHOV_IND];
    fluxR[RHOW_IND] = ur[RHOW_IND];
    fluxR[RHOE_IND] = ur[RHOE_IND] + pr[PRES_IND];
    for (int sp = 0; sp < c.nspec; sp++) {
        fluxL[NCVARS + sp] = ul[NCVARS + sp];
        fluxR[NCVARS + sp] = ur[NCVARS + sp];
    }
    double mod_M_half = std::fabs(M_half);
    if (mod_M_half <= delta) mod_M_half = (M_half * M_half + delta * delta) / (two * delta);
    for (int i = 0; i < NCVARS + c.nspec; i++)
        fhalf[i] = (half * M_half * (fluxL[i] + fluxR[i]) - half * mod_M_half * (fluxR[i] - fluxL[i])) * a_half;
    double alpha = three * sixteenth * (-four + five * fa_Mo * fa_Mo);
    double PLplus = split_pres(ML, alpha, one);
    double PRminus = split_pres(MR, alpha, -one);
    double p_half = (PLplus * pl[PRES_IND] + PRminus * pr[PRES_IND]);
    p_half = p_half - Ku * PLplus * PRminus * (pl[DENS_IND] + pr[DENS_IND]) * (fa_Mo * a_half) * (vR - vL);
    fhalf[RHOU_IND] += p_half * nx;
    fhalf[RHOV_IND] += p_half * ny;
    fhalf[RHOW_IND] += p_half * nz;
}

inline void central_with_diss_flux(const Ctx& c, const double* uim1, const double* ui, const double* uim2,
                                   const double* uip1, double* fhalf, const double* n,
                                   double dissfactor) {  // :313-361
    double fim1[MAXC], fi[MAXC], fim2[MAXC], fip1[MAXC];
    geteulerflux(c, uim2, fim2, n);
    geteulerflux(c, uim1, fim1, n);
    geteulerflux(c, ui, fi, n);
    geteulerflux(c, uip1, fip1, n);
    double rhoL = uim1[RHO_IND], rhoR = ui[RHO_IND];
    double rhoeL = uim1[RHOE_IND] - half * (uim1[RHOU_IND] * uim1[RHOU_IND] + uim1[RHOV_IND] * uim1[RHOV_IND] +
                                            uim1[RHOW_IND] * uim1[RHOW_IND]) / uim1[RHO_IND];
    double rhoeR = ui[RHOE_IND] - half * (ui[RHOU_IND] * ui[RHOU_IND] + ui[RHOV_IND] * ui[RHOV_IND] +
                                          ui[RHOW_IND] * ui[RHOW_IND]) / ui[RHO_IND];
    double presL = get_p_from_rec(c, rhoeL, uim1[RHO_IND], uim1 + NCVARS);
    double presR = get_p_from_rec(c, rhoeR, ui[RHO_IND], ui + NCVARS);
    double veln_L = (uim1[RHOU_IND] * n[0] + uim1[RHOV_IND] * n[1] + uim1[RHOW_IND] * n[2]) / uim1[RHO_IND];
    double veln_R = (ui[RHOU_IND] * n[0] + ui[RHOV_IND] * n[1] + ui[RHOW_IND] * n[2]) / ui[RHO_IND];
    double veln = std::max(std::fabs(veln_L), std::fabs(veln_R));
    double gamaL = get_gama_from_rpc(c, rhoL, presL, uim1 + NCVARS);
    double gamaR = get_gama_from_rpc(c, rhoR, presR, ui + NCVARS);
    double ahalf = std::max(std::sqrt(gamaL * presL / rhoL), std::sqrt(gamaR * presR / rhoR));
    for (int i = 0; i < NCVARS + c.nspec; i++) {
        fhalf[i] = twelveth * (7 * fi[i] + 7 * fim1[i] - fim2[i] - fip1[i]);
        fhalf[i] -= twelveth * (3 * ui[i] - 3 * uim1[i] - uip1[i] + ui[i]) * (veln + ahalf) * dissfactor;
    }
}

inline void weno_reconstruct(int nc, const double* uim2, const double* uim1, const double* ui,
                             const double* uip1, const double* uip2, const double* uip3,
                             double* umhalf, double* uphalf) {  // :373-446
    constexpr double eps = 1e-6;
    double vl[3], vr[3], beta[3], alpha[3], s[6];
    for (int c = 0; c < nc; c++) {
        s[0] = uim2[c]; s[1] = uim1[c]; s[2] = ui[c];
        s[3] = uip1[c]; s[4] = uip2[c]; s[5] = uip3[c];
        double t;
        // pow(x, 2) is x*x (glibc pow is correctly rounded; GCC folds it).
        t = s[0] - 2.0 * s[1] + s[2];
        double t2 = s[0] - 4.0 * s[1] + 3.0 * s[2];
        beta[2] = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
        t = s[1] - 2.0 * s[2] + s[3];
        beta[1] = (13.0 / 12.0) * (t * t) + 0.25 * (s[1] - s[3]) * (s[1] - s[3]);
        t = s[2] - 2.0 * s[3] + s[4];
        t2 = 3.0 * s[2] - 4.0 * s[3] + s[4];
        beta[0] = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
        beta[2] = 1.0 / ((eps + beta[2]) * (eps + beta[2]));
        beta[1] = 1.0 / ((eps + beta[1]) * (eps + beta[1]));
        beta[0] = 1.0 / ((eps + beta[0]) * (eps + beta[0]));
        alpha[2] = beta[2];
        alpha[1] = 6.0 * beta[1];
        alpha[0] = 3.0 * beta[0];
        double alpha1 = 1.0 / (alpha[2] + alpha[1] + alpha[0]);
        vl[2] = 2.0 * s[0] - 7.0 * s[1] + 11.0 * s[2];
        vl[1] = -s[1] + 5.0 * s[2] + 2.0 * s[3];
        vl[0] = 2.0 * s[2] + 5.0 * s[3] - s[4];
        uphalf[c] = (1.0 / 6.0) * alpha1 * (alpha[2] * vl[2] + alpha[1] * vl[1] + alpha[0] * vl[0]);

        t = s[5] - 2.0 * s[4] + s[3];
        t2 = s[5] - 4.0 * s[4] + 3.0 * s[3];
        beta[2] = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
        t = s[4] - 2.0 * s[3] + s[2];
        beta[1] = (13.0 / 12.0) * (t * t) + 0.25 * (s[4] - s[2]) * (s[4] - s[2]);
        t = s[3] - 2.0 * s[2] + s[1];
        t2 = 3.0 * s[3] - 4.0 * s[2] + s[1];
        beta[0] = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
        beta[2] = 1.0 / ((eps + beta[2]) * (eps + beta[2]));
        beta[1] = 1.0 / ((eps + beta[1]) * (eps + beta[1]));
        beta[0] = 1.0 / ((eps + beta[0]) * (eps + beta[0]));
        alpha[2] = beta[2];
        alpha[1] = 6.0 * beta[1];
        alpha[0] = 3.0 * beta[0];
        alpha1 = 1.0 / (alpha[2] + alpha[1] + alpha[0]);
        vr[2] = 11.0 * s[3] - 7.0 * s[4] + 2.0 * s[5];
        vr[1] = -s[4] + 5.0 * s[3] + 2.0 * s[2];
        vr[0] = 2.0 * s[3] + 5.0 * s[2] - s[1];
        umhalf[c] = (1.0 / 6.0) * alpha1 * (alpha[2] * vr[2] + alpha[1] * vr[1] + alpha[0] * vr[0]);
    }
}

inline void weno_flux(const Ctx& c, const double* ulm2, const double* ulm1, const double* ul,
                      const double* ur, const double* urp1, const double* urp2, double* fhalf,
                      const double* normal) {  // :450-495
    int nc = NCVARS + c.nspec;
    double fr[MAXC] = {0}, frp1[MAXC] = {0}, frp2[MAXC] = {0}, fl[MAXC] = {0}, flm1[MAXC] = {0}, flm2[MAXC] = {0};
    double fphalf[MAXC] = {0}, fmhalf[MAXC] = {0}, uphalf[MAXC] = {0}, umhalf[MAXC] = {0};
    double lambda_max = get_max_eigenvalue(c, ul, ur, normal);
    geteulerflux(c, ul, fl, normal);
    geteulerflux(c, ulm1, flm1, normal);
    geteulerflux(c, ulm2, flm2, normal);
    geteulerflux(c, ur, fr, normal);
    geteulerflux(c, urp1, frp1, normal);
    geteulerflux(c, urp2, frp2, normal);
    weno_reconstruct(nc, flm2, flm1, fl, fr, frp1, frp2, fmhalf, fphalf);
    weno_reconstruct(nc, ulm2, ulm1, ul, ur, urp1, urp2, umhalf, uphalf);
    for (int k = 0; k < nc; k++)
        fhalf[k + RHO_IND] = half * (fphalf[k] + lambda_max * uphalf[k]) + half * (fmhalf[k] - lambda_max * umhalf[k]);
}

// ---------------------------------------------------------------------------
// Source/Src_3d/compute_flux_3d.H
// ---------------------------------------------------------------------------
inline double harmonic_mean(double d1, double d2) {  // :18-22
    double heps = 1e-30;
    return (2.0 * d1 * d2 / (d1 + d2 + heps));
}

inline void get_higherorder_states(int nc, double* uLh, double* uRh, const double* uL, const double* uR,
                                   const double* uim2, const double* uip1) {  // :33-65
    double L[MAXC];
    for (int c = 0; c < nc; c++) {
        double delt1 = uip1[c] - uR[c];
        double delt2 = uL[c] - uim2[c];
        double q = std::fabs((delt1 - delt2) / (std::fabs(delt1) + std::fabs(delt2) + TINYVAL));
        double psi = one - q * q;  // pow(q, sigma=2)
        L[c] = half * psi * (delt1 + delt2);
    }
    for (int c = 0; c < nc; c++) {
        uLh[c] = uL[c] + half * L[c];
        uRh[c] = uR[c] - half * L[c];
    }
}

// One face flux (:88-430).  fx holds zeros on entry (setVal, mflo_evolve.cpp:572).
inline int compute_flux(const Ctx& c, int i, int j, int k, int sweepdir, const A4& phi, const A4& fx,
                        const double* dx) {
    const mfg_params* P = c.P;
    const int ns = c.nspec, nc = NCVARS + ns;
    double ur[MAXC] = {0}, urp1[MAXC] = {0}, urp2[MAXC] = {0}, ul[MAXC] = {0}, ulm1[MAXC] = {0}, ulm2[MAXC] = {0};
    double ul2[MAXC] = {0}, ur2[MAXC] = {0}, fhalf[MAXC] = {0};
    double normal[3] = {zeroval, zeroval, zeroval};
    double gradu[3], gradv[3], gradw[3], tau[3][3];
    double spec_dcoeff[MAXS];
    normal[sweepdir] = one;
    int ivm3[3] = {i, j, k}, ivm2[3] = {i, j, k}, ivm1[3] = {i, j, k}, iv[3] = {i, j, k}, ivp1[3] = {i, j, k},
        ivp2[3] = {i, j, k};
    int left[3] = {i, j, k}, right[3] = {i, j, k}, left1[3] = {i, j, k}, right1[3] = {i, j, k};
    int top_left[3] = {i, j, k}, bot_left[3] = {i, j, k}, top_right[3] = {i, j, k}, bot_right[3] = {i, j, k};
    int frt_left[3] = {i, j, k}, bck_left[3] = {i, j, k}, frt_right[3] = {i, j, k}, bck_right[3] = {i, j, k};
    int trans1dir = (sweepdir + 1) % 3, trans2dir = (sweepdir + 2) % 3;
    left[sweepdir] -= 1; top_left[sweepdir] -= 1; bot_left[sweepdir] -= 1; frt_left[sweepdir] -= 1; bck_left[sweepdir] -= 1;
    top_left[trans1dir] += 1; top_right[trans1dir] += 1; bot_left[trans1dir] -= 1; bot_right[trans1dir] -= 1;
    frt_left[trans2dir] += 1; frt_right[trans2dir] += 1; bck_left[trans2dir] -= 1; bck_right[trans2dir] -= 1;
    left1[sweepdir] -= 2; right1[sweepdir] += 1;
    ivm3[sweepdir] -= 3; ivm2[sweepdir] -= 2; ivm1[sweepdir] -= 1; ivp1[sweepdir] += 1; ivp2[sweepdir] += 2;

    // Q1: viscosity / conductivity always from (i,j,k) and (i-1,j,k) (:179-180)
    double visc = harmonic_mean(visc_at(c, phi, i, j, k), visc_at(c, phi, i - 1, j, k));
    double thcond = harmonic_mean(cond_at(c, phi, i, j, k), cond_at(c, phi, i - 1, j, k));
    for (int sp = 0; sp < ns; sp++) spec_dcoeff[sp] = harmonic_mean(diff_at(c, phi, left, sp), diff_at(c, phi, right, sp));

    double facevel[3];
    facevel[XDIR] = half * (phi.at(left, VELX_INDX) + phi.at(right, VELX_INDX));
    facevel[YDIR] = half * (phi.at(left, VELY_INDX) + phi.at(right, VELY_INDX));
    facevel[ZDIR] = half * (phi.at(left, VELZ_INDX) + phi.at(right, VELZ_INDX));
    double facevfrac = half * (phi.at(left, VFRAC_INDX) + phi.at(right, VFRAC_INDX));

    for (int q = 0; q < NCVARS; q++) {
        ul[q] = phi.at(ivm1, q); ulm1[q] = phi.at(ivm2, q); ulm2[q] = phi.at(ivm3, q);
        ur[q] = phi.at(iv, q); urp1[q] = phi.at(ivp1, q); urp2[q] = phi.at(ivp2, q);
    }
    for (int q = 0; q < ns; q++) {
        ul[q + NCVARS] = phi.at(ivm1, q + FLO_NVARS); ulm1[q + NCVARS] = phi.at(ivm2, q + FLO_NVARS);
        ulm2[q + NCVARS] = phi.at(ivm3, q + FLO_NVARS); ur[q + NCVARS] = phi.at(iv, q + FLO_NVARS);
        urp1[q + NCVARS] = phi.at(ivp1, q + FLO_NVARS); urp2[q + NCVARS] = phi.at(ivp2, q + FLO_NVARS);
    }

    if (P->do_ns) {
        if (phi.at(ivm3, VFRAC_INDX) < one || phi.at(ivm2, VFRAC_INDX) < one || phi.at(ivm1, VFRAC_INDX) < one ||
            phi.at(iv, VFRAC_INDX) < one || phi.at(ivp1, VFRAC_INDX) < one || phi.at(ivp2, VFRAC_INDX) < one) {
            for (int q = 0; q < nc; q++) {  // first-order fallback (:233-249)
                ulm1[q] = ul[q]; ulm2[q] = ul[q];
                urp1[q] = ur[q]; urp2[q] = ur[q];
            }
        }
        if (facevfrac >= 0.5) {
            if (P->order_hyp == 1) {
                ausmp_up_flux(c, ul, ur, fhalf, normal);
            } else if (P->order_hyp == 2) {
                get_higherorder_states(nc, ul2, ur2, ul, ur, ulm1, urp1);
                ausmp_up_flux(c, ul2, ur2, fhalf, normal);
            } else if (P->order_hyp == 4) {
                central_with_diss_flux(c, ul, ur, ulm1, urp1, fhalf, normal, P->dissfactor);
            } else if (P->order_hyp == 5) {
                weno_flux(c, ulm2, ulm1, ul, ur, urp1, urp2, fhalf, normal);
            } else {
                return MFG_ERR_SCHEME;
            }
            for (int q = 0; q < NCVARS; q++) fx(i, j, k, q + RHO_INDX) = fhalf[q + RHO_IND];
            for (int sp = 0; sp < ns; sp++) fx(i, j, k, sp + FLO_NVARS) = P->advect_flag[sp] * fhalf[NCVARS + sp];

            double dxs = dx[sweepdir], dt1 = dx[trans1dir], dt2 = dx[trans2dir];
            gradu[0] = (phi.at(right, VELX_INDX) - phi.at(left, VELX_INDX)) / dxs;
            gradu[1] = (half * (phi.at(top_left, VELX_INDX) + phi.at(top_right, VELX_INDX)) -
                        half * (phi.at(bot_left, VELX_INDX) + phi.at(bot_right, VELX_INDX))) / (two * dt1);
            gradu[2] = (half * (phi.at(frt_left, VELX_INDX) + phi.at(frt_right, VELX_INDX)) -
                        half * (phi.at(bck_left, VELX_INDX) + phi.at(bck_right, VELX_INDX))) / (two * dt2);
            gradv[0] = (phi.at(right, VELY_INDX) - phi.at(left, VELY_INDX)) / dxs;
            gradv[1] = (half * (phi.at(top_left, VELY_INDX) + phi.at(top_right, VELY_INDX)) -
                        half * (phi.at(bot_left, VELY_INDX) + phi.at(bot_right, VELY_INDX))) / (two * dt1);
            gradv[2] = (half * (phi.at(frt_left, VELY_INDX) + phi.at(frt_right, VELY_INDX)) -
                        half * (phi.at(bck_left, VELY_INDX) + phi.at(bck_right, VELY_INDX))) / (two * dt2);
            gradw[0] = (phi.at(right, VELZ_INDX) - phi.at(left, VELZ_INDX)) / dxs;
            gradw[1] = (half * (phi.at(top_left, VELZ_INDX) + phi.at(top_right, VELZ_INDX)) -
                        half * (phi.at(bot_left, VELZ_INDX) + phi.at(bot_right, VELZ_INDX))) / (two * dt1);
            gradw[2] = (half * (phi.at(frt_left, VELZ_INDX) + phi.at(frt_right, VELZ_INDX)) -
                        half * (phi.at(bck_left, VELZ_INDX) + phi.at(bck_right, VELZ_INDX))) / (two * dt2);
            int gx = GET_XDIR(sweepdir), gy = GET_YDIR(sweepdir), gz = GET_ZDIR(sweepdir);
            double dudx = gradu[gx], dudy = gradu[gy], dudz = gradu[gz];
            double dvdx = gradv[gx], dvdy = gradv[gy], dvdz = gradv[gz];
            double dwdx = gradw[gx], dwdy = gradw[gy], dwdz = gradw[gz];
            double delu = dudx + dvdy + dwdz;
            tau[XDIR][XDIR] = visc * (two * dudx - two3rd * delu);
            tau[XDIR][YDIR] = visc * (dudy + dvdx);
            tau[XDIR][ZDIR] = visc * (dudz + dwdx);
            tau[YDIR][XDIR] = visc * (dvdx + dudy);
            tau[YDIR][YDIR] = visc * (two * dvdy - two3rd * delu);
            tau[YDIR][ZDIR] = visc * (dvdz + dwdy);
            tau[ZDIR][XDIR] = visc * (dwdx + dudz);
            tau[ZDIR][YDIR] = visc * (dwdy + dvdz);
            tau[ZDIR][ZDIR] = visc * (two * dwdz - two3rd * delu);
            fx(i, j, k, RHOU_INDX) -= (tau[XDIR][XDIR] * normal[XDIR] + tau[YDIR][XDIR] * normal[YDIR] + tau[ZDIR][XDIR] * normal[ZDIR]);
            fx(i, j, k, RHOV_INDX) -= (tau[XDIR][YDIR] * normal[XDIR] + tau[YDIR][YDIR] * normal[YDIR] + tau[ZDIR][YDIR] * normal[ZDIR]);
            fx(i, j, k, RHOW_INDX) -= (tau[XDIR][ZDIR] * normal[XDIR] + tau[YDIR][ZDIR] * normal[YDIR] + tau[ZDIR][ZDIR] * normal[ZDIR]);
            fx(i, j, k, RHOE_INDX) -= (tau[XDIR][XDIR] * normal[XDIR] + tau[YDIR][XDIR] * normal[YDIR] + tau[ZDIR][XDIR] * normal[ZDIR]) * facevel[XDIR];
            fx(i, j, k, RHOE_INDX) -= (tau[XDIR][YDIR] * normal[XDIR] + tau[YDIR][YDIR] * normal[YDIR] + tau[ZDIR][YDIR] * normal[ZDIR]) * facevel[YDIR];
            fx(i, j, k, RHOE_INDX) -= (tau[XDIR][ZDIR] * normal[XDIR] + tau[YDIR][ZDIR] * normal[YDIR] + tau[ZDIR][ZDIR] * normal[ZDIR]) * facevel[ZDIR];
        }
        double dTdn = (phi.at(right, TEMP_INDX) - phi.at(left, TEMP_INDX)) / dx[sweepdir];
        fx(i, j, k, RHOE_INDX) -= thcond * dTdn;
    } else {
        for (int sp = 0; sp < ns; sp++) {  // species convection (:382-421)
            double phi_im2 = phi.at(left1, FLO_NVARS + sp);
            double phi_im1 = phi.at(left, FLO_NVARS + sp);
            double phi_i = phi.at(right, FLO_NVARS + sp);
            double phi_ip1 = phi.at(right1, FLO_NVARS + sp);
            double phiL = phi_im1, phiR = phi_i;
            if (!P->species_in_solid) {
                if (phi.at(right1, VFRAC_INDX) < one || phi.at(right, VFRAC_INDX) < one ||
                    phi.at(left, VFRAC_INDX) < one || phi.at(left1, VFRAC_INDX) < one) {
                    phi_im2 = phi_im1;
                    phi_ip1 = phi_i;
                }
            }
            (void)phi_im2; (void)phi_ip1;  // Q2: the scalar get_higherorder_states is a by-value no-op (:69-83)
            double velface = facevel[sweepdir];
            if (P->species_in_solid) {
                double weightL = (phi.at(left, VFRAC_INDX) < one) ? zeroval : one;
                double weightR = (phi.at(left, VFRAC_INDX) < one) ? zeroval : one;  // Q3 (sic) :411
                velface = (weightL * phi.at(left, VELX_INDX + sweepdir) + weightR * phi.at(right, VELX_INDX + sweepdir)) /
                          (weightL + weightR + TINYVAL);
            }
            fx(i, j, k, FLO_NVARS + sp) = P->advect_flag[sp] *
                (half * (velface + std::fabs(velface)) * phiL + half * (velface - std::fabs(velface)) * phiR);
        }
    }
    for (int sp = 0; sp < ns; sp++)  // species diffusion (:425-428)
        fx(i, j, k, FLO_NVARS + sp) -= spec_dcoeff[sp] * (ur[NCVARS + sp] - ul[NCVARS + sp]) / dx[sweepdir];
    return MFG_OK;
}

// Source/Src_3d/div_3d.H:13-76 (source term is zero: compute_fluid_source of every case)
inline int update_residual(const Ctx& c, int i, int j, int k, int n, const A4& dsdt, const A4& phi, const A4& fx,
                           const A4& fy, const A4& fz, const double* dx) {
    const mfg_params* P = c.P;
    double src = 0.0;
    dsdt(i, j, k, n) = (fx(i, j, k, n) - fx(i + 1, j, k, n)) / dx[0] + (fy(i, j, k, n) - fy(i, j + 1, k, n)) / dx[1] +
                       (fz(i, j, k, n) - fz(i, j, k + 1, n)) / dx[2] + src;
    int nvars_to_nullify = (P->species_in_solid == 1) ? FLO_NVARS : FLO_NVARS + c.nspec;
    if (n != RHOE_INDX) {
        if (n < nvars_to_nullify && phi(i, j, k, VFRAC_INDX) < one) dsdt(i, j, k, n) = zeroval;
    } else {
        if (!P->conj_ht) {
            if (phi(i, j, k, VFRAC_INDX) < one) dsdt(i, j, k, n) = zeroval;
        } else {
            if (phi(i, j, k, VFRAC_INDX) > zeroval && phi(i, j, k, VFRAC_INDX) < one) dsdt(i, j, k, n) = zeroval;
        }
    }
    if (dsdt(i, j, k, n) != dsdt(i, j, k, n)) return MFG_ERR_NAN;
    return MFG_OK;
}

// ---------------------------------------------------------------------------
// Source/Src_3d/ib_utils.H
// ---------------------------------------------------------------------------
inline double basis1d(int i, double zeta) {  // :14-35
    if (i == -1) return half * zeta * (zeta - one);
    if (i == 0) return (one - zeta * zeta);
    if (i == 1) return half * zeta * (zeta + one);
    return 0.0;
}
inline double basisder1d(int i, double zeta) {  // :38-59
    if (i == -1) return half * (two * zeta - one);
    if (i == 0) return -two * zeta;
    if (i == 1) return half * (two * zeta + one);
    return 0.0;
}
inline double basisderval(int l, int m, int n, int dir, const double* xp, const double* dx) {  // :80-96
    double alpha = xp[XDIR] / dx[XDIR], beta = xp[YDIR] / dx[YDIR], gama = xp[ZDIR] / dx[ZDIR];
    double lval = (dir == 0) ? basisder1d(l, alpha) / dx[XDIR] : basis1d(l, alpha);
    double mval = (dir == 1) ? basisder1d(m, beta) / dx[YDIR] : basis1d(m, beta);
    double nval = (dir == 2) ? basisder1d(n, gama) / dx[ZDIR] : basis1d(n, gama);
    return (lval * mval * nval);
}

inline double do_interpolation_dirichlet(int i, int j, int k, int ngrow, double dist, double dist_cutoff,
                                         double dircval, const A4& phi, int comp, const double* dx) {  // :99-152
    double dxmin = std::min(dx[XDIR], std::min(dx[YDIR], dx[ZDIR]));
    double dx_nd[3] = {dx[0] / dxmin, dx[1] / dxmin, dx[2] / dxmin};
    double dist_nd = std::fabs(dist) / dxmin;
    double cellval;
    if (std::fabs(dist) < dist_cutoff) {
        cellval = dircval;
    } else {
        double sum = 0.0, sumwts = 0.0;
        for (int n = -ngrow; n <= ngrow; n++)
            for (int m = -ngrow; m <= ngrow; m++)
                for (int l = -ngrow; l <= ngrow; l++) {
                    if (l == 0 && m == 0 && n == 0) continue;
                    if (phi(i + l, j + m, k + n, VFRAC_INDX) == 1.0) {
                        double a = l * dx_nd[0], b = m * dx_nd[1], d = n * dx_nd[2];
                        double dist2 = a * a + b * b + d * d;  // std::pow(.,2.0)
                        sum += phi(i + l, j + m, k + n, comp) / (dist2 + TINYVAL2);
                        sumwts += 1.0 / (dist2 + TINYVAL2);
                    }
                }
        sum += dircval / (dist_nd * dist_nd);
        sumwts += 1.0 / (dist_nd * dist_nd);
        cellval = sum / sumwts;
    }
    return cellval;
}

inline double do_interpolation_hom_neumann(int i, int j, int k, int ngrow, const double* xp, const A4& phi, int comp,
                                           const double* dx) {  // :155-198
    double dxmin = std::min(dx[XDIR], std::min(dx[YDIR], dx[ZDIR]));
    double dx_nd[3] = {dx[0] / dxmin, dx[1] / dxmin, dx[2] / dxmin};
    double xp_nd[3] = {xp[0] / dxmin, xp[1] / dxmin, xp[2] / dxmin};
    double sum = 0.0, sumwts = 0.0;
    for (int n = -ngrow; n <= ngrow; n++)
        for (int m = -ngrow; m <= ngrow; m++)
            for (int l = -ngrow; l <= ngrow; l++) {
                if (phi(i + l, j + m, k + n, VFRAC_INDX) == 1.0) {
                    double a = (l * dx_nd[0] - xp_nd[0]), b = (m * dx_nd[1] - xp_nd[1]), d = (n * dx_nd[2] - xp_nd[2]);
                    double dist2 = a * a + b * b + d * d;
                    sum += phi(i + l, j + m, k + n, comp) / (dist2 + TINYVAL2);
                    sumwts += 1.0 / (dist2 + TINYVAL2);
                }
            }
    if (sumwts > 0.0) return sum / sumwts;
    return phi(i, j, k, comp);
}

// In place on the state, for one valid cell (:272-436).
inline void update_cutcells(const Ctx& c, int i, int j, int k, const A4& phi, const double* dx) {
    const mfg_params* P = c.P;
    double lsgrad[3] = {0.0, 0.0, 0.0}, center[3] = {0.0, 0.0, 0.0};
    double tol = 1e-5;
    double primvars[NCVARS] = {0}, consvars[MAXC] = {0};
    double dxmin = std::min(dx[XDIR], std::min(dx[YDIR], dx[ZDIR]));
    double closest_dist = dxmin * tol;
    const int STENCILGROW = 2;
    double vf = phi(i, j, k, VFRAC_INDX);
    if (!(vf > zeroval && vf < one)) return;
    for (int n = -1; n <= 1; n++)
        for (int m = -1; m <= 1; m++)
            for (int l = -1; l <= 1; l++) {
                lsgrad[XDIR] += phi(i + l, j + m, k + n, VFRAC_INDX) * basisderval(l, m, n, XDIR, center, dx);
                lsgrad[YDIR] += phi(i + l, j + m, k + n, VFRAC_INDX) * basisderval(l, m, n, YDIR, center, dx);
                lsgrad[ZDIR] += phi(i + l, j + m, k + n, VFRAC_INDX) * basisderval(l, m, n, ZDIR, center, dx);
            }
    double lsgrad_mag = std::sqrt(lsgrad[XDIR] * lsgrad[XDIR] + lsgrad[YDIR] * lsgrad[YDIR] + lsgrad[ZDIR] * lsgrad[ZDIR]);
    double dist = zeroval, xp[3] = {zeroval, zeroval, zeroval}, lsetnormal[3] = {zeroval, zeroval, zeroval};
    if (lsgrad_mag > TINYVAL) {
        dist = (phi(i, j, k, VFRAC_INDX) - half) / lsgrad_mag;
        for (int d = 0; d < 3; d++) {
            lsetnormal[d] = lsgrad[d] / lsgrad_mag;
            xp[d] = -dist * lsetnormal[d];
        }
    }
    phi(i, j, k, VELX_INDX) = do_interpolation_dirichlet(i, j, k, STENCILGROW, dist, closest_dist, 0.0, phi, VELX_INDX, dx);
    phi(i, j, k, VELY_INDX) = do_interpolation_dirichlet(i, j, k, STENCILGROW, dist, closest_dist, 0.0, phi, VELY_INDX, dx);
    phi(i, j, k, VELZ_INDX) = do_interpolation_dirichlet(i, j, k, STENCILGROW, dist, closest_dist, 0.0, phi, VELZ_INDX, dx);
    phi(i, j, k, PRES_INDX) = do_interpolation_hom_neumann(i, j, k, STENCILGROW, xp, phi, PRES_INDX, dx);
    if (!P->conj_ht) {
        phi(i, j, k, TEMP_INDX) = do_interpolation_hom_neumann(i, j, k, STENCILGROW, xp, phi, TEMP_INDX, dx);
    } else {
        double sumtemp = 0.0;
        int cnt = 0;
        for (int n = -1; n <= 1; n++)
            for (int m = -1; m <= 1; m++)
                for (int l = -1; l <= 1; l++)
                    if (!(l == 0 && m == 0 && n == 0)) {
                        sumtemp += phi(i + l, j + m, k + n, TEMP_INDX);
                        cnt++;
                    }
        phi(i, j, k, TEMP_INDX) = sumtemp / double(cnt);
    }
    if (!P->species_in_solid) {
        phi(i, j, k, DENS_INDX) = do_interpolation_hom_neumann(i, j, k, STENCILGROW, xp, phi, DENS_INDX, dx);
        for (int sp = 0; sp < c.nspec; sp++) {
            phi(i, j, k, FLO_NVARS + sp) = do_interpolation_hom_neumann(i, j, k, STENCILGROW, xp, phi, FLO_NVARS + sp, dx);
            consvars[NCVARS + sp] = phi(i, j, k, FLO_NVARS + sp);
        }
    } else {
        for (int sp = 0; sp < c.nspec; sp++) consvars[NCVARS + sp] = phi(i, j, k, FLO_NVARS + sp);
        phi(i, j, k, DENS_INDX) = do_interpolation_hom_neumann(i, j, k, STENCILGROW, xp, phi, DENS_INDX, dx);
    }
    primvars[DENS_IND] = phi(i, j, k, DENS_INDX);
    primvars[VELX_IND] = phi(i, j, k, VELX_INDX);
    primvars[VELY_IND] = phi(i, j, k, VELY_INDX);
    primvars[VELZ_IND] = phi(i, j, k, VELZ_INDX);
    primvars[PRES_IND] = phi(i, j, k, PRES_INDX);
    prim_to_cons(c, consvars, primvars);
    for (int q = 0; q < NCVARS; q++) phi(i, j, k, RHO_IND + q) = consvars[q];
}

// ---------------------------------------------------------------------------
// Reaction source: py_utils/rxnscheme_writer/example/chemistry.H:14-55
// (table form, rate = rateconsts[r] * prod c^|nu|).  Extension: rate constant
// A_r * exp(-Ea_r/(RU*T)) with T the cell's TEMP_INDX; Ea_r = 0 gives A_r.
// ---------------------------------------------------------------------------
inline void compute_spec_source(const Ctx& c, const double* spec, double temp, double* wdot) {
    const mfg_params* P = c.P;
    for (int sp = 0; sp < c.nspec; sp++) wdot[sp] = zeroval;
    if (!P->chem_on) return;
    for (int r = 0; r < P->nreact; r++) {
        double concmult = 1.0;
        for (int sp = 0; sp < c.nspec; sp++) {
            if (P->order[r][sp] > 0.0) concmult *= std::pow(spec[sp], P->order[r][sp]);
        }
        double kr = P->A[r];
        if (P->Ea[r] != 0.0) kr = P->A[r] * std::exp(-P->Ea[r] / (RU * temp));
        double reactrate = kr * concmult;
        for (int sp = 0; sp < c.nspec; sp++) {
            if (std::fabs(P->nu[r][sp]) > 0.0) wdot[sp] += P->nu[r][sp] * reactrate;
        }
    }
}

}  // namespace oracle
