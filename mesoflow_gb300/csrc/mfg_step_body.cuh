// Per-cell bodies of the step bookends (chemistry source and SSP-RK3
// sub-step, primitive refresh, species clipping), shared by the per-box
// launches (mfg_step.cu) and the batched launches (mfg_batch.cu).
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {
namespace {

struct Valid {
    int lo[3], len[3];
    int64_t n;
};

__host__ __device__ inline Valid valid_of(const mfg_box& b) {
    Valid v;
    v.n = 1;
    for (int d = 0; d < 3; ++d) {
        v.lo[d] = b.lo[d];
        v.len[d] = b.hi[d] - b.lo[d] + 1;
        v.n *= v.len[d];
    }
    return v;
}

__device__ __forceinline__ void cell_of(const Valid& v, int64_t t, int& i, int& j, int& k) {
    split3(t, v.len[0], v.len[1], i, j, k);
    i += v.lo[0];
    j += v.lo[1];
    k += v.lo[2];
}

// Reaction source wdot (chemistry.H compute_spec_source, table form of
// py_utils/rxnscheme_writer/example/chemistry.H:27-54).  Rate constant:
// A_r, or A_r exp(-Ea_r/(RU T)) when Ea_r != 0.  Integer reaction orders 1
// and 2 are exact products (pow(c,1) = c, pow(c,2) = c*c).
template <int NS>
__device__ __forceinline__ void spec_source(const double* spec, double temp, double* wdot) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) wdot[s] = 0.0;
    if (!P.chem_on) return;
    for (int r = 0; r < P.nreact; ++r) {
        double cm = 1.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const double o = P.order[r][s];
            if ((P.ord_mask[r] >> s) & 1u) {
                const double c = spec[s];
                cm *= (o == 1.0) ? c : (o == 2.0) ? c * c : pow(c, o);
            }
        }
        double kr = P.A[r];
        if (P.Ea[r] != 0.0) kr = P.A[r] * exp(-P.Ea[r] / (kRU * temp));
        const double rate = kr * cm;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if ((P.nu_mask[r] >> s) & 1u) wdot[s] += P.nu[r][s] * rate;
    }
}

template <int NS>
__device__ __forceinline__ void chem_source_body(const Valid& v, const Fab& S, const Fab& D, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    double spec[NS], w[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < c_P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
    spec_source<NS>(spec, S(i, j, k, TEMP), w);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < c_P.nspec) D(i, j, k, NFLO + s) = add(D(i, j, k, NFLO + s), add(0.0, w[s]));
}

// SSP-RK3 sub-step of the reaction source for one cell, all three stages in
// registers (the chemistry right-hand side is local to the cell).  Stage
// states S_i = S_old + sum_j (dt*a_ij) F_j, result S_old + sum_i (dt*w_i) F_i
// (AMReX RKIntegrator with the SSPRK3 tableau: a21=1, a31=a32=1/4,
// w=1/6,1/6,2/3).  Components without a source keep S_old.
template <int NS>
__device__ __forceinline__ void chem_substep_body(const Valid& v, const Fab& So, const Fab& Sn, double dt, int ncomp,
                                                  int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const int ns = c_P.nspec;
    double s0[NS], s1[NS], f0[NS], f1[NS], f2[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) s0[s] = (s < ns) ? So(i, j, k, NFLO + s) : 0.0;
    const double temp = So(i, j, k, TEMP);
    spec_source<NS>(s0, temp, f0);
    const double c10 = dt * 1.0, c20 = dt * 0.25, c21 = dt * 0.25;
#pragma unroll
    for (int s = 0; s < NS; ++s) s1[s] = add(s0[s], mul(c10, add(0.0, add(0.0, f0[s]))));
    spec_source<NS>(s1, temp, f1);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        s1[s] = add(add(s0[s], mul(c20, add(0.0, add(0.0, f0[s])))), mul(c21, add(0.0, add(0.0, f1[s]))));
    spec_source<NS>(s1, temp, f2);
    const double w0 = dt * (1.0 / 6.0), w1 = dt * (1.0 / 6.0), w2 = dt * (2.0 / 3.0);
    for (int n = 0; n < ncomp; ++n) {
        if (n >= NFLO) continue;
        Sn(i, j, k, n) = So(i, j, k, n);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        double r = s0[s];
        r = add(r, mul(w0, add(0.0, add(0.0, f0[s]))));
        r = add(r, mul(w1, add(0.0, add(0.0, f1[s]))));
        r = add(r, mul(w2, add(0.0, add(0.0, f2[s]))));
        Sn(i, j, k, NFLO + s) = r;
    }
}

// mflo::Advance_chemistry (Source/mflo_splitchem.cpp:177-199), the explicit
// midpoint chemistry step of the split driver.  The reference first swaps
// phi_old and phi_new, so its stage-1 source is evaluated on the previous
// phi_old (one chemistry step behind) and only the stage-2 source on the
// midpoint:
//   mid = 1*X + (dt/2) F(Y),  new = 1*X + dt F(mid),  X = s_new, Y = s_old;
// on exit s_old = X, s_new = new.  F is the reaction source on the species
// components and zero elsewhere (compute_dsdt_chemistry, :684-720), and the
// LinComb runs over every component.
template <int NS>
__device__ __forceinline__ void chem_rk2_body(const Valid& v, const Fab& So, const Fab& Sn, double dt, int ncomp,
                                              int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const int ns = c_P.nspec;
    double y[NS], f[NS], m[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) y[s] = (s < ns) ? So(i, j, k, NFLO + s) : 0.0;
    spec_source<NS>(y, So(i, j, k, TEMP), f);
    const double h = 0.5 * dt;
    // midpoint: non-species components X + h*0, species X + h F(Y)
#pragma unroll
    for (int s = 0; s < NS; ++s)
        m[s] = (s < ns) ? add(mul(1.0, Sn(i, j, k, NFLO + s)), mul(h, add(0.0, add(0.0, f[s])))) : 0.0;
    const double tmid = add(mul(1.0, Sn(i, j, k, TEMP)), mul(h, 0.0));
    spec_source<NS>(m, tmid, f);
    for (int n = 0; n < NFLO && n < ncomp; ++n) {
        const double x = Sn(i, j, k, n);
        So(i, j, k, n) = x;
        Sn(i, j, k, n) = add(mul(1.0, x), mul(dt, 0.0));
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        const double x = Sn(i, j, k, NFLO + s);
        So(i, j, k, NFLO + s) = x;
        Sn(i, j, k, NFLO + s) = add(mul(1.0, x), mul(dt, add(0.0, add(0.0, f[s]))));
    }
}

// mflo::store_inertgas_conc (Source/mflo_splitchem.cpp:150-175): fluid cells
// keep the untracked background-gas concentration in the density slot while
// the chemistry runs.
template <int NS>
__device__ __forceinline__ void inertgas_body(const Valid& v, const Fab& S, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    if (!(S(i, j, k, VFRAC) >= 1.0)) return;
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < c_P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
    S(i, j, k, DENS) = thermo_bgasconc<NS>(S(i, j, k, RHO), spec);
}

// mflo::update_vars_after_chemsolve (Source/mflo_splitchem.cpp:74-148): in
// fluid cells the density follows the new concentrations (plus the stored
// background gas when bg is set), the momenta follow density x the primitive
// velocities, the energy is kept, and the primitives and temperature are
// recomputed from the conserved state; negative pressure raises a status bit.
template <int NS>
__device__ __forceinline__ void vars_after_chem_body(const Valid& v, const Fab& S, int bg, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const DevParams& P = c_P;
    if (S(i, j, k, VFRAC) >= 1.0) {
        double spec[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
        const double rho = thermo_r_from_c<NS>(spec, bg ? S(i, j, k, DENS) : 0.0);
        S(i, j, k, RHO) = rho;
        S(i, j, k, DENS) = rho;
        const double ru = mul(rho, S(i, j, k, VELX)), rv = mul(rho, S(i, j, k, VELY)), rw = mul(rho, S(i, j, k, VELZ));
        S(i, j, k, RHOU) = ru;
        S(i, j, k, RHOV) = rv;
        S(i, j, k, RHOW) = rw;
        const double vx = ru / rho, vy = rv / rho, vz = rw / rho;
        const double rhoe = S(i, j, k, RHOE) - (0.5 * rho) * ((vx * vx + vy * vy) + vz * vz);
        const double p = thermo_p<NS>(rhoe, rho, spec);
        S(i, j, k, VELX) = vx;
        S(i, j, k, VELY) = vy;
        S(i, j, k, VELZ) = vz;
        S(i, j, k, PRES) = p;
        S(i, j, k, TEMP) = thermo_t<NS>(rho, p, spec);
    }
    if (P.do_ns && S(i, j, k, PRES) < 0.0) raise_status(MFG_STATUS_NEG_PRESSURE);
}

// cons -> prim refresh (Source/mflo_evolve.cpp:114-171); negative pressure
// raises a status bit instead of aborting.
template <int NS>
__device__ __forceinline__ void prims_body(const Valid& v, const Fab& S, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const DevParams& P = c_P;
    const double vf = S(i, j, k, VFRAC);
    if (vf == 1.0) {
        const double rho = S(i, j, k, RHO);
        double spec[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
        const double vx = S(i, j, k, RHOU) / rho, vy = S(i, j, k, RHOV) / rho, vz = S(i, j, k, RHOW) / rho;
        const double rhoe = S(i, j, k, RHOE) - (0.5 * rho) * ((vx * vx + vy * vy) + vz * vz);
        const double p = thermo_p<NS>(rhoe, rho, spec);
        S(i, j, k, DENS) = rho;
        S(i, j, k, VELX) = vx;
        S(i, j, k, VELY) = vy;
        S(i, j, k, VELZ) = vz;
        S(i, j, k, PRES) = p;
        S(i, j, k, TEMP) = thermo_t<NS>(rho, p, spec);
    } else if (P.conj_ht && vf == 0.0) {
        S(i, j, k, TEMP) = P.solid_temp;
    }
    if (P.do_ns && S(i, j, k, PRES) < 0.0) raise_status(MFG_STATUS_NEG_PRESSURE);
}

__device__ __forceinline__ void atomic_max_nonneg(double* a, double v) {
    // IEEE order of non-negative doubles equals the order of their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

// One cell's wave speed |u| + do_ns c and largest species diffusivity
// (EstTimeStep, Source/mflo_timestep.cpp:83-133), both non-negative.
template <int NS>
__device__ __forceinline__ void timestep_cell(const Fab& S, int i, int j, int k, double& ws, double& md) {
    const DevParams& P = c_P;
    ws = 0.0;
    const double vf = S(i, j, k, VFRAC);
    if (vf > 0.0) {
        const double ux = S(i, j, k, VELX), uy = S(i, j, k, VELY), uz = S(i, j, k, VELZ);
        const double fsp = sqrt((ux * ux + uy * uy) + uz * uz);
        double spec[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
        const double gam = thermo_gamma<NS>(S(i, j, k, DENS), spec);
        const double ss = sqrt((gam * S(i, j, k, PRES)) / S(i, j, k, DENS));
        ws = fsp + (double)P.do_ns * ss;
    }
    double m = blend(P.diff_mode[0], P.diff_gas[0], P.diff_solid[0], vf);
    for (int s = 0; s < P.nspec; ++s) {
        const double dd = blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf);
        if (dd > m) m = dd;
    }
    md = fabs(m);
    ws = fabs(ws);
}

__device__ __forceinline__ void clip_body(const Valid& v, const Fab& S, int nspec, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    for (int s = 0; s < nspec; ++s)
        if (S(i, j, k, NFLO + s) < 0.0) S(i, j, k, NFLO + s) = 0.0;
}

}  // namespace
}  // namespace mfg
