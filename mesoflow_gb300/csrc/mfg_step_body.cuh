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
// Rate constants of every reaction at temperature temp.
__device__ __forceinline__ void rate_constants(double temp, double* kr) {
    const DevParams& P = c_P;
    for (int r = 0; r < P.nreact; ++r) {
        kr[r] = P.A[r];
        if (P.Ea[r] != 0.0) kr[r] = P.A[r] * exp(-P.Ea[r] / (kRU * temp));
    }
}

// wdot from precomputed rate constants (the chemistry sub-steps hold the
// temperature fixed, so their stages share one set).
template <int NS>
__device__ __forceinline__ void spec_source_k(const double* spec, const double* kr, double* wdot) {
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
        const double rate = kr[r] * cm;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if ((P.nu_mask[r] >> s) & 1u) wdot[s] += P.nu[r][s] * rate;
    }
}

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

// Reaction source and its Jacobian d wdot_s / d c_q (mass action: the
// derivative of c^o is 1 for o = 1, 2c for o = 2, o c^(o-1) otherwise).
template <int NS>
__device__ __forceinline__ void spec_source_jac(const double* spec, double temp, double* wdot, double (*J)[NS]) {
    const DevParams& P = c_P;
    const int ns = P.nspec;
    for (int s = 0; s < ns; ++s) {
        wdot[s] = 0.0;
        for (int q = 0; q < ns; ++q) J[s][q] = 0.0;
    }
    if (!P.chem_on) return;
    for (int r = 0; r < P.nreact; ++r) {
        double kr = P.A[r];
        if (P.Ea[r] != 0.0) kr = P.A[r] * exp(-P.Ea[r] / (kRU * temp));
        double cm = 1.0;
        for (int s = 0; s < ns; ++s) {
            if (!((P.ord_mask[r] >> s) & 1u)) continue;
            const double o = P.order[r][s], c = spec[s];
            cm *= (o == 1.0) ? c : (o == 2.0) ? c * c : pow(c, o);
        }
        const double rate = kr * cm;
        for (int s = 0; s < ns; ++s)
            if ((P.nu_mask[r] >> s) & 1u) wdot[s] += P.nu[r][s] * rate;
        for (int q = 0; q < ns; ++q) {
            if (!((P.ord_mask[r] >> q) & 1u)) continue;
            double dr = kr;
            for (int p = 0; p < ns; ++p) {
                if (!((P.ord_mask[r] >> p) & 1u)) continue;
                const double o = P.order[r][p], c = spec[p];
                if (p == q)
                    dr *= (o == 1.0) ? 1.0 : (o == 2.0) ? 2.0 * c : o * pow(c, o - 1.0);
                else
                    dr *= (o == 1.0) ? c : (o == 2.0) ? c * c : pow(c, o);
            }
            for (int s = 0; s < ns; ++s)
                if ((P.nu_mask[r] >> s) & 1u) J[s][q] += P.nu[r][s] * dr;
        }
    }
}

// Solves W x = b in place (b -> x) for the LU factors of W (unit lower, upper,
// row exchanges piv) from lu_factor.
template <int NS>
__device__ __forceinline__ void lu_factor(double (*W)[NS], int* piv, int n) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        double amax = fabs(W[k][k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(W[i][k]) > amax) {
                amax = fabs(W[i][k]);
                p = i;
            }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < n; ++j) {
                const double t = W[k][j];
                W[k][j] = W[p][j];
                W[p][j] = t;
            }
        const double ip = 1.0 / W[k][k];
        for (int i = k + 1; i < n; ++i) {
            const double l = W[i][k] * ip;
            W[i][k] = l;
            for (int j = k + 1; j < n; ++j) W[i][j] -= l * W[k][j];
        }
    }
}

template <int NS>
__device__ __forceinline__ void lu_solve(const double (*W)[NS], const int* piv, int n, double* b) {
    for (int k = 0; k < n; ++k)
        if (piv[k] != k) {
            const double t = b[k];
            b[k] = b[piv[k]];
            b[piv[k]] = t;
        }
    for (int i = 1; i < n; ++i)
        for (int j = 0; j < i; ++j) b[i] -= W[i][j] * b[j];
    for (int i = n - 1; i >= 0; --i) {
        for (int j = i + 1; j < n; ++j) b[i] -= W[i][j] * b[j];
        b[i] /= W[i][i];
    }
}

// Implicit chemistry of one cell over dt: ROS2 (Verwer et al. 1999), L-stable,
//   (I - g h J) k1 = f(y),  (I - g h J) k2 = f(y + h k1) - 2 k1,
//   y+ = y + 3/2 h k1 + 1/2 h k2,  g = 1 + 1/sqrt(2),
// with the embedded first-order error y+ - (y + h k1) = h (k1 + k2) / 2, the
// RMS norm of err / (atol + rtol max(|y|, |y+|)), acceptance at <= 1 and the
// step factor min(5, max(0.2, 0.9 / sqrt(norm))).  Returns false (and raises
// MFG_STATUS_CHEM_STEPS) after chem_maxsub attempts.
template <int NS>
__device__ bool chem_ros2_cell(double* y, double temp, double dt) {
    const DevParams& P = c_P;
    const int ns = P.nspec;
    const double g = 1.7071067811865475;
    double W[NS][NS], f0[NS], k1[NS], k2[NS], y1[NS];
    int piv[NS];
    double t = 0.0, h = dt;
    for (int att = 0; att < P.chem_maxsub; ++att) {
        bool last = false;
        if (t + h >= dt) {
            h = dt - t;
            last = true;
        }
        spec_source_jac<NS>(y, temp, f0, W);
        for (int s = 0; s < ns; ++s) {
            for (int q = 0; q < ns; ++q) W[s][q] = -(g * h) * W[s][q];
            W[s][s] += 1.0;
        }
        lu_factor<NS>(W, piv, ns);
        for (int s = 0; s < ns; ++s) k1[s] = f0[s];
        lu_solve<NS>(W, piv, ns, k1);
        for (int s = 0; s < ns; ++s) y1[s] = y[s] + h * k1[s];
        spec_source<NS>(y1, temp, k2);
        for (int s = 0; s < ns; ++s) k2[s] -= 2.0 * k1[s];
        lu_solve<NS>(W, piv, ns, k2);
        double e2 = 0.0;
        for (int s = 0; s < ns; ++s) {
            const double yn = y[s] + (1.5 * h) * k1[s] + (0.5 * h) * k2[s];
            const double err = (0.5 * h) * (k1[s] + k2[s]);
            const double sc = P.chem_atol + P.chem_rtol * fmax(fabs(y[s]), fabs(yn));
            e2 += (err / sc) * (err / sc);
            y1[s] = yn;
        }
        const double en = sqrt(e2 / (double)ns);
        if (en <= 1.0) {
            for (int s = 0; s < ns; ++s) y[s] = y1[s];
            t += h;
            if (last) return true;
        }
        const double fac = (en > 0.0) ? fmin(5.0, fmax(0.2, 0.9 / sqrt(en))) : 5.0;
        h *= fac;
    }
    raise_status(MFG_STATUS_CHEM_STEPS);
    return false;
}

// SSP-RK3 sub-step of the reaction source for one cell, all three stages in
// registers (the chemistry right-hand side is local to the cell).  Stage
// states S_i = S_old + sum_j (dt*a_ij) F_j, result S_old + sum_i (dt*w_i) F_i
// (AMReX RKIntegrator with the SSPRK3 tableau: a21=1, a31=a32=1/4,
// w=1/6,1/6,2/3).  Components without a source keep S_old.
// Species of one cell after the explicit SSP-RK3 chemistry sub-step over dt
// from s0 (the reference's AMReX TimeIntegrator, rk.type 3: nodes 0, 1, 1/2;
// a21 = 1, a31 = a32 = 1/4; weights 1/6, 1/6, 2/3), or after the implicit
// ROS2 sub-step; the flow components are not changed by it.
template <int NS>
__device__ __forceinline__ void chem_species(const double* s0, double temp, double dt, double* out) {
    const int ns = c_P.nspec;
    if (c_P.chem_kind == 1) {  // implicit (ROS2) chemistry
#pragma unroll
        for (int s = 0; s < NS; ++s) out[s] = s0[s];
        chem_ros2_cell<NS>(out, temp, dt);
        return;
    }
    double s1[NS], f0[NS], f1[NS], f2[NS];
    double kr[MAXR];
    rate_constants(temp, kr);
    spec_source_k<NS>(s0, kr, f0);
    const double c10 = dt * 1.0, c20 = dt * 0.25, c21 = dt * 0.25;
#pragma unroll
    for (int s = 0; s < NS; ++s) s1[s] = add(s0[s], mul(c10, add(0.0, add(0.0, f0[s]))));
    spec_source_k<NS>(s1, kr, f1);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        s1[s] = add(add(s0[s], mul(c20, add(0.0, add(0.0, f0[s])))), mul(c21, add(0.0, add(0.0, f1[s]))));
    spec_source_k<NS>(s1, kr, f2);
    const double w0 = dt * (1.0 / 6.0), w1 = dt * (1.0 / 6.0), w2 = dt * (2.0 / 3.0);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        double r = s0[s];
        r = add(r, mul(w0, add(0.0, add(0.0, f0[s]))));
        r = add(r, mul(w1, add(0.0, add(0.0, f1[s]))));
        r = add(r, mul(w2, add(0.0, add(0.0, f2[s]))));
        out[s] = r;
    }
}

template <int NS>
__device__ __forceinline__ void chem_substep_body(const Valid& v, const Fab& So, const Fab& Sn, double dt, int ncomp,
                                                  int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const int ns = c_P.nspec;
    double s0[NS], s1[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) s0[s] = (s < ns) ? So(i, j, k, NFLO + s) : 0.0;
    chem_species<NS>(s0, So(i, j, k, TEMP), dt, s1);
    for (int n = 0; n < ncomp; ++n) {
        if (n >= NFLO) continue;
        Sn(i, j, k, n) = So(i, j, k, n);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < ns) Sn(i, j, k, NFLO + s) = s1[s];
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
// update_primitive_vars of one cell held in registers (u: the NFLO flow
// components, spec: the species), Source/mflo_evolve.cpp:114-171: in gas cells
// the primitives from the conserved variables, in solid cells of a conjugate
// heat transfer run the solid temperature; a negative pressure raises the
// sticky status.  Returns a bit mask of the flow components it wrote.
template <int NS>
__device__ __forceinline__ unsigned prims_cell(double* u, const double* spec) {
    const DevParams& P = c_P;
    const double vf = u[VFRAC];
    unsigned wrote = 0;
    // the volume-fraction, pressure and finiteness tests of the bookends run
    // on the integer pipe (the FP64 pipe bounds this kernel)
    if (is_one(vf)) {
        const double rho = u[RHO];
        // one Newton-refined reciprocal of the (positive) density for the three
        // velocities and the mass-single temperature instead of four divisions
        const double irho = rcp_pos(rho);
        const double vx = u[RHOU] * irho, vy = u[RHOV] * irho, vz = u[RHOW] * irho;
        const double rhoe = u[RHOE] - (0.5 * rho) * ((vx * vx + vy * vy) + vz * vz);
        const double p = thermo_p<NS>(rhoe, rho, spec);
        u[DENS] = rho;
        u[VELX] = vx;
        u[VELY] = vy;
        u[VELZ] = vz;
        u[PRES] = p;
        // p / R / rho of the mass-single family as (p / rho) / R with the
        // reciprocals above and from mfg_init (a few ulp from the two divisions)
        u[TEMP] = (P.thermo_kind == MFG_THERMO_MASS_SINGLE) ? (p * irho) * P.inv_gas_R : thermo_t<NS>(rho, p, spec);
        wrote = (1u << DENS) | (1u << VELX) | (1u << VELY) | (1u << VELZ) | (1u << PRES) | (1u << TEMP);
    } else if (P.conj_ht && is_zero_bits(vf)) {
        u[TEMP] = P.solid_temp;
        wrote = 1u << TEMP;
    }
    if (P.do_ns && is_negative(u[PRES])) raise_status(MFG_STATUS_NEG_PRESSURE);
    return wrote;
}

template <int NS>
__device__ __forceinline__ void prims_body(const Valid& v, const Fab& S, int64_t t) {
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    double u[NFLO], spec[NS];
#pragma unroll
    for (int n = 0; n < NFLO; ++n) u[n] = S(i, j, k, n);
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < c_P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
    const unsigned wrote = prims_cell<NS>(u, spec);
#pragma unroll
    for (int n = DENS; n <= TEMP; ++n)
        if ((wrote >> n) & 1u) S(i, j, k, n) = u[n];
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

// The step's bookends of one cell after the three RK3 stages, fused
// (Source/mflo_evolve.cpp:33-58, 470-493, 521-540, 91-112): with chem,
// phi_old <- phi_new and the chemistry sub-step phi_new = chem(phi_old); the
// primitive refresh; species clipping when clip.  With NORMS the
// residual-norm terms ((a s_new + b s_old) [* old vfrac for the flow
// components])^2 of every component are added to acc[n].  Reads the
// cell's components once and writes only what changes.  With chem, s_old is
// the incoming s_new, so the components the bookends leave alone (the
// conserved flow variables and the volume fraction) have the term
// (a u + b u)^2 = 0 exactly (b = -a), NaN where u is not finite: only
// nonfinite is raised for them.
// CHEM: 0 no sub-step (only_flow), 1 the explicit sub-step of a zero source
// (no reactions: each species becomes s + 0, which is what the RK3 stages
// compute then), 2 the sub-step of chem_species.
template <int NS, int CHEM, bool NORMS>
__device__ __forceinline__ void post_cell(const Fab& So, const Fab& Sn, int i, int j, int k, double dt, bool clip,
                                          double a, double b, double* acc, bool& nonfinite) {
    constexpr bool chem = CHEM != 0;
    const int ns = c_P.nspec;
    double u[NFLO], spec[NS];
#pragma unroll
    for (int n = 0; n < NFLO; ++n) u[n] = Sn(i, j, k, n);
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? Sn(i, j, k, NFLO + s) : 0.0;
    double o6[TEMP - DENS + 1], os[NS];  // with chem: the old values the bookends change
    if (chem) {
#pragma unroll
        for (int n = 0; n < NFLO; ++n) So(i, j, k, n) = u[n];
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < ns) So(i, j, k, NFLO + s) = spec[s];
#pragma unroll
        for (int n = DENS; n <= TEMP; ++n) o6[n - DENS] = u[n];
#pragma unroll
        for (int s = 0; s < NS; ++s) os[s] = spec[s];
        if (CHEM == 2) {
            double s1[NS];
            chem_species<NS>(spec, u[TEMP], dt, s1);
#pragma unroll
            for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? s1[s] : 0.0;
        } else {
#pragma unroll
            for (int s = 0; s < NS; ++s) spec[s] = plus_zero(spec[s]);
        }
    }
    const unsigned wrote = prims_cell<NS>(u, spec);
#pragma unroll
    for (int n = DENS; n <= TEMP; ++n)
        if ((wrote >> n) & 1u) Sn(i, j, k, n) = u[n];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        const bool neg = is_negative(spec[s]);
        if (clip && neg) spec[s] = 0.0;
        // stored when the sub-step or the clipping may have changed it
        if (chem || (clip && neg)) Sn(i, j, k, NFLO + s) = spec[s];
    }
    if (!NORMS) return;
    // LinComb then Multiply, rounded as the reference (no contraction); acc
    // holds one running sum per component in registers
    const double vfo = chem ? u[VFRAC] : So(i, j, k, VFRAC);
#pragma unroll
    for (int n = 0; n < NFLO; ++n) {
        const bool changed = n >= DENS && n <= TEMP;
        if (chem && !changed) {  // (a u + b u)^2 = 0 unless u is not finite
            nonfinite |= !is_finite_bits(u[n]);
            continue;
        }
        const double on = chem ? o6[changed ? n - DENS : 0] : So(i, j, k, n);
        double d = add(mul(a, u[n]), mul(b, on));
        if (n < VFRAC) d = mul(d, vfo);
        acc[n] += d * d;
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        const double on = chem ? os[s] : So(i, j, k, NFLO + s);
        const double d = add(mul(a, spec[s]), mul(b, on));
        acc[NFLO + s] += d * d;
    }
}

}  // namespace
}  // namespace mfg
