// Hand-written FP64 discrete adjoint of the single-level step of
// mfg_advance_level (fill patch, cut cells, WENO5 right-hand side and RK3
// stage algebra x 3, SSP-RK3 chemistry sub-step, primitive refresh, species
// clipping), for the gradients of the integrated surface reaction rate
//     J = V_cell * sum_cells sum_r k_r(T) prod_j c_j^{o_rj}
// on the state after n steps with respect to the log pre-exponentials log A_r
// and the normal velocity of the velocity-inlet boundaries.
//
// Reverse sweep of one step, each phase's vector-Jacobian product written out:
//   clipping -> primitive refresh -> chemistry sub-step (per cell, the three
//   SSP-RK3 stages in reverse) -> for stage 3, 2, 1: stage algebra with the
//   update_residual mask, face fluxes (WENO5-JS edges, LLF eigenvalue, Euler
//   fluxes, viscous stress, heat conduction, species diffusion), per-cell
//   primitives, cut cells (the inverse-distance weights depend on the volume
//   fraction only, which the dynamics never changes), ghost fill (physical
//   boundaries corners -> edges -> faces, then the copies from the owners).
// Face and cell contributions are scattered with FP64 atomics, so gradients
// agree between runs to rounding, not bitwise.  Forward intermediates are
// recomputed: the state is kept every checkpoint_every steps, the steps of a
// segment are re-run to recover their start states, and each step is re-run
// once more, saving its three stage states, just before its reverse.
//
// Scope: WENO5 (order_hyp 5) with Navier-Stokes terms, molar or mass-single
// thermo, constant viscosity and conductivity (diffusivities may blend with
// the volume fraction), no conjugate heat transfer, boundaries periodic,
// foextrap, wall, or ext_dir with a velocity inlet or a fixed state.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mfg_fill_body.cuh"
#include "mfg_ib_body.cuh"
#include "mfg_rhs_body.cuh"
#include "mfg_step_body.cuh"

namespace mfg {

cudaError_t launch_cutcells_box(const mfg_box& b, const mfg_geom& g, double* tcht_scratch, int* list,
                                unsigned* count, cudaStream_t st);
cudaError_t launch_chem_substep(const mfg_box& b, double dt, cudaStream_t st);

namespace {

constexpr int AT = 128;
constexpr double kK1 = 13.0 / 12.0;

// ---------------------------------------------------------------------------
// thermodynamic partial derivatives (molar and mass-single families; neither
// pressure law depends on rho)
// ---------------------------------------------------------------------------
// p(rhoe, c): dp/drhoe and dp/dc_k
template <int NS>
__device__ void dpres(double rhoe, const double* c, double& dp_drhoe, double* dp_dc) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) dp_dc[s] = 0.0;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) {
        dp_drhoe = P.gm1_single;
        return;
    }
    double cvs = 0.0, S = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) {
            cvs += P.cv[s] * c[s];
            S += c[s];
        }
    const double icvs = 1.0 / cvs;
    const double T = rhoe * icvs;
    dp_drhoe = P.R_univ * S * icvs;
    const double RT = P.R_univ * T, Sic = S * icvs;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) dp_dc[s] = RT * (1.0 - Sic * P.cv[s]);
}

// dgamma/dc_k of gamma = 1 + 1/A, A = sum_s (c_s/S)/(gamma_s - 1)
template <int NS>
__device__ void dgamma(const double* c, double* dg_dc) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) dg_dc[s] = 0.0;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) return;
    // 1/(gamma_s - 1) = cv_s / R for the molar families
    double S = 0.0, Ac = 0.0;
    const double iR = 1.0 / P.R_univ;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) {
            S += c[s];
            Ac += c[s] * P.cv[s];
        }
    const double iS = 1.0 / S;
    const double A = Ac * iR * iS;
    const double k = -iS / (A * A);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) dg_dc[s] = k * (P.cv[s] * iR - A);
}

// T(rho, p, c) partials
template <int NS>
__device__ void dtemp(double rho, double p, const double* c, double& dT_dp, double& dT_drho, double* dT_dc) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) dT_dc[s] = 0.0;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) {
        dT_dp = 1.0 / (P.gas_R * rho);
        dT_drho = -(p / P.gas_R / rho) / rho;
        return;
    }
    double S = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) S += c[s];
    const double T = p / (S * P.R_univ);
    dT_dp = 1.0 / (S * P.R_univ);
    dT_drho = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) dT_dc[s] = -T / S;
}

// e(rho, p, c) with its partials
template <int NS>
__device__ double de_int(double rho, double p, const double* c, double& de_drho, double& de_dp, double* de_dc) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) de_dc[s] = 0.0;
    if (P.thermo_kind == MFG_THERMO_MASS_SINGLE) {
        const double e = p / (P.gamma_single - 1.0) / rho;
        de_dp = 1.0 / ((P.gamma_single - 1.0) * rho);
        de_drho = -e / rho;
        return e;
    }
    double S = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) S += c[s];
    const double T = p / (S * P.R_univ);
    if (P.energy_form == MFG_EFORM_MASS_CV) {
        double cvbar = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) cvbar += P.cvmass[s] * (c[s] / S);
        de_dp = cvbar / (S * P.R_univ);
        de_drho = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.ngas) de_dc[s] = T * (P.cvmass[s] - 2.0 * cvbar) / S;
        return cvbar * T;
    }
    double scv = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) scv += P.cv[s] * c[s];
    const double e = scv * T / rho;
    de_dp = scv / (S * P.R_univ * rho);
    de_drho = -e / rho;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < P.ngas) de_dc[s] = (T / rho) * (P.cv[s] - scv / S);
    return e;
}

// Atomic add that skips +-0 (tested on the integer pipe: the FP64 pipe bounds these kernels).
__device__ __forceinline__ void aadd(double* p, double v) {
    if ((__double_as_longlong(v) << 1) != 0) atomicAdd(p, v);
}

// ---------------------------------------------------------------------------
// WENO5-JS edge (one-division normalisation) and its vector-Jacobian product;
// returns the edge value, writes d(ob * edge)/d(a..e) to g.
// ---------------------------------------------------------------------------
struct EdgeGrad {
    double a, b, c, d, e;
};

__device__ __forceinline__ double weno_edge_vjp(double a, double b, double c, double d, double e, double ob,
                                                EdgeGrad& g) {
    const double t2 = (a - 2.0 * b) + c, u2 = (a - 4.0 * b) + 3.0 * c;
    const double t1 = (b - 2.0 * c) + d, q1 = b - d;
    const double t0 = (c - 2.0 * d) + e, u0 = (3.0 * c - 4.0 * d) + e;
    const double s2 = kEpsWeno + (kK1 * (t2 * t2) + 0.25 * (u2 * u2));
    const double s1 = kEpsWeno + (kK1 * (t1 * t1) + (0.25 * q1) * q1);
    const double s0 = kEpsWeno + (kK1 * (t0 * t0) + 0.25 * (u0 * u0));
    const double v2 = (2.0 * a - 7.0 * b) + 11.0 * c;
    const double v1 = (-b + 5.0 * c) + 2.0 * d;
    const double v0 = (2.0 * c + 5.0 * d) - e;
    const double D2 = s2 * s2, D1 = s1 * s1, D0 = s0 * s0;
    const double e2 = D1 * D0, e1 = 6.0 * (D2 * D0), e0 = 3.0 * (D2 * D1);
    const double num = (e2 * v2 + e1 * v1) + e0 * v0;
    const double den = (e2 + e1) + e0;
    const double r6 = rcp_pos(6.0 * den);  // den > 0: a sum of products of squares of eps + b_k
    const double out = num * r6;
    const double nb = ob * r6;
    const double db = -(nb * 6.0) * out;
    const double e2b = nb * v2 + db, e1b = nb * v1 + db, e0b = nb * v0 + db;
    const double v2b = nb * e2, v1b = nb * e1, v0b = nb * e0;
    // D_k = s_k^2, s_k = eps + K1 t^2 + u^2/4:  d/dt = 4 K1 s_k t D_k_bar, d/du = s_k u D_k_bar
    const double P2 = (e1b * (6.0 * D0) + e0b * (3.0 * D1)) * s2;
    const double P1 = (e2b * D0 + e0b * (3.0 * D2)) * s1;
    const double P0 = (e2b * D1 + e1b * (6.0 * D2)) * s0;
    const double t2b = P2 * ((4.0 * kK1) * t2), u2b = P2 * u2;
    const double t1b = P1 * ((4.0 * kK1) * t1), q1b = P1 * q1;
    const double t0b = P0 * ((4.0 * kK1) * t0), u0b = P0 * u0;
    g.a = (t2b + u2b) + 2.0 * v2b;
    g.b = ((-2.0 * t2b - 4.0 * u2b) + (t1b + q1b)) - (7.0 * v2b + v1b);
    g.c = ((t2b + 3.0 * u2b) + (-2.0 * t1b) + (t0b + 3.0 * u0b)) + ((11.0 * v2b + 5.0 * v1b) + 2.0 * v0b);
    g.d = ((t1b - q1b) + (-2.0 * t0b - 4.0 * u0b)) + (2.0 * v1b + 5.0 * v0b);
    g.e = (t0b + u0b) - v0b;
    return out;
}

// ---------------------------------------------------------------------------
// right-hand side reversed
// ---------------------------------------------------------------------------
struct AdjBox {
    RhsBox B;    // forward views: sb = the stage state after cut cells, aux = its per-cell scalars
    Fab lamL;    // adjoint of the masked dsdt (valid cells, all components)
    Fab lamSb;   // adjoint of the stage state (grown by 3, all components)
    Fab lamAux;  // adjoint of the per-cell scalars (grown by 3, NAUX components)
};

// d(dsdt)/dF: dsdt(cell) = (F(face lo) - F(face hi))/dx, so the adjoint of
// face f's flux of state component sc is (lamL(right cell) - lamL(left cell))/dx.
__device__ __forceinline__ double face_bar(const RhsBox& B, const Fab& LL, const Idx3& f, int d, int sc) {
    const int fd = (d == 0) ? f.i : (d == 1) ? f.j : f.k;
    const int64_t ld = (d == 0) ? 1 : (d == 1) ? LL.js : LL.ks;
    const int64_t lR = LL.off(f.i, f.j, f.k) + sc * LL.ns;
    double v = 0.0;
    if (fd <= B.hi[d]) v += LL.p[lR];
    if (fd - 1 >= B.lo[d]) v -= LL.p[lR - ld];
    return v * B.idx[d];
}

// One thread per (face of direction d, advected component c)
// (compute_flux_3d.H:88-430 for order 5): the component's hyperbolic flux
// fh = (fp + lam up)/2 + (fm - lam um)/2 reversed through the WENO5 edges of
// the state (up, um) and of the Euler fluxes (fp, fm), the Euler flux of each
// stencil cell (consprim_funcs.H:48-81), species diffusion and heat
// conduction.  The eigenvalue's adjoint is summed per face into FS_MH.
template <int NS>
__global__ void __launch_bounds__(AT, 4) adj_flux_kernel(AdjBox A, int d) {
    const RhsBox& B = A.B;
    const int c = blockIdx.y;
    int len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    const int64_t nf = (int64_t)len[0] * len[1] * len[2];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf) return;
    const Idx3 f = delinear(t, B.lo, len);
    const DevParams& P = c_P;
    const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
    const double Fb = face_bar(B, A.lamL, f, d, sc);
    if (Fb == 0.0) return;
    const Fab& S = B.sb;
    const Fab& G = A.lamSb;
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t oR = S.off(f.i, f.j, f.k), oL = oR - sd;
    if (c == RHOE) {  // heat conduction F_E -= k (T_R - T_L)/dx, on every face
        const double kb = P.cond_hm * B.idx[d] * Fb;
        aadd(&G.p[oR + TEMP * G.ns], -kb);
        aadd(&G.p[oL + TEMP * G.ns], kb);
    }
    if (c >= NCONS) {  // species diffusion F_s -= D (c_R - c_L)/dx, on every face
        const int s = c - NCONS;
        const double* vf = S.p + VFRAC * S.ns;
        const double Dh = (P.diff_mode[s] == MFG_TRANSPORT_CONST)
                              ? P.diff_hm[s]
                              : harmonic_mean(blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oL]),
                                              blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oR]));
        const double v = Dh * B.idx[d] * Fb;
        aadd(&G.p[oR + sc * G.ns], -v);
        aadd(&G.p[oL + sc * G.ns], v);
    }
    const Fab& FS = B.fs[d];
    const int64_t qf = FS.off(f.i, f.j, f.k);
    const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
    if (!(flags & 1)) return;
    const double hb = (c < NCONS) ? Fb : P.advect_flag[c - NCONS] * Fb;
    if (hb == 0.0) return;
    const bool fallback = flags & 2;
    const double lam = FS.p[qf + FS_LAMBDA * FS.ns];
    const Fab& X = B.aux;
    const Fab& GA = A.lamAux;
    const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
    const int64_t xR = X.off(f.i, f.j, f.k);
    double us[6], fl[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int cq = fallback ? ((q < 3) ? -1 : 0) : q - 3;
        const int64_t os = oR + cq * sd, ox = xR + cq * xd;
        us[q] = S.p[os + sc * S.ns];
        const double va = (c >= 1 && c <= 3) ? X.p[ox + (AUX_VX + c - 1) * X.ns] : 0.0;
        fl[q] = euler_flux(c, d, us[q], S.p[os + RHO * S.ns], va, X.p[ox + (AUX_VX + d) * X.ns],
                           X.p[ox + AUX_PF * X.ns], S.p[os + RHOE * S.ns]);
    }
    EdgeGrad g;
    double usb[6] = {0, 0, 0, 0, 0, 0}, flb[6] = {0, 0, 0, 0, 0, 0};
    weno_edge_vjp(fl[0], fl[1], fl[2], fl[3], fl[4], 0.5 * hb, g);
    flb[0] += g.a; flb[1] += g.b; flb[2] += g.c; flb[3] += g.d; flb[4] += g.e;
    weno_edge_vjp(fl[5], fl[4], fl[3], fl[2], fl[1], 0.5 * hb, g);
    flb[5] += g.a; flb[4] += g.b; flb[3] += g.c; flb[2] += g.d; flb[1] += g.e;
    const double up = weno_edge_vjp(us[0], us[1], us[2], us[3], us[4], 0.5 * lam * hb, g);
    usb[0] += g.a; usb[1] += g.b; usb[2] += g.c; usb[3] += g.d; usb[4] += g.e;
    const double um = weno_edge_vjp(us[5], us[4], us[3], us[2], us[1], -0.5 * lam * hb, g);
    usb[5] += g.a; usb[4] += g.b; usb[3] += g.c; usb[2] += g.d; usb[1] += g.e;
    aadd(&FS.p[qf + FS_MH * FS.ns], 0.5 * hb * (up - um));
    // with the first-order fallback the six stencil entries are two cells: sum first
    int q0 = 0, nq = 6;
    if (fallback) {
        usb[2] = (usb[0] + usb[1]) + usb[2];
        flb[2] = (flb[0] + flb[1]) + flb[2];
        usb[3] = (usb[3] + usb[4]) + usb[5];
        flb[3] = (flb[3] + flb[4]) + flb[5];
        q0 = 2;
        nq = 4;
    }
    for (int q = q0; q < nq; ++q) {
        const int cq = q - 3;
        const int64_t os = oR + cq * sd, ox = xR + cq * xd;
        const double fb = flb[q];
        const double vd = X.p[ox + (AUX_VX + d) * X.ns];
        double ub = usb[q], rb = 0.0, vab = 0.0, vdb = 0.0, pb = 0.0, Eb = 0.0;
        if (c == RHO) {
            rb = fb * vd;
            vdb = fb * us[q];
        } else if (c <= RHOW) {
            const double rho = S.p[os + RHO * S.ns], va = X.p[ox + (AUX_VX + c - 1) * X.ns];
            rb = fb * va * vd;
            vab = fb * rho * vd;
            vdb = fb * rho * va;
            if (c - 1 == d) pb = fb;
        } else if (c == RHOE) {
            Eb = fb * vd;
            pb = fb * vd;
            vdb = fb * (us[q] + X.p[ox + AUX_PF * X.ns]);
        } else {
            ub += fb * vd;
            vdb = fb * us[q];
        }
        if (c == RHO) ub += rb;
        if (c == RHOE) ub += Eb;
        aadd(&G.p[os + sc * G.ns], ub);
        if (c != RHO) aadd(&G.p[os + RHO * G.ns], rb);
        if (c != RHOE) aadd(&G.p[os + RHOE * G.ns], Eb);
        aadd(&GA.p[ox + (AUX_VX + d) * GA.ns], vdb);
        if (c >= 1 && c <= 3) aadd(&GA.p[ox + (AUX_VX + c - 1) * GA.ns], vab);
        aadd(&GA.p[ox + AUX_PF * GA.ns], pb);
    }
}

// Adjoint of one stencil cell's Euler flux of component c and of its state
// value (consprim_funcs.H:48-81 reversed), given the summed adjoints fb of the
// flux and ub of the state value from the WENO5 edges.
__device__ __forceinline__ void euler_vjp_scatter(const AdjBox& A, int c, int d, int sc, int64_t os, int64_t ox,
                                                  double u, double fb, double ub) {
    const RhsBox& B = A.B;
    const Fab& S = B.sb;
    const Fab& X = B.aux;
    const Fab& G = A.lamSb;
    const Fab& GA = A.lamAux;
    const double vd = X.p[ox + (AUX_VX + d) * X.ns];
    double rb = 0.0, vab = 0.0, vdb = 0.0, pb = 0.0, Eb = 0.0;
    if (c == RHO) {
        rb = fb * vd;
        vdb = fb * u;
    } else if (c <= RHOW) {
        const double rho = S.p[os + RHO * S.ns], va = X.p[ox + (AUX_VX + c - 1) * X.ns];
        rb = fb * va * vd;
        vab = fb * rho * vd;
        vdb = fb * rho * va;
        if (c - 1 == d) pb = fb;
    } else if (c == RHOE) {
        Eb = fb * vd;
        pb = fb * vd;
        vdb = fb * (u + X.p[ox + AUX_PF * X.ns]);
    } else {
        ub += fb * vd;
        vdb = fb * u;
    }
    if (c == RHO) ub += rb;
    if (c == RHOE) ub += Eb;
    aadd(&G.p[os + sc * G.ns], ub);
    if (c != RHO) aadd(&G.p[os + RHO * G.ns], rb);
    if (c != RHOE) aadd(&G.p[os + RHOE * G.ns], Eb);
    aadd(&GA.p[ox + (AUX_VX + d) * GA.ns], vdb);
    if (c >= 1 && c <= 3) aadd(&GA.p[ox + (AUX_VX + c - 1) * GA.ns], vab);
    aadd(&GA.p[ox + AUX_PF * GA.ns], pb);
}

// Column-sweep form of adj_flux_kernel: one thread per (segment of seg faces
// along d in one column, advected component c).  A window of the six stencil
// cells slides with the face; each cell's state value and Euler flux are
// evaluated once, the edge adjoints of the faces that use the cell are summed
// in registers, and the Euler-flux reversal and its atomic scatter run once
// per cell as it leaves the window (cells at the segment ends also receive
// the neighbouring segments' sums, so the scatter stays atomic).  Same
// mathematics as the per-face form; the order of the summation differs.
template <int NS>
__device__ __forceinline__ void adj_flux_sweep_body(const AdjBox& A, int d, int seg, int c, int64_t t) {
    const RhsBox& B = A.B;
    int ta, tb;
    sweep_dirs(d, ta, tb);
    const int na = B.hi[ta] - B.lo[ta] + 1, nb = B.hi[tb] - B.lo[tb] + 1;
    const int nseg = sweep_nseg(B, d, seg);
    if (t >= (int64_t)na * nb * nseg) return;
    int ia, ib, is;
    split3(t, na, nb, ia, ib, is);
    const int nfd = B.hi[d] - B.lo[d] + 2;
    const int f0 = B.lo[d] + is * seg, f1 = B.lo[d] + min(nfd, (is + 1) * seg);  // faces [f0, f1)
    const DevParams& P = c_P;
    const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
    const Fab& S = B.sb;
    const Fab& X = B.aux;
    const Fab& G = A.lamSb;
    const Fab& FS = B.fs[d];
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
    Idx3 f;
    int* fc[3] = {&f.i, &f.j, &f.k};
    *fc[ta] = B.lo[ta] + ia;
    *fc[tb] = B.lo[tb] + ib;
    *fc[d] = f0;
    // window: position q holds cell (face - 3 + q)
    double us[6], fl[6], usb[6], flb[6];
    const int64_t oR0 = S.off(f.i, f.j, f.k), xR0 = X.off(f.i, f.j, f.k);
    auto load = [&](int q, int64_t os, int64_t ox) {
        us[q] = S.p[os + sc * S.ns];
        const double va = (c >= 1 && c <= 3) ? X.p[ox + (AUX_VX + c - 1) * X.ns] : 0.0;
        fl[q] = euler_flux(c, d, us[q], S.p[os + RHO * S.ns], va, X.p[ox + (AUX_VX + d) * X.ns],
                           X.p[ox + AUX_PF * X.ns], S.p[os + RHOE * S.ns]);
        usb[q] = 0.0;
        flb[q] = 0.0;
    };
#pragma unroll
    for (int q = 0; q < 6; ++q) load(q, oR0 + (q - 3) * sd, xR0 + (q - 3) * xd);
    for (int fd = f0; fd < f1; ++fd) {
        *fc[d] = fd;
        const int64_t oR = oR0 + (fd - f0) * sd, oL = oR - sd, xR = xR0 + (fd - f0) * xd;
        const double Fb = face_bar(B, A.lamL, f, d, sc);
        if (Fb != 0.0) {
            if (c == RHOE) {  // heat conduction F_E -= k (T_R - T_L)/dx, on every face
                const double kb = P.cond_hm * B.idx[d] * Fb;
                aadd(&G.p[oR + TEMP * G.ns], -kb);
                aadd(&G.p[oL + TEMP * G.ns], kb);
            }
            if (c >= NCONS) {  // species diffusion F_s -= D (c_R - c_L)/dx, on every face
                const int s = c - NCONS;
                const double* vf = S.p + VFRAC * S.ns;
                const double Dh = (P.diff_mode[s] == MFG_TRANSPORT_CONST)
                                      ? P.diff_hm[s]
                                      : harmonic_mean(blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oL]),
                                                      blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oR]));
                const double v = Dh * B.idx[d] * Fb;
                aadd(&G.p[oR + sc * G.ns], -v);
                aadd(&G.p[oL + sc * G.ns], v);
            }
            const int64_t qf = FS.off(f.i, f.j, f.k);
            const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
            const double hb = (c < NCONS) ? Fb : P.advect_flag[c - NCONS] * Fb;
            if ((flags & 1) && hb != 0.0) {
                const bool fallback = flags & 2;
                const double lam = FS.p[qf + FS_LAMBDA * FS.ns];
                // the same four edge reversals for every lane (with the first-order
                // fallback the six stencil entries are the two face cells), then the
                // stencil adjoints are added to the window, collapsed for the fallback
                double sf[6], su[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const int w = fallback ? ((q < 3) ? 2 : 3) : q;
                    sf[q] = fl[w];
                    su[q] = us[w];
                }
                double gf[6] = {0, 0, 0, 0, 0, 0}, gu[6] = {0, 0, 0, 0, 0, 0};
                EdgeGrad g;
                weno_edge_vjp(sf[0], sf[1], sf[2], sf[3], sf[4], 0.5 * hb, g);
                gf[0] += g.a; gf[1] += g.b; gf[2] += g.c; gf[3] += g.d; gf[4] += g.e;
                weno_edge_vjp(sf[5], sf[4], sf[3], sf[2], sf[1], 0.5 * hb, g);
                gf[5] += g.a; gf[4] += g.b; gf[3] += g.c; gf[2] += g.d; gf[1] += g.e;
                const double up = weno_edge_vjp(su[0], su[1], su[2], su[3], su[4], 0.5 * lam * hb, g);
                gu[0] += g.a; gu[1] += g.b; gu[2] += g.c; gu[3] += g.d; gu[4] += g.e;
                const double um = weno_edge_vjp(su[5], su[4], su[3], su[2], su[1], -0.5 * lam * hb, g);
                gu[5] += g.a; gu[4] += g.b; gu[3] += g.c; gu[2] += g.d; gu[1] += g.e;
                if (fallback) {
                    flb[2] += (gf[0] + gf[1]) + gf[2];
                    flb[3] += (gf[3] + gf[4]) + gf[5];
                    usb[2] += (gu[0] + gu[1]) + gu[2];
                    usb[3] += (gu[3] + gu[4]) + gu[5];
                } else {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        flb[q] += gf[q];
                        usb[q] += gu[q];
                    }
                }
                aadd(&FS.p[qf + FS_MH * FS.ns], 0.5 * hb * (up - um));
            }
        }
        if (fd + 1 < f1) {  // cell fd - 3 leaves the window; cell fd + 3 enters
            if (usb[0] != 0.0 || flb[0] != 0.0)
                euler_vjp_scatter(A, c, d, sc, oR - 3 * sd, xR - 3 * xd, us[0], flb[0], usb[0]);
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                us[q] = us[q + 1];
                fl[q] = fl[q + 1];
                usb[q] = usb[q + 1];
                flb[q] = flb[q + 1];
            }
            load(5, oR + 3 * sd, xR + 3 * xd);
        }
    }
    const int64_t oR = oR0 + (f1 - 1 - f0) * sd, xR = xR0 + (f1 - 1 - f0) * xd;
#pragma unroll
    for (int q = 0; q < 6; ++q)
        if (usb[q] != 0.0 || flb[q] != 0.0)
            euler_vjp_scatter(A, c, d, sc, oR + (q - 3) * sd, xR + (q - 3) * xd, us[q], flb[q], usb[q]);
}

// Every box of a stage in one launch (blockIdx.z = box): the boxes' adjoint
// accumulations are disjoint, and one box alone leaves too few columns.
template <int NS>
__global__ void __launch_bounds__(AT, 3) adj_flux_sweep_kernel(const AdjBox* __restrict__ boxes, int d, int seg) {
    adj_flux_sweep_body<NS>(boxes[blockIdx.z], d, seg, blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// One thread per face of direction d: viscous stress (F_{m_a} -= tau_a,
// F_E -= tau_a facevel_a, tau linear in the lagged velocity gradients,
// compute_flux_3d.H:293-367) and the LLF eigenvalue
// lam = max(aL, aR) + max(|vL|, |vR|), aR with the left cell's species
// (flux_schemes.H:21-43), reversed.
template <int NS>
__global__ void __launch_bounds__(AT) adj_face_kernel(AdjBox A, int d) {
    const RhsBox& B = A.B;
    int len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    const int64_t nf = (int64_t)len[0] * len[1] * len[2];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf) return;
    const Idx3 f = delinear(t, B.lo, len);
    const Fab& FS = B.fs[d];
    const int64_t qf = FS.off(f.i, f.j, f.k);
    const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
    if (!(flags & 1)) return;
    const DevParams& P = c_P;
    const Fab& S = B.sb;
    const Fab& G = A.lamSb;
    const Fab& GA = A.lamAux;
    const int ns = P.nspec;
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t oR = S.off(f.i, f.j, f.k), oL = oR - sd;
    const double FbE = face_bar(B, A.lamL, f, d, RHOE);
    double FbM[3];
    for (int a = 0; a < 3; ++a) FbM[a] = face_bar(B, A.lamL, f, d, RHOU + a);
    if (FbE != 0.0 || FbM[0] != 0.0 || FbM[1] != 0.0 || FbM[2] != 0.0) {
        const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
        const int64_t st1 = (t1 == 0) ? 1 : (t1 == 1) ? S.js : S.ks;
        const int64_t st2 = (t2 == 0) ? 1 : (t2 == 1) ? S.js : S.ks;
        const double ids = B.idx[d], ih1 = 0.5 * B.idx[t1], ih2 = 0.5 * B.idx[t2];
        const double mu = P.visc_hm;
        int role[3];  // sweep role (0 normal, 1 t1, 2 t2) of each Cartesian axis
        role[d] = 0;
        role[t1] = 1;
        role[t2] = 2;
        double Gc[3][3];  // Gc[a][x] = dV_a/dx_x
        for (int a = 0; a < 3; ++a) {
            const double* V = S.p + (VELX + a) * S.ns;
            double g[3];
            g[0] = (V[oR] - V[oL]) * ids;
            g[1] = (0.5 * (V[oL + st1] + V[oR + st1]) - 0.5 * (V[oL - st1] + V[oR - st1])) * ih1;
            g[2] = (0.5 * (V[oL + st2] + V[oR + st2]) - 0.5 * (V[oL - st2] + V[oR - st2])) * ih2;
            for (int x = 0; x < 3; ++x) Gc[a][x] = g[role[x]];
        }
        const double delu = (Gc[0][0] + Gc[1][1]) + Gc[2][2];
        double Gb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < 3; ++a) {
            const double* V = S.p + (VELX + a) * S.ns;
            const double tau = mu * (Gc[a][d] + Gc[d][a]) - ((a == d) ? kTwo3rd * mu * delu : 0.0);
            const double fvel = 0.5 * (V[oL] + V[oR]);
            const double tb = -FbM[a] - FbE * fvel;
            const double fvb = -FbE * tau;
            aadd(&G.p[oL + (VELX + a) * G.ns], 0.5 * fvb);
            aadd(&G.p[oR + (VELX + a) * G.ns], 0.5 * fvb);
            Gb[a][d] += mu * tb;
            Gb[d][a] += mu * tb;
            if (a == d)
                for (int b = 0; b < 3; ++b) Gb[b][b] -= kTwo3rd * mu * tb;
        }
        for (int a = 0; a < 3; ++a) {
            double gb[3];
            for (int x = 0; x < 3; ++x) gb[role[x]] = Gb[a][x];
            double* Vb = G.p + (VELX + a) * G.ns;
            aadd(&Vb[oR], gb[0] * ids);
            aadd(&Vb[oL], -gb[0] * ids);
            const double h1 = 0.5 * ih1 * gb[1], h2 = 0.5 * ih2 * gb[2];
            aadd(&Vb[oL + st1], h1);
            aadd(&Vb[oR + st1], h1);
            aadd(&Vb[oL - st1], -h1);
            aadd(&Vb[oR - st1], -h1);
            aadd(&Vb[oL + st2], h2);
            aadd(&Vb[oR + st2], h2);
            aadd(&Vb[oL - st2], -h2);
            aadd(&Vb[oR - st2], -h2);
        }
    }
    const double lamb = FS.p[qf + FS_MH * FS.ns];
    if (lamb == 0.0) return;
    const Fab& X = B.aux;
    const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
    const int64_t xR = X.off(f.i, f.j, f.k), xL = xR - xd;
    const double vdL = X.p[xL + (AUX_VX + d) * X.ns], vdR = X.p[xR + (AUX_VX + d) * X.ns];
    const double aL = X.p[xL + AUX_AOWN * X.ns];
    double specL[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) specL[s] = (s < ns) ? S.p[oL + (NFLO + s) * S.ns] : 0.0;
    const double rhoR = S.p[oR + RHO * S.ns];
    const double reigR = X.p[xR + AUX_REIG * X.ns];
    const double gamR = X.p[xR + AUX_GAM * X.ns];
    const double pRp = thermo_p<NS>(reigR, rhoR, specL);
    const double qR = (gamR * pRp) / rhoR;
    const double aR = sqrt(qR);
    if (aL >= aR) {
        aadd(&GA.p[xL + AUX_AOWN * GA.ns], lamb);
    } else {
        const double qb = lamb / (2.0 * aR);
        aadd(&GA.p[xR + AUX_GAM * GA.ns], qb * pRp / rhoR);
        const double pb = qb * gamR / rhoR;
        aadd(&G.p[oR + RHO * G.ns], -qb * qR / rhoR);
        double dpr, dpc[NS];
        dpres<NS>(reigR, specL, dpr, dpc);
        aadd(&GA.p[xR + AUX_REIG * GA.ns], pb * dpr);
        for (int s = 0; s < ns; ++s) aadd(&G.p[oL + (NFLO + s) * G.ns], pb * dpc[s]);
    }
    if (fabs(vdL) >= fabs(vdR))
        aadd(&GA.p[xL + (AUX_VX + d) * GA.ns], lamb * (vdL >= 0.0 ? 1.0 : -1.0));
    else
        aadd(&GA.p[xR + (AUX_VX + d) * GA.ns], lamb * (vdR >= 0.0 ? 1.0 : -1.0));
}

// Per-cell scalars (prim_body) reversed: adjoints of (v, p, rho e_eig, a, gamma)
// pushed into the conserved state of the cell.
template <int NS>
__global__ void __launch_bounds__(AT) adj_aux_kernel(AdjBox A) {
    const RhsBox& B = A.B;
    int lo[3], len[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = B.lo[d] - MFG_NGROW;
        len[d] = B.hi[d] - B.lo[d] + 1 + 2 * MFG_NGROW;
    }
    const int64_t n = (int64_t)len[0] * len[1] * len[2];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const Idx3 c = delinear(t, lo, len);
    const Fab& S = B.sb;
    const Fab& GA = A.lamAux;
    const Fab& G = A.lamSb;
    const int64_t o = S.off(c.i, c.j, c.k);
    const int64_t q = GA.off(c.i, c.j, c.k);
    double ab[NAUX];
    bool any = false;
    for (int k = 0; k < NAUX; ++k) {
        ab[k] = GA.p[q + k * GA.ns];
        any |= ab[k] != 0.0;
    }
    if (!any) return;
    const int ns = c_P.nspec;
    const double rho = S.p[o + RHO * S.ns];
    const double m[3] = {S.p[o + RHOU * S.ns], S.p[o + RHOV * S.ns], S.p[o + RHOW * S.ns]};
    const double E = S.p[o + RHOE * S.ns];
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? S.p[o + (NFLO + s) * S.ns] : 0.0;
    const double irho = 1.0 / rho;
    const double v[3] = {m[0] * irho, m[1] * irho, m[2] * irho};
    const double k2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
    const double rhoe = E - (0.5 * rho) * k2;
    const double mm = (m[0] * m[0] + m[1] * m[1]) + m[2] * m[2];
    const double reig = E - (0.5 * mm) * irho;
    const double peig = thermo_p<NS>(reig, rho, spec);
    const double gam = thermo_gamma<NS>(rho, spec);
    const double qa = (gam * peig) * irho;
    const double aown = sqrt(qa);
    double rb = 0.0, mb[3] = {0, 0, 0}, Eb = 0.0, sb[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) sb[s] = 0.0;
    double vb[3] = {ab[AUX_VX], ab[AUX_VY], ab[AUX_VZ]};
    double gb = ab[AUX_GAM], reb = ab[AUX_REIG];
    if (ab[AUX_AOWN] != 0.0) {  // a = sqrt(gamma p_eig / rho)
        const double qb = ab[AUX_AOWN] * (0.5 / aown);
        gb += qb * peig * irho;
        const double pb = qb * gam * irho;
        rb -= qb * qa * irho;
        double dpr, dpc[NS];
        dpres<NS>(reig, spec, dpr, dpc);
        reb += pb * dpr;
#pragma unroll
        for (int s = 0; s < NS; ++s) sb[s] += pb * dpc[s];
    }
    if (gb != 0.0) {
        double dg[NS];
        dgamma<NS>(spec, dg);
#pragma unroll
        for (int s = 0; s < NS; ++s) sb[s] += gb * dg[s];
    }
    // rho e_eig = E - (m.m)/(2 rho)
    Eb += reb;
    for (int a = 0; a < 3; ++a) mb[a] -= reb * v[a];
    rb += reb * (0.5 * mm) * (irho * irho);
    // p = p(E - rho |v|^2 / 2, c)
    if (ab[AUX_PF] != 0.0) {
        double dpr, dpc[NS];
        dpres<NS>(rhoe, spec, dpr, dpc);
        const double rhoeb = ab[AUX_PF] * dpr;
#pragma unroll
        for (int s = 0; s < NS; ++s) sb[s] += ab[AUX_PF] * dpc[s];
        Eb += rhoeb;
        rb -= 0.5 * k2 * rhoeb;
        for (int a = 0; a < 3; ++a) vb[a] -= rho * v[a] * rhoeb;
    }
    // v = m / rho
    for (int a = 0; a < 3; ++a) {
        mb[a] += vb[a] * irho;
        rb -= vb[a] * v[a] * irho;
    }
    aadd(&G.p[o + RHO * G.ns], rb);
    for (int a = 0; a < 3; ++a) aadd(&G.p[o + (RHOU + a) * G.ns], mb[a]);
    aadd(&G.p[o + RHOE * G.ns], Eb);
    for (int s = 0; s < ns; ++s) aadd(&G.p[o + (NFLO + s) * G.ns], sb[s]);
}

// Cut cells reversed (update_cutcells, ib_utils.H:272-436).  c.S is the stage
// state after the cut-cell update: at a cut cell it holds the outputs, at its
// vfrac == 1 neighbours the unchanged inputs.  The adjoints of the outputs are
// consumed and distributed to the neighbours with the forward weights.
// Lists the cut cells (0 < vfrac < 1) of a box; the volume fraction never
// changes, so one list serves every stage of every step.
__global__ void adj_cut_list_kernel(CutBox c, int* __restrict__ list, unsigned* __restrict__ count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool cut = false;
    if (t < c.n) {
        int i, j, k;
        cell_of(c, t, i, j, k);
        const double vf = c.S(i, j, k, VFRAC);
        cut = vf > 0.0 && vf < 1.0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, cut);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    unsigned base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (cut) list[base + __popc(m & ((1u << lane) - 1u))] = (int)t;
}

template <int NS>
__global__ void __launch_bounds__(AT, 4) adj_cut_kernel(CutBox c, Fab G, const int* __restrict__ list, int count) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    const int64_t t = list[w];
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const double vf = S.p[o + VFRAC * S.ns];
    if (!(vf > 0.0 && vf < 1.0)) return;
    const DevParams& P = c_P;
    const int ns = P.nspec;
    const double* V = S.p + VFRAC * S.ns;
    const double hx = 0.5 / c.dx[0], hy = 0.5 / c.dx[1], hz = 0.5 / c.dx[2];
    const double gx = add(mul(V[o - 1], -hx), mul(V[o + 1], hx));
    const double gy = add(mul(V[o - S.js], -hy), mul(V[o + S.js], hy));
    const double gz = add(mul(V[o - S.ks], -hz), mul(V[o + S.ks], hz));
    const double mag = sqrt((gx * gx + gy * gy) + gz * gz);
    double dist = 0.0, xp[3] = {0.0, 0.0, 0.0};
    if (mag > kTiny) {
        dist = (vf - 0.5) / mag;
        xp[0] = -dist * (gx / mag);
        xp[1] = -dist * (gy / mag);
        xp[2] = -dist * (gz / mag);
    }
    const double dxnd[3] = {c.dx[0] / c.dxmin, c.dx[1] / c.dxmin, c.dx[2] / c.dxmin};
    const double xpn[3] = {xp[0] / c.dxmin, xp[1] / c.dxmin, xp[2] / c.dxmin};
    double swd = 0.0, swn = 0.0;
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const int64_t q = o + l + m * S.js + n * S.ks;
                if (!is_one(V[q])) continue;
                if (!(l == 0 && m == 0 && n == 0)) swd += c_wdir[(l + SG) + SW * ((m + SG) + SW * (n + SG))];
                const double a = l * dxnd[0] - xpn[0], b = m * dxnd[1] - xpn[1], e = n * dxnd[2] - xpn[2];
                swn += rcp_pos(((a * a + b * b) + e * e) + kTiny2);
            }
    const bool velzero = fabs(dist) < c.dxmin * 1e-5;
    double den = 0.0;
    if (!velzero) {
        const double dn = fabs(dist) / c.dxmin;
        den = swd + 1.0 / (dn * dn);
    }
    const bool have = swn > 0.0;
    const double dens = S.p[o + DENS * S.ns], pres = S.p[o + PRES * S.ns];
    const double vel[3] = {S.p[o + VELX * S.ns], S.p[o + VELY * S.ns], S.p[o + VELZ * S.ns]};
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? S.p[o + (NFLO + s) * S.ns] : 0.0;
    double de_dr, de_dp, de_dc[NS];
    const double e = de_int<NS>(dens, pres, spec, de_dr, de_dp, de_dc);
    const double ke = (vel[0] * vel[0] + vel[1] * vel[1]) + vel[2] * vel[2];
    // prim_to_cons reversed: rho = dens, m = dens v, E = dens e + dens |v|^2 / 2
    const double lR = G.p[o + RHO * G.ns], lE = G.p[o + RHOE * G.ns];
    const double lM[3] = {G.p[o + RHOU * G.ns], G.p[o + RHOV * G.ns], G.p[o + RHOW * G.ns]};
    double densb = G.p[o + DENS * G.ns] + lR + lE * ((e + dens * de_dr) + 0.5 * ke);
    const double presb = G.p[o + PRES * G.ns] + lE * dens * de_dp;
    const double tempb = G.p[o + TEMP * G.ns];
    double velb[3];
    for (int a = 0; a < 3; ++a) {
        densb += lM[a] * vel[a];
        velb[a] = G.p[o + (VELX + a) * G.ns] + lM[a] * dens + lE * dens * vel[a];
    }
    double specb[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) specb[s] = (s < ns) ? G.p[o + (NFLO + s) * G.ns] + lE * dens * de_dc[s] : 0.0;
    const bool interp_spec = !P.species_in_solid;
    G.p[o + RHO * G.ns] = 0.0;
    G.p[o + RHOE * G.ns] = 0.0;
    for (int a = 0; a < 3; ++a) {
        G.p[o + (RHOU + a) * G.ns] = 0.0;
        G.p[o + (VELX + a) * G.ns] = 0.0;
    }
    // without fluid neighbours the cell keeps its own pressure, temperature, density, species
    G.p[o + DENS * G.ns] = have ? 0.0 : densb;
    G.p[o + PRES * G.ns] = have ? 0.0 : presb;
    G.p[o + TEMP * G.ns] = have ? 0.0 : tempb;
    for (int s = 0; s < ns; ++s) G.p[o + (NFLO + s) * G.ns] = (interp_spec && have) ? 0.0 : specb[s];
    const double iswn = have ? 1.0 / swn : 0.0, iden = velzero ? 0.0 : 1.0 / den;
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const int64_t q = o + l + m * S.js + n * S.ks;
                if (!is_one(V[q])) continue;
                if (!velzero && !(l == 0 && m == 0 && n == 0)) {
                    const double wd = c_wdir[(l + SG) + SW * ((m + SG) + SW * (n + SG))] * iden;
                    for (int a = 0; a < 3; ++a) aadd(&G.p[q + (VELX + a) * G.ns], velb[a] * wd);
                }
                if (have) {
                    const double a = l * dxnd[0] - xpn[0], b = m * dxnd[1] - xpn[1], ee = n * dxnd[2] - xpn[2];
                    const double wn = rcp_pos(((a * a + b * b) + ee * ee) + kTiny2) * iswn;
                    aadd(&G.p[q + PRES * G.ns], presb * wn);
                    aadd(&G.p[q + TEMP * G.ns], tempb * wn);
                    aadd(&G.p[q + DENS * G.ns], densb * wn);
                    if (interp_spec)
                        for (int s = 0; s < ns; ++s) aadd(&G.p[q + (NFLO + s) * G.ns], specb[s] * wn);
                }
            }
}

// Stage algebra reversed (mflo_evolve.cpp:276-311); lamS holds the adjoint of
// the stage output on entry and of the previous stage output's direct use on exit:
//   stage 1: S1 = Sb + dt L;  stage 2: S2 = (S1 + dt L + 3 S_old)/4;
//   stage 3: S3 = (S_old + 2 (S2 + dt L))/3.
// L is the masked dsdt (div_3d.H:13-76), so masked components get no adjoint.
__global__ void adj_stage_kernel(Valid v, Fab lamS, Fab lamOld, Fab lamL, Fab lamSb, Fab sb, int stage, double dt,
                                 int ncomp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (t >= v.n || n >= ncomp) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const double a = lamS(i, j, k, n);
    double cl, co, cs;
    if (stage == 3) {
        cl = kThird * 2.0 * dt;
        co = kThird;
        cs = kThird * 2.0;
    } else if (stage == 2) {
        cl = 0.25 * dt;
        co = 0.75;
        cs = 0.25;
    } else {
        cl = dt;
        co = 0.0;
        cs = 0.0;
        lamSb(i, j, k, n) += a;
    }
    const DevParams& P = c_P;
    const double vf = sb(i, j, k, VFRAC);
    const int nnull = (P.species_in_solid == 1) ? NFLO : NFLO + P.nspec;
    const bool masked = (n != RHOE) ? (n < nnull && vf < 1.0) : (vf < 1.0);
    lamL(i, j, k, n) = masked ? 0.0 : cl * a;
    if (co != 0.0) lamOld(i, j, k, n) += co * a;
    lamS(i, j, k, n) = cs * a;
}

// Physical-boundary ghost fill reversed, one stage (3 corners, 2 edges, 1 faces)
// per launch; the ghost cell's adjoint goes to the cell it was taken from.
// A velocity inlet's ghost state depends on the inlet velocity only:
// d(ghost)/d(vel_normal) = (VEL: 1, MOM: dens, RHOE: dens vel) accumulates in gin.
__global__ void adj_bc_kernel(Fab G, int lo0, int lo1, int lo2, int hi0, int hi1, int hi2, mfg_geom g, int stage,
                              int nc, double* gin) {
    const int l0 = hi0 - lo0 + 7, l1 = hi1 - lo1 + 7, l2 = hi2 - lo2 + 7;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)l0 * l1 * l2) return;
    const int64_t a = t / l0;
    const int iv[3] = {lo0 - 3 + (int)(t - a * l0), lo1 - 3 + (int)(a % l1), lo2 - 3 + (int)(a / l1)};
    bool out[3];
    int nout = 0;
    for (int d = 0; d < 3; ++d) {
        out[d] = !g.is_periodic[d] && (iv[d] < g.domain_lo[d] || iv[d] > g.domain_hi[d]);
        nout += out[d];
    }
    if (nout != stage) return;
    const DevParams& P = c_P;
    int dext = -1, dlast = -1;
    for (int d = 0; d < 3; ++d) {
        if (!out[d]) continue;
        dlast = d;
        const int kind = (iv[d] < g.domain_lo[d]) ? P.bc_lo[d] : P.bc_hi[d];
        if (kind == MFG_BC_EXT_DIR) dext = d;
    }
    const int ds = (dext >= 0) ? dext : dlast;
    const bool lo = iv[ds] < g.domain_lo[ds];
    const int kind = lo ? P.bc_lo[ds] : P.bc_hi[ds];
    int sv[3] = {iv[0], iv[1], iv[2]};
    const int64_t qd = G.off(iv[0], iv[1], iv[2]);
    if (dext >= 0) {
        const mfg_extbc& E = lo ? P.ext_lo[ds] : P.ext_hi[ds];
        if (E.kind == MFG_EXT_VELOCITY_INLET) {
            const double s = (G.p[qd + (VELX + ds) * G.ns] + G.p[qd + (RHOU + ds) * G.ns] * E.dens) +
                             G.p[qd + RHOE * G.ns] * (E.dens * E.vel[ds]);
            aadd(gin, s);
        } else if (E.kind == MFG_EXT_FIXED_STATE && E.keep_interior_pres) {
            sv[ds] = lo ? g.domain_lo[ds] : g.domain_hi[ds];
            aadd(&G.p[G.off(sv[0], sv[1], sv[2]) + PRES * G.ns], G.p[qd + PRES * G.ns]);
        }
        return;
    }
    if (kind == MFG_BC_FOEXTRAP) {
        sv[ds] = lo ? g.domain_lo[ds] : g.domain_hi[ds];
        const int64_t qs = G.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < nc; ++c) aadd(&G.p[qs + c * G.ns], G.p[qd + c * G.ns]);
    } else {
        sv[ds] = lo ? (2 * g.domain_lo[ds] - iv[ds] - 1) : (2 * g.domain_hi[ds] - iv[ds] + 1);
        const int64_t qs = G.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < nc; ++c) {
            const double x = G.p[qd + c * G.ns];
            aadd(&G.p[qs + c * G.ns], odd_at_wall(c) ? -x : x);
        }
    }
}

// Ghost-fill copies reversed: each in-domain cell of a box's grown region
// (its own valid cells, other boxes' cells, periodic images) returns its
// adjoint to the valid cell of the owning box it was copied from.
struct CopyTab {
    int lo[3], hi[3];
    Fab G;    // adjoint of this box's stage state (grown)
    Fab dst;  // adjoint of this box's fill source (valid)
};

__global__ void adj_copy_kernel(const CopyTab* __restrict__ tab, int b, mfg_geom g, const int* __restrict__ owner,
                                int gran, int m0, int m1, int m2, int nc) {
    const CopyTab& T = tab[b];
    const int l0 = T.hi[0] - T.lo[0] + 7, l1 = T.hi[1] - T.lo[1] + 7, l2 = T.hi[2] - T.lo[2] + 7;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)l0 * l1 * l2) return;
    const int64_t a = t / l0;
    const int iv[3] = {T.lo[0] - 3 + (int)(t - a * l0), T.lo[1] - 3 + (int)(a % l1), T.lo[2] - 3 + (int)(a / l1)};
    int w[3] = {iv[0], iv[1], iv[2]};
    for (int d = 0; d < 3; ++d) {
        const int len = g.domain_hi[d] - g.domain_lo[d] + 1;
        if (g.is_periodic[d]) {
            while (w[d] < g.domain_lo[d]) w[d] += len;
            while (w[d] > g.domain_hi[d]) w[d] -= len;
        } else if (w[d] < g.domain_lo[d] || w[d] > g.domain_hi[d]) {
            return;
        }
    }
    const int x0 = (w[0] - g.domain_lo[0]) / gran, x1 = (w[1] - g.domain_lo[1]) / gran,
              x2 = (w[2] - g.domain_lo[2]) / gran;
    if (x0 >= m0 || x1 >= m1 || x2 >= m2) return;
    const int ob = owner[x0 + m0 * (x1 + m1 * x2)];
    if (ob < 0) return;
    const CopyTab& O = tab[ob];
    const int64_t qs = T.G.off(iv[0], iv[1], iv[2]);
    const int64_t qd = O.dst.off(w[0], w[1], w[2]);
    for (int c = 0; c < nc; ++c) aadd(&O.dst.p[qd + c * O.dst.ns], T.G.p[qs + c * T.G.ns]);
}

// Primitive refresh reversed (mflo_evolve.cpp:114-171), vfrac == 1 cells:
// DENS, VEL, PRES, TEMP are overwritten from the conserved state.
template <int NS>
__global__ void adj_prims_kernel(Valid v, Fab Sc, Fab lam) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    if (!is_one(Sc(i, j, k, VFRAC))) return;
    const int ns = c_P.nspec;
    const double rho = Sc(i, j, k, RHO);
    const double m[3] = {Sc(i, j, k, RHOU), Sc(i, j, k, RHOV), Sc(i, j, k, RHOW)};
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < ns) ? Sc(i, j, k, NFLO + s) : 0.0;
    const double vel[3] = {m[0] / rho, m[1] / rho, m[2] / rho};
    const double k2 = (vel[0] * vel[0] + vel[1] * vel[1]) + vel[2] * vel[2];
    const double rhoe = Sc(i, j, k, RHOE) - (0.5 * rho) * k2;
    const double p = thermo_p<NS>(rhoe, rho, spec);
    double dTp, dTr, dTc[NS];
    dtemp<NS>(rho, p, spec, dTp, dTr, dTc);
    const double Tb = lam(i, j, k, TEMP);
    const double pb = lam(i, j, k, PRES) + Tb * dTp;
    double rb = lam(i, j, k, DENS) + Tb * dTr;
    double sb[NS];
    double dpr, dpc[NS];
    dpres<NS>(rhoe, spec, dpr, dpc);
#pragma unroll
    for (int s = 0; s < NS; ++s) sb[s] = Tb * dTc[s] + pb * dpc[s];
    const double rhoeb = pb * dpr;
    rb -= 0.5 * k2 * rhoeb;
    double mb[3];
    for (int a = 0; a < 3; ++a) {
        const double vb = lam(i, j, k, VELX + a) - rho * vel[a] * rhoeb;
        mb[a] = vb / rho;
        rb -= vb * m[a] / (rho * rho);
    }
    lam(i, j, k, RHO) += rb;
    for (int a = 0; a < 3; ++a) lam(i, j, k, RHOU + a) += mb[a];
    lam(i, j, k, RHOE) += rhoeb;
    for (int s = 0; s < ns; ++s) lam(i, j, k, NFLO + s) += sb[s];
    lam(i, j, k, DENS) = 0.0;
    lam(i, j, k, VELX) = 0.0;
    lam(i, j, k, VELY) = 0.0;
    lam(i, j, k, VELZ) = 0.0;
    lam(i, j, k, PRES) = 0.0;
    lam(i, j, k, TEMP) = 0.0;
}

// Species clipping reversed: a clipped species has no dependence on its input.
__global__ void adj_clip_kernel(Valid v, Fab Sp, Fab lam, int nspec) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    for (int s = 0; s < nspec; ++s)
        if (Sp(i, j, k, NFLO + s) < 0.0) lam(i, j, k, NFLO + s) = 0.0;
}

// c^o for the orders of the reaction tables (integer 1 and 2 exact, as spec_source)
__device__ __forceinline__ double cpow(double c, double o) {
    return (o == 1.0) ? c : (o == 2.0) ? c * c : pow(c, o);
}
__device__ __forceinline__ double dcpow(double c, double o) {
    return (o == 1.0) ? 1.0 : (o == 2.0) ? 2.0 * c : o * pow(c, o - 1.0);
}

// Rate constants at T (spec_source's k_r = A_r, or A_r exp(-Ea_r/(RU T))) and
// d log k_r / dT = Ea_r/(RU T^2); T is fixed through a chemistry sub-step.
template <int NS>
__device__ void rate_constants(double T, double* kr, double* eT) {
    const DevParams& P = c_P;
    for (int r = 0; r < P.nreact; ++r) {
        kr[r] = P.A[r];
        eT[r] = 0.0;
        if (P.Ea[r] != 0.0) {
            kr[r] = P.A[r] * exp(-P.Ea[r] / (kRU * T));
            eT[r] = P.Ea[r] / (kRU * T * T);
        }
    }
}

// Rate of reaction r (k_r prod c^o) with d rate/dc_j.
template <int NS>
__device__ double rate_k(int r, double kr, const double* c, double* dc) {
    const DevParams& P = c_P;
    double cm = 1.0;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if ((P.ord_mask[r] >> s) & 1u) cm *= cpow(c[s], P.order[r][s]);
    }
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        dc[j] = 0.0;
        if (!((P.ord_mask[r] >> j) & 1u)) continue;
        double pr = kr;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            if (!((P.ord_mask[r] >> s) & 1u)) continue;
            const double o = P.order[r][s];
            pr *= (s == j) ? dcpow(c[s], o) : cpow(c[s], o);
        }
        dc[j] = pr;
    }
    return kr * cm;
}

// wdot with given rate constants (spec_source without the exponentials).
template <int NS>
__device__ void wdot_k(const double* c, const double* kr, double* w) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) w[s] = 0.0;
    for (int r = 0; r < P.nreact; ++r) {
        double cm = 1.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            if ((P.ord_mask[r] >> s) & 1u) cm *= cpow(c[s], P.order[r][s]);
        }
        const double rate = kr[r] * cm;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if ((P.nu_mask[r] >> s) & 1u) w[s] += P.nu[r][s] * rate;
    }
}

// wdot = sum_r nu_r rate_r reversed for the adjoint fb of wdot: species into
// cb, temperature into Tb, d/dlog A_r (= rate_r times the seed) into thb.
template <int NS>
__device__ void wdot_vjp(const double* c, const double* kr, const double* eT, const double* fb, double* cb,
                         double& Tb, double* thb) {
    const DevParams& P = c_P;
    for (int r = 0; r < P.nreact; ++r) {
        double rb = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if ((P.nu_mask[r] >> s) & 1u) rb += P.nu[r][s] * fb[s];
        if (rb == 0.0) continue;
        double dc[NS];
        const double rate = rate_k<NS>(r, kr[r], c, dc);
        thb[r] += rb * rate;
        Tb += (rb * rate) * eT[r];
#pragma unroll
        for (int j = 0; j < NS; ++j) cb[j] += rb * dc[j];
    }
}

__device__ __forceinline__ void warp_add(double x, double* dst) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x != 0.0) atomicAdd(dst, x);
}

// Chemistry sub-step reversed per cell (chem_substep_body: s1 = s0 + dt f0,
// s2 = s0 + dt/4 (f0 + f1), out = s0 + dt (f0/6 + f1/6 + 2 f2/3), T fixed);
// S3 is the sub-step's input.  Non-species components pass through.
template <int NS>
__global__ void adj_chem_kernel(Valid v, Fab S3, Fab lam, double dt, double* gth) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const DevParams& P = c_P;
    double thb[MAXR];
    for (int r = 0; r < MAXR; ++r) thb[r] = 0.0;
    if (t < v.n && P.chem_on) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        const int ns = P.nspec;
        double s0[NS], s1[NS], s2[NS], f0[NS], f1[NS], snb[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            s0[s] = (s < ns) ? S3(i, j, k, NFLO + s) : 0.0;
            snb[s] = (s < ns) ? lam(i, j, k, NFLO + s) : 0.0;
        }
        const double T = S3(i, j, k, TEMP);
        double kr[MAXR], eT[MAXR];
        rate_constants<NS>(T, kr, eT);
        const double c10 = dt * 1.0, c20 = dt * 0.25, c21 = dt * 0.25;
        const double w0 = dt * (1.0 / 6.0), w1 = dt * (1.0 / 6.0), w2 = dt * (2.0 / 3.0);
        wdot_k<NS>(s0, kr, f0);
#pragma unroll
        for (int s = 0; s < NS; ++s) s1[s] = s0[s] + c10 * f0[s];
        wdot_k<NS>(s1, kr, f1);
#pragma unroll
        for (int s = 0; s < NS; ++s) s2[s] = (s0[s] + c20 * f0[s]) + c21 * f1[s];
        double Tb = 0.0;
        double f0b[NS], f1b[NS], f2b[NS], s0b[NS], s1b[NS], s2b[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            f0b[s] = w0 * snb[s];
            f1b[s] = w1 * snb[s];
            f2b[s] = w2 * snb[s];
            s0b[s] = snb[s];
            s1b[s] = 0.0;
            s2b[s] = 0.0;
        }
        wdot_vjp<NS>(s2, kr, eT, f2b, s2b, Tb, thb);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            s0b[s] += s2b[s];
            f0b[s] += c20 * s2b[s];
            f1b[s] += c21 * s2b[s];
        }
        wdot_vjp<NS>(s1, kr, eT, f1b, s1b, Tb, thb);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            s0b[s] += s1b[s];
            f0b[s] += c10 * s1b[s];
        }
        wdot_vjp<NS>(s0, kr, eT, f0b, s0b, Tb, thb);
        for (int s = 0; s < ns; ++s) lam(i, j, k, NFLO + s) = s0b[s];
        lam(i, j, k, TEMP) += Tb;
    }
    for (int r = 0; r < P.nreact && r < MAXR; ++r) warp_add(thb[r], &gth[r]);
}

// Objective on the valid cells of one box, and (lam.p != null) its seed
// dJ/d(species, T) with the direct dJ/dlog A_r.
template <int NS>
__global__ void objective_kernel(Valid v, Fab S, Fab lam, double vol, double* Jacc, double* gth) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const DevParams& P = c_P;
    double jloc = 0.0, th[MAXR];
    for (int r = 0; r < MAXR; ++r) th[r] = 0.0;
    if (t < v.n) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        const int ns = P.nspec;
        double c[NS], cb[NS], dc[NS], Tb = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            c[s] = (s < ns) ? S(i, j, k, NFLO + s) : 0.0;
            cb[s] = 0.0;
        }
        const double T = S(i, j, k, TEMP);
        double kr[MAXR], eT[MAXR];
        rate_constants<NS>(T, kr, eT);
        for (int r = 0; r < P.nreact; ++r) {
            const double rate = rate_k<NS>(r, kr[r], c, dc);
            jloc += rate;
            th[r] = vol * rate;
            Tb += vol * (rate * eT[r]);
#pragma unroll
            for (int s = 0; s < NS; ++s) cb[s] += vol * dc[s];
        }
        if (lam.p) {
            for (int s = 0; s < ns; ++s) lam(i, j, k, NFLO + s) = cb[s];
            lam(i, j, k, TEMP) = Tb;
        }
    }
    warp_add(jloc * vol, Jacc);
    if (gth)
        for (int r = 0; r < P.nreact && r < MAXR; ++r) warp_add(th[r], &gth[r]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
inline unsigned nblk(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

int ns_bucket(int ns) { return ns <= 1 ? 1 : ns <= 2 ? 2 : ns <= 4 ? 4 : ns <= 8 ? 8 : 16; }

#define ADJ_UNPACK(...) __VA_ARGS__
#define ADJ_NS(KER, CFG, ARGS)                            \
    switch (ns_bucket(c_host_params().nspec)) {          \
        case 1: KER<1><<<ADJ_UNPACK CFG>>> ARGS; break;   \
        case 2: KER<2><<<ADJ_UNPACK CFG>>> ARGS; break;   \
        case 4: KER<4><<<ADJ_UNPACK CFG>>> ARGS; break;   \
        case 8: KER<8><<<ADJ_UNPACK CFG>>> ARGS; break;   \
        default: KER<16><<<ADJ_UNPACK CFG>>> ARGS; break; \
    }

// Returns MFG_ERR_CUDA from the enclosing function when a CUDA call fails,
// recording which step failed for mfg_last_error.
#define ADJ_TRY(call, where)                   \
    do {                                       \
        const cudaError_t e_ = (call);         \
        if (e_ != cudaSuccess) {               \
            note_cuda_error(e_, where);        \
            return MFG_ERR_CUDA;               \
        }                                      \
    } while (0)

int igcd(int a, int b) {
    a = a < 0 ? -a : a;
    b = b < 0 ? -b : b;
    while (b) {
        const int t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Device buffers of one adjoint run: level-wide arrays holding every box's
// valid (or grown) cells back to back, dense, component-major per box.
struct Work {
    std::vector<mfg_box> boxes;
    mfg_geom g;
    int nbox = 0, N = 0;
    std::vector<size_t> vcell, gcell;  // per-box offsets in cells
    size_t vtot = 0, gtot = 0;         // cells
    std::vector<size_t> fsoff;         // per box and direction: offset of its face scalars (doubles)
    size_t fstot = 0;
    std::vector<double*> owned;
    int* d_owner = nullptr;
    int gran = 1, mlen[3] = {1, 1, 1};
    CopyTab* d_tab = nullptr;  // [nbox] -> lam, [nbox] -> lamOld
    AdjBox* d_adj = nullptr;   // the stage's AdjBox views of every box (batched adjoint flux)
    double* d_scratch = nullptr;
    int* d_list = nullptr;
    unsigned* d_count = nullptr;
    double* d_g = nullptr;  // [J, d/du_in, d/dlog A_r ...]
    int* d_cutlist = nullptr;        // per box (at vcell[b]): its cut cells
    unsigned* d_cutcount = nullptr;  // per box
    std::vector<int> ncut;

    ~Work() {
        for (double* p : owned) cudaFree(p);
        cudaFree(d_owner);
        cudaFree(d_tab);
        cudaFree(d_scratch);
        cudaFree(d_list);
        cudaFree(d_count);
        cudaFree(d_g);
        cudaFree(d_adj);
        cudaFree(d_cutlist);
        cudaFree(d_cutcount);
    }
    double* alloc(size_t doubles) {
        double* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(doubles, 1) * sizeof(double));
        if (e != cudaSuccess) {
            note_cuda_error(e, "allocation");
            return nullptr;
        }
        owned.push_back(p);
        return p;
    }
    double* valid_buf() { return alloc(vtot * N); }
    double* grown_buf(int nc) { return alloc(gtot * nc); }
    Fab vfab(double* base, int b, int nc) const {
        const mfg_box& x = boxes[b];
        const int len[3] = {x.hi[0] - x.lo[0] + 1, x.hi[1] - x.lo[1] + 1, x.hi[2] - x.lo[2] + 1};
        return dense_fab(base + vcell[b] * nc, x.lo, len);
    }
    Fab vfab(double* base, int b) const { return vfab(base, b, N); }
    Fab gfab(double* base, int b, int nc) const {
        const mfg_box& x = boxes[b];
        const int lo[3] = {x.lo[0] - 3, x.lo[1] - 3, x.lo[2] - 3};
        const int len[3] = {x.hi[0] - x.lo[0] + 7, x.hi[1] - x.lo[1] + 7, x.hi[2] - x.lo[2] + 7};
        return dense_fab(base + gcell[b] * nc, lo, len);
    }
    mfg_array4 ga4(double* base, int b) const {
        const Fab f = gfab(base, b, N);
        mfg_array4 a;
        memset(&a, 0, sizeof(a));
        a.p = f.p;
        a.jstride = f.js;
        a.kstride = f.ks;
        a.nstride = f.ns;
        for (int d = 0; d < 3; ++d) {
            a.begin[d] = boxes[b].lo[d] - 3;
            a.end[d] = boxes[b].hi[d] + 4;
        }
        a.ncomp = N;
        return a;
    }
    int64_t grown_cells(int b) const {
        int64_t n = 1;
        for (int d = 0; d < 3; ++d) n *= boxes[b].hi[d] - boxes[b].lo[d] + 7;
        return n;
    }
};

__global__ void copy_box_kernel(Fab dst, Fab src, Valid v, int nc) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (t >= v.n || n >= nc) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    dst(i, j, k, n) = src(i, j, k, n);
}

cudaError_t copy_region(const Fab& dst, const Fab& src, const int lo[3], const int hi[3], int nc, cudaStream_t st) {
    Valid v;
    v.n = 1;
    for (int d = 0; d < 3; ++d) {
        v.lo[d] = lo[d];
        v.len[d] = hi[d] - lo[d] + 1;
        v.n *= v.len[d];
    }
    dim3 g(nblk(v.n, 256), nc);
    ProfScope ps(K_SNAPSHOT, st);
    copy_box_kernel<<<g, 256, 0, st>>>(dst, src, v, nc);
    return cudaGetLastError();
}

// Form of the adjoint flux kernel (mfg_set_adjoint_flux_form): column sweep
// (default) or the per-face form of the same mathematics.
int g_adj_flux_form = 1;
bool adj_flux_sweep() { return g_adj_flux_form == 1; }

constexpr int kAdjSeg = 16;  // faces per column segment of the batched adjoint flux sweep

// Forward intermediates of one step.
struct Snap {
    double* sb[3];   // stage states after the cut cells (grown)
    double* aux[3];  // per-cell primitives of each stage (grown, NAUX components)
    double* fs[3];   // face scalars of each stage (NFS per face, three directions)
    double* s3;      // flow result = chemistry input (valid)
    double* sc;      // chemistry result (valid)
    double* sp;      // after the primitive refresh, before clipping (valid)
};

// Points a stage's per-cell primitives and face scalars at box b's part of the
// snapshot: the forward writes them there, the reverse sweep reads them (for
// order 5 the face pass leaves FS_MH zero; the reverse sums the eigenvalue's
// adjoint into it, so each snapshot serves one reverse stage).
void snap_views(const Work& W, RhsBox& B, const Snap& sn, int stage, int b) {
    B.aux = W.gfab(sn.aux[stage - 1], b, NAUX);
    const mfg_box& x = W.boxes[b];
    for (int d = 0; d < 3; ++d) {
        const int len[3] = {x.hi[0] - x.lo[0] + 1 + (d == 0), x.hi[1] - x.lo[1] + 1 + (d == 1),
                            x.hi[2] - x.lo[2] + 1 + (d == 2)};
        B.fs[d] = dense_fab(sn.fs[stage - 1] + W.fsoff[3 * b + d], x.lo, len);
    }
}

// One step on the caller's arrays, as mfg_advance_level (chemistry and
// clipping on, no norms); with snap the intermediates are saved.
int fwd_step(Work& W, double dt, const Snap* snap, cudaStream_t st) {
    const int N = W.N;
    Fab none;
    memset(&none, 0, sizeof(none));
    for (int b = 0; b < W.nbox; ++b)
        ADJ_TRY(launch_axpy_valid(W.boxes[b], make_fab(W.boxes[b].s_old), none, 0.0, true,
                                  make_fab(W.boxes[b].s_new), N, st),
                "forward: phi_old copy");
    for (int stage = 1; stage <= 3; ++stage) {
        ADJ_TRY(launch_fill_patch(W.boxes.data(), W.nbox, W.g, stage == 1 ? 0 : 1, 0.0, st), "forward: fill patch");
        // the level-wide pass of mfg_cutcells, else box by box (bitwise the same)
        const int lv = launch_cutcells_level(W.boxes.data(), W.nbox, W.g, st);
        if (lv < 0) return MFG_ERR_CUDA;
        if (lv == 0)
            for (int b = 0; b < W.nbox; ++b)
                ADJ_TRY(launch_cutcells_box(W.boxes[b], W.g, nullptr, W.d_list, W.d_count, st), "forward: cut cells");
        for (int b = 0; b < W.nbox; ++b) {
            const mfg_box& x = W.boxes[b];
            if (snap) {
                const int lo[3] = {x.lo[0] - 3, x.lo[1] - 3, x.lo[2] - 3};
                const int hi[3] = {x.hi[0] + 3, x.hi[1] + 3, x.hi[2] + 3};
                ADJ_TRY(copy_region(W.gfab(snap->sb[stage - 1], b, N), make_fab(x.sborder), lo, hi, N, st),
                        "forward: stage snapshot");
            }
            RhsBox B = layout_rhs_box(x, W.g, W.d_scratch);
            if (snap) snap_views(W, B, *snap, stage, b);  // keep the stage's primitives and face scalars
            ADJ_TRY(launch_rhs_box(B, stage, dt, weno_fast_mode(), st), "forward: right-hand side");
        }
    }
    if (!snap) {  // no intermediates kept: the bookends in one pass, as mfg_advance_level
        for (int b = 0; b < W.nbox; ++b)
            ADJ_TRY(launch_post_step(W.boxes[b], dt, true, true, nullptr, nullptr, st), "forward: bookends");
        return MFG_OK;
    }
    for (int b = 0; b < W.nbox; ++b) {
        const mfg_box& x = W.boxes[b];
        if (snap) ADJ_TRY(copy_region(W.vfab(snap->s3, b), make_fab(x.s_new), x.lo, x.hi, N, st), "forward: snapshot");
        ADJ_TRY(launch_axpy_valid(x, make_fab(x.s_old), none, 0.0, true, make_fab(x.s_new), N, st),
                "forward: chemistry copy");
        ADJ_TRY(launch_chem_substep(x, dt, st), "forward: chemistry");
        if (snap) ADJ_TRY(copy_region(W.vfab(snap->sc, b), make_fab(x.s_new), x.lo, x.hi, N, st), "forward: snapshot");
        ADJ_TRY(launch_update_prims(x, nullptr, st), "forward: primitives");
        if (snap) ADJ_TRY(copy_region(W.vfab(snap->sp, b), make_fab(x.s_new), x.lo, x.hi, N, st), "forward: snapshot");
        ADJ_TRY(launch_clip_species(x, st), "forward: clipping");
    }
    return MFG_OK;
}

// Reverse of one step: lam holds the adjoint of the step's output on entry and
// of its input on exit.
int adj_step(Work& W, double dt, const Snap& sn, double* lam, double* lamOld, double* lamL, double* lamSb,
             double* lamAux, cudaStream_t st) {
    const int N = W.N, ns = c_host_params().nspec;
    ADJ_TRY(cudaMemsetAsync(lamOld, 0, W.vtot * N * sizeof(double), st), "reverse: clear");
    for (int b = 0; b < W.nbox; ++b) {
        const Valid v = valid_of(W.boxes[b]);
        {
            ProfScope ps(K_ADJ_LOCAL, st);
            adj_clip_kernel<<<nblk(v.n, 256), 256, 0, st>>>(v, W.vfab(sn.sp, b), W.vfab(lam, b), ns);
        }
        {
            ProfScope ps(K_ADJ_LOCAL, st);
            ADJ_NS(adj_prims_kernel, (nblk(v.n, AT), AT, 0, st), (v, W.vfab(sn.sc, b), W.vfab(lam, b)));
        }
        {
            ProfScope ps(K_ADJ_LOCAL, st);
            ADJ_NS(adj_chem_kernel, (nblk(v.n, AT), AT, 0, st),
                   (v, W.vfab(sn.s3, b), W.vfab(lam, b), dt, W.d_g + 2));
        }
        ADJ_TRY(cudaGetLastError(), "reverse: clipping, primitives, chemistry");
    }
    const double dxmin = std::min(W.g.dx[0], std::min(W.g.dx[1], W.g.dx[2]));
    for (int stage = 3; stage >= 1; --stage) {
        double* sb = sn.sb[stage - 1];
        ADJ_TRY(cudaMemsetAsync(lamSb, 0, W.gtot * N * sizeof(double), st), "reverse: clear");
        ADJ_TRY(cudaMemsetAsync(lamAux, 0, W.gtot * NAUX * sizeof(double), st), "reverse: clear");
        for (int b = 0; b < W.nbox; ++b) {
            const Valid v = valid_of(W.boxes[b]);
            dim3 g(nblk(v.n, 256), N);
            ProfScope ps(K_ADJ_LOCAL, st);
            adj_stage_kernel<<<g, 256, 0, st>>>(v, W.vfab(lam, b), W.vfab(lamOld, b), W.vfab(lamL, b),
                                                W.gfab(lamSb, b, N), W.gfab(sb, b, N), stage, dt, N);
            ADJ_TRY(cudaGetLastError(), "reverse: stage algebra");
        }
        // forward views of the stage for every box: its state, per-cell primitives
        // and face scalars as the forward computed them
        std::vector<AdjBox> adj(W.nbox);
        for (int b = 0; b < W.nbox; ++b) {
            mfg_box x = W.boxes[b];
            x.sborder = W.ga4(sb, b);
            AdjBox& A = adj[b];
            A.B = layout_rhs_box(x, W.g, W.d_scratch);
            snap_views(W, A.B, sn, stage, b);
            A.lamL = W.vfab(lamL, b);
            A.lamSb = W.gfab(lamSb, b, N);
            A.lamAux = W.gfab(lamAux, b, NAUX);
        }
        const int C = NCONS + c_host_params().nspec;
        const bool sweep = adj_flux_sweep();
        if (sweep) {  // hyperbolic fluxes of all boxes, one column-sweep launch per direction
            ADJ_TRY(cudaMemcpyAsync(W.d_adj, adj.data(), W.nbox * sizeof(AdjBox), cudaMemcpyHostToDevice, st),
                    "reverse: box views");
            for (int d = 0; d < 3; ++d) {
                unsigned nbs = 1;
                for (int b = 0; b < W.nbox; ++b) nbs = std::max(nbs, nblk(sweep_items(adj[b].B, d, kAdjSeg), AT));
                ProfScope ps(K_ADJ_FLUX, st);
                ADJ_NS(adj_flux_sweep_kernel, (dim3(nbs, C, W.nbox), AT, 0, st), (W.d_adj, d, kAdjSeg));
                ADJ_TRY(cudaGetLastError(), "reverse: face fluxes");
            }
        }
        for (int b = 0; b < W.nbox; ++b) {
            const AdjBox& A = adj[b];
            const mfg_box& x = W.boxes[b];
            const int64_t ng = W.grown_cells(b);
            for (int d = 0; d < 3; ++d) {
                const unsigned nbf = nblk(face_items(A.B, d), AT);
                if (!sweep) {
                    ProfScope ps(K_ADJ_FLUX, st);
                    ADJ_NS(adj_flux_kernel, (dim3(nbf, C), AT, 0, st), (A, d));
                }
                {
                    ProfScope ps(K_ADJ_FACE, st);
                    ADJ_NS(adj_face_kernel, (nbf, AT, 0, st), (A, d));
                }
                ADJ_TRY(cudaGetLastError(), "reverse: face fluxes");
            }
            {
                ProfScope ps(K_ADJ_CELL, st);
                ADJ_NS(adj_aux_kernel, (nblk(ng, AT), AT, 0, st), (A));
            }
            ADJ_TRY(cudaGetLastError(), "reverse: per-cell primitives (adjoint)");
            CutBox c;
            memset(&c, 0, sizeof(c));
            c.n = 1;
            for (int d = 0; d < 3; ++d) {
                c.lo[d] = x.lo[d];
                c.len[d] = x.hi[d] - x.lo[d] + 1;
                c.n *= c.len[d];
                c.dx[d] = W.g.dx[d];
            }
            c.S = W.gfab(sb, b, N);
            c.dxmin = dxmin;
            if (W.ncut[b] > 0) {
                ProfScope ps(K_ADJ_CUT, st);
                ADJ_NS(adj_cut_kernel, (nblk(W.ncut[b], AT), AT, 0, st),
                       (c, W.gfab(lamSb, b, N), W.d_cutlist + W.vcell[b], W.ncut[b]));
            }
            ADJ_TRY(cudaGetLastError(), "reverse: cut cells");
            if (!(W.g.is_periodic[0] && W.g.is_periodic[1] && W.g.is_periodic[2]))
                for (int s = 3; s >= 1; --s) {
                    ProfScope ps(K_ADJ_FILL, st);
                    adj_bc_kernel<<<nblk(ng, 256), 256, 0, st>>>(W.gfab(lamSb, b, N), x.lo[0], x.lo[1], x.lo[2],
                                                                 x.hi[0], x.hi[1], x.hi[2], W.g, s, N, W.d_g + 1);
                }
            ADJ_TRY(cudaGetLastError(), "reverse: physical boundaries");
        }
        // the copies return the adjoint to the fill source: S_old in stage 1, else the previous stage
        const CopyTab* tab = W.d_tab + (stage == 1 ? W.nbox : 0);
        for (int b = 0; b < W.nbox; ++b) {
            ProfScope ps(K_ADJ_FILL, st);
            adj_copy_kernel<<<nblk(W.grown_cells(b), 256), 256, 0, st>>>(tab, b, W.g, W.d_owner, W.gran, W.mlen[0],
                                                                         W.mlen[1], W.mlen[2], N);
        }
        ADJ_TRY(cudaGetLastError(), "reverse: ghost copies");
    }
    ADJ_TRY(cudaMemcpyAsync(lam, lamOld, W.vtot * N * sizeof(double), cudaMemcpyDeviceToDevice, st), "reverse: copy");
    return MFG_OK;
}

int check_adjoint_scope() {
    const DevParams& P = c_host_params();
    if (P.order_hyp != 5 || !P.do_ns || P.conj_ht || P.thermo_kind == MFG_THERMO_BG_GAS ||
        P.visc_mode != MFG_TRANSPORT_CONST || P.cond_mode != MFG_TRANSPORT_CONST)
        return MFG_ERR_STATE;
    for (int d = 0; d < 3; ++d) {
        const mfg_extbc* e[2] = {&P.ext_lo[d], &P.ext_hi[d]};
        const int k[2] = {P.bc_lo[d], P.bc_hi[d]};
        for (int s = 0; s < 2; ++s)
            if (k[s] == MFG_BC_EXT_DIR && !(e[s]->kind == MFG_EXT_VELOCITY_INLET || e[s]->kind == MFG_EXT_FIXED_STATE))
                return MFG_ERR_STATE;
    }
    return MFG_OK;
}

int launch_objective(const mfg_box* boxes, int nbox, const mfg_geom& g, double* Jacc, Work* W, double* lam,
                     double* gth, cudaStream_t st) {
    const double vol = g.dx[0] * g.dx[1] * g.dx[2];
    for (int b = 0; b < nbox; ++b) {
        const Valid v = valid_of(boxes[b]);
        Fab L;
        memset(&L, 0, sizeof(L));
        if (W && lam) L = W->vfab(lam, b);
        ProfScope ps(K_ADJ_LOCAL, st);
        ADJ_NS(objective_kernel, (nblk(v.n, 256), 256, 0, st), (v, make_fab(boxes[b].s_new), L, vol, Jacc, gth));
        ADJ_TRY(cudaGetLastError(), "objective");
    }
    return MFG_OK;
}

}  // namespace
}  // namespace mfg

using namespace mfg;

extern "C" int mfg_reaction_objective(const mfg_box* boxes, int nbox, const mfg_geom* geom, double* J, void* stream) {
    int rc = validate_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    if (!geom || !J) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return MFG_ERR_CUDA;
    rc = MFG_OK;
    if (cudaMemsetAsync(d, 0, sizeof(double), st) != cudaSuccess) rc = MFG_ERR_CUDA;
    if (!rc) rc = launch_objective(boxes, nbox, *geom, d, nullptr, nullptr, nullptr, st);
    if (!rc && (cudaMemcpyAsync(J, d, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = MFG_ERR_CUDA;
    cudaFree(d);
    return rc;
}

extern "C" int mfg_set_adjoint_flux_form(int form) {
    if (form != 0 && form != 1) return MFG_ERR_ARG;
    g_adj_flux_form = form;
    return MFG_OK;
}

extern "C" int mfg_adjoint_objective(const mfg_box* boxes, int nbox, const mfg_geom* geom, int nsteps, double dt,
                                     int checkpoint_every, double* J, double* grad_logA, double* grad_uin,
                                     void* stream) {
    int rc = validate_boxes(boxes, nbox, true, false, true, true);
    if (rc) return rc;
    if (!geom || !J || nbox < 1 || nsteps < 1 || checkpoint_every < 0 || !(dt > 0.0)) return MFG_ERR_ARG;
    if ((rc = check_adjoint_scope())) return rc;
    const DevParams& P = c_host_params();
    cudaStream_t st = (cudaStream_t)stream;
    ADJ_TRY(cudaGetLastError(), "an earlier CUDA error was pending");
    Work W;
    W.boxes.assign(boxes, boxes + nbox);
    W.g = *geom;
    W.nbox = nbox;
    W.N = NFLO + P.nspec;
    W.vcell.resize(nbox);
    W.gcell.resize(nbox);
    size_t maxcells = 0, maxscr = 0;
    for (int b = 0; b < nbox; ++b) {
        int n[3];
        for (int d = 0; d < 3; ++d) n[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
        W.vcell[b] = W.vtot;
        W.gcell[b] = W.gtot;
        for (int d = 0; d < 3; ++d) {
            W.fsoff.push_back(W.fstot);
            W.fstot += face_doubles(n, d, NFS);
        }
        W.vtot += (size_t)n[0] * n[1] * n[2];
        W.gtot += (size_t)(n[0] + 6) * (n[1] + 6) * (n[2] + 6);
        maxcells = std::max(maxcells, (size_t)n[0] * n[1] * n[2]);
        maxscr = std::max(maxscr, rhs_box_scratch_doubles(n));
    }
    ADJ_TRY(cudaMalloc(&W.d_scratch, maxscr * sizeof(double)), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_list, maxcells * sizeof(int)), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_count, 256), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_g, (2 + MAXR) * sizeof(double)), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_tab, 2 * (size_t)nbox * sizeof(CopyTab)), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_adj, (size_t)std::max(nbox, 1) * sizeof(AdjBox)), "allocation");
    ADJ_TRY(cudaMemsetAsync(W.d_g, 0, (2 + MAXR) * sizeof(double), st), "clear");
    // cut-cell lists of every box (from the volume fraction of s_new)
    ADJ_TRY(cudaMalloc(&W.d_cutlist, std::max<size_t>(W.vtot, 1) * sizeof(int)), "allocation");
    ADJ_TRY(cudaMalloc(&W.d_cutcount, nbox * sizeof(unsigned)), "allocation");
    ADJ_TRY(cudaMemsetAsync(W.d_cutcount, 0, nbox * sizeof(unsigned), st), "clear");
    for (int b = 0; b < nbox; ++b) {
        CutBox c;
        memset(&c, 0, sizeof(c));
        c.n = 1;
        for (int d = 0; d < 3; ++d) {
            c.lo[d] = boxes[b].lo[d];
            c.len[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
            c.n *= c.len[d];
        }
        c.S = make_fab(boxes[b].s_new);
        adj_cut_list_kernel<<<nblk(c.n, 256), 256, 0, st>>>(c, W.d_cutlist + W.vcell[b], W.d_cutcount + b);
    }
    ADJ_TRY(cudaGetLastError(), "cut-cell lists");
    {
        std::vector<unsigned> h(nbox);
        ADJ_TRY(cudaMemcpyAsync(h.data(), W.d_cutcount, nbox * sizeof(unsigned), cudaMemcpyDeviceToHost, st),
                "cut-cell lists");
        ADJ_TRY(cudaStreamSynchronize(st), "cut-cell lists");
        W.ncut.assign(h.begin(), h.end());
    }
    // owner map of the copies (as the ghost fill's)
    {
        int gr = 0;
        for (int d = 0; d < 3; ++d) gr = igcd(gr, geom->domain_hi[d] - geom->domain_lo[d] + 1);
        for (int b = 0; b < nbox; ++b)
            for (int d = 0; d < 3; ++d) {
                gr = igcd(gr, boxes[b].lo[d] - geom->domain_lo[d]);
                gr = igcd(gr, boxes[b].hi[d] + 1 - geom->domain_lo[d]);
            }
        if (gr <= 0) gr = 1;
        W.gran = gr;
        for (int d = 0; d < 3; ++d) W.mlen[d] = (geom->domain_hi[d] - geom->domain_lo[d] + 1) / gr;
        std::vector<int> own((size_t)W.mlen[0] * W.mlen[1] * W.mlen[2], -1);
        for (int b = 0; b < nbox; ++b) {
            int a[3], z[3];
            for (int d = 0; d < 3; ++d) {
                a[d] = (boxes[b].lo[d] - geom->domain_lo[d]) / gr;
                z[d] = (boxes[b].hi[d] + 1 - geom->domain_lo[d]) / gr;
            }
            for (int q2 = a[2]; q2 < z[2]; ++q2)
                for (int q1 = a[1]; q1 < z[1]; ++q1)
                    for (int q0 = a[0]; q0 < z[0]; ++q0)
                        if (q0 >= 0 && q1 >= 0 && q2 >= 0 && q0 < W.mlen[0] && q1 < W.mlen[1] && q2 < W.mlen[2])
                            own[q0 + (size_t)W.mlen[0] * (q1 + (size_t)W.mlen[1] * q2)] = b;
        }
        ADJ_TRY(cudaMalloc(&W.d_owner, own.size() * sizeof(int)), "allocation");
        ADJ_TRY(cudaMemcpy(W.d_owner, own.data(), own.size() * sizeof(int), cudaMemcpyHostToDevice), "owner map");
    }
    // checkpoint_every == 0: every step's intermediates stay in device memory, nothing is recomputed
    const bool keep_all = checkpoint_every == 0;
    const int ce = keep_all ? 1 : std::min(checkpoint_every, nsteps);
    const int nseg = keep_all ? 0 : (nsteps + ce - 1) / ce;
    // With checkpoints, the snapshots of one whole segment are kept when they
    // fit in device memory: each segment is then recomputed once (the last one
    // not at all: its snapshots come from the first forward sweep) and reversed
    // from its snapshots.  Otherwise one snapshot is kept: the segment's states
    // are recomputed and stored, and each step is recomputed once more with its
    // snapshot before its reverse.
    const size_t snap_doubles = 3 * (W.gtot * (size_t)W.N + W.gtot * (size_t)NAUX + W.fstot) + 3 * W.vtot * (size_t)W.N;
    bool seg_keep = false;
    if (!keep_all) {
        size_t free_b = 0, total_b = 0;
        ADJ_TRY(cudaMemGetInfo(&free_b, &total_b), "memory query");
        const size_t need = (size_t)ce * snap_doubles * sizeof(double) + ((size_t)nseg + 6) * W.vtot * W.N * sizeof(double);
        seg_keep = need + (size_t)2 * 1024 * 1024 * 1024 < free_b;
    }
    std::vector<double*> ckpt(nseg), zst((keep_all || seg_keep) ? 0 : ce);
    for (auto& p : ckpt)
        if (!(p = W.valid_buf())) return MFG_ERR_CUDA;
    for (auto& p : zst)
        if (!(p = W.valid_buf())) return MFG_ERR_CUDA;
    std::vector<Snap> snaps(keep_all ? nsteps : seg_keep ? ce : 1);
    for (Snap& sn : snaps) {
        for (int s = 0; s < 3; ++s)
            if (!(sn.sb[s] = W.grown_buf(W.N)) || !(sn.aux[s] = W.grown_buf(NAUX)) ||
                !(sn.fs[s] = W.alloc(W.fstot)))
                return MFG_ERR_CUDA;
        if (!(sn.s3 = W.valid_buf()) || !(sn.sc = W.valid_buf()) || !(sn.sp = W.valid_buf())) return MFG_ERR_CUDA;
    }
    Snap& sn = snaps[0];
    double* lam = W.valid_buf();
    double* lamOld = W.valid_buf();
    double* lamL = W.valid_buf();
    double* lamSb = W.grown_buf(W.N);
    double* lamAux = W.grown_buf(NAUX);
    double* fin = keep_all ? lam : W.valid_buf();
    if (!lam || !lamOld || !lamL || !lamSb || !lamAux || !fin) return MFG_ERR_CUDA;
    {
        std::vector<CopyTab> tab(2 * (size_t)nbox);
        for (int h = 0; h < 2; ++h)
            for (int b = 0; b < nbox; ++b) {
                CopyTab& T = tab[(size_t)h * nbox + b];
                memset(&T, 0, sizeof(T));
                for (int d = 0; d < 3; ++d) {
                    T.lo[d] = boxes[b].lo[d];
                    T.hi[d] = boxes[b].hi[d];
                }
                T.G = W.gfab(lamSb, b, W.N);
                T.dst = W.vfab(h ? lamOld : lam, b);
            }
        ADJ_TRY(cudaMemcpy(W.d_tab, tab.data(), tab.size() * sizeof(CopyTab), cudaMemcpyHostToDevice), "copy table");
    }
    auto save = [&](double* dst) -> int {
        for (int b = 0; b < nbox; ++b)
            ADJ_TRY(copy_region(W.vfab(dst, b), make_fab(boxes[b].s_new), boxes[b].lo, boxes[b].hi, W.N, st),
                    "checkpoint");
        return MFG_OK;
    };
    auto restore = [&](double* src) -> int {
        for (int b = 0; b < nbox; ++b)
            ADJ_TRY(copy_region(make_fab(boxes[b].s_new), W.vfab(src, b), boxes[b].lo, boxes[b].hi, W.N, st),
                    "restore");
        return MFG_OK;
    };
    // forward sweep with checkpoints (or with every step's intermediates); with
    // whole-segment snapshots the last segment keeps them here already
    const int last0 = keep_all ? 0 : (nseg - 1) * ce;
    for (int n = 0; n < nsteps; ++n) {
        if (!keep_all && n % ce == 0 && (rc = save(ckpt[n / ce]))) return rc;
        const Snap* keep = keep_all ? &snaps[n] : (seg_keep && n >= last0) ? &snaps[n - last0] : nullptr;
        if ((rc = fwd_step(W, dt, keep, st))) return rc;
    }
    // objective and its seed on the final state
    ADJ_TRY(cudaMemsetAsync(lam, 0, W.vtot * W.N * sizeof(double), st), "clear");
    if ((rc = launch_objective(boxes, nbox, *geom, W.d_g, &W, lam, W.d_g + 2, st))) return rc;
    if (keep_all) {
        for (int n = nsteps - 1; n >= 0; --n)
            if ((rc = adj_step(W, dt, snaps[n], lam, lamOld, lamL, lamSb, lamAux, st))) return rc;
    }
    if (!keep_all && (rc = save(fin))) return rc;
    // reverse sweep, one checkpoint segment at a time
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int n0 = seg * ce, n1 = std::min(nsteps, n0 + ce);
        if (seg_keep) {
            if (seg != nseg - 1) {
                if ((rc = restore(ckpt[seg]))) return rc;
                for (int n = n0; n < n1; ++n)
                    if ((rc = fwd_step(W, dt, &snaps[n - n0], st))) return rc;
            }
            for (int n = n1 - 1; n >= n0; --n)
                if ((rc = adj_step(W, dt, snaps[n - n0], lam, lamOld, lamL, lamSb, lamAux, st))) return rc;
            continue;
        }
        if ((rc = restore(ckpt[seg]))) return rc;
        for (int n = n0; n < n1; ++n) {
            if ((rc = save(zst[n - n0]))) return rc;
            if (n + 1 < n1 && (rc = fwd_step(W, dt, nullptr, st))) return rc;
        }
        for (int n = n1 - 1; n >= n0; --n) {
            if ((rc = restore(zst[n - n0]))) return rc;
            if ((rc = fwd_step(W, dt, &sn, st))) return rc;
            if ((rc = adj_step(W, dt, sn, lam, lamOld, lamL, lamSb, lamAux, st))) return rc;
        }
    }
    if (!keep_all && (rc = restore(fin))) return rc;
    double h[2 + MAXR];
    ADJ_TRY(cudaMemcpyAsync(h, W.d_g, sizeof(h), cudaMemcpyDeviceToHost, st), "result copy");
    ADJ_TRY(cudaStreamSynchronize(st), "synchronize");
    unsigned status = 0;
    ADJ_TRY(read_status(&status, false), "status");
    if (status & MFG_STATUS_NAN) return MFG_ERR_NAN;
    *J = h[0];
    if (grad_uin) *grad_uin = h[1];
    if (grad_logA)
        for (int r = 0; r < P.nreact; ++r) grad_logA[r] = h[2 + r];
    return MFG_OK;
}
