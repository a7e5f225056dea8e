// Per-item bodies of the flow right-hand side (prim / face / flux / update),
// shared by the per-box launches (mfg_rhs.cu) and the batched persistent
// launches over all boxes of all levels (mfg_batch.cu).  See mfg_rhs.cu for
// the structure and the reference semantics.
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {
namespace {

constexpr double kEpsWeno = 1e-6;

// ---------------------------------------------------------------------------
// index helpers
// ---------------------------------------------------------------------------
struct Idx3 {
    int i, j, k;
};

__device__ __forceinline__ Idx3 delinear(int64_t t, const int lo[3], const int len[3]) {
    Idx3 r;
    split3(t, len[0], len[1], r.i, r.j, r.k);
    r.i += lo[0];
    r.j += lo[1];
    r.k += lo[2];
    return r;
}

// Euler flux of component c along d at one cell (consprim_funcs.H:48-81 with
// a unit normal e_d: the products with the zero normal components are exact
// zeros and drop out).  Rounding-faithful helpers keep the reference's
// separate multiply and add.
__device__ __forceinline__ double euler_flux(int c, int d, double u_c, double rho, double va, double vd,
                                             double p, double E) {
    if (c == RHO) return mul(rho, vd);
    if (c <= RHOW) {
        double t = mul(mul(rho, va), vd);
        return (c - 1 == d) ? add(t, p) : t;
    }
    if (c == RHOE) return mul(add(E, p), vd);
    return mul(u_c, vd);
}

// One WENO5-JS edge value (flux_schemes.H:373-446).  Inputs are the five
// stencil values ordered from the far upwind cell (a) to the far downwind
// cell (e); the right-biased edge passes them mirrored.  MIR selects the
// operand order of the reference's third candidate polynomial for the mirrored
// call.  FAST normalises the three nonlinear weights with one division
// (w_k/(eps+b_k)^2 / sum = w_k e_k / sum w_j e_j, e_k = prod_{j!=k} (eps+b_j)^2)
// instead of four; the result differs from the reference by a few ulp.
template <bool MIR, bool FAST>
__device__ __forceinline__ double weno_edge(double a, double b, double c, double d, double e) {
    double t = (a - 2.0 * b) + c;
    double t2 = (a - 4.0 * b) + 3.0 * c;
    double b2 = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
    t = (b - 2.0 * c) + d;
    double b1 = (13.0 / 12.0) * (t * t) + (0.25 * (b - d)) * (b - d);
    t = (c - 2.0 * d) + e;
    t2 = (3.0 * c - 4.0 * d) + e;
    double b0 = (13.0 / 12.0) * (t * t) + 0.25 * (t2 * t2);
    double v2 = MIR ? (11.0 * c - 7.0 * b) + 2.0 * a : (2.0 * a - 7.0 * b) + 11.0 * c;
    double v1 = (-b + 5.0 * c) + 2.0 * d;
    double v0 = (2.0 * c + 5.0 * d) - e;
    if (FAST) {
        double d2 = (kEpsWeno + b2) * (kEpsWeno + b2);
        double d1 = (kEpsWeno + b1) * (kEpsWeno + b1);
        double d0 = (kEpsWeno + b0) * (kEpsWeno + b0);
        double e2 = d1 * d0, e1 = 6.0 * (d2 * d0), e0 = 3.0 * (d2 * d1);
        double num = (e2 * v2 + e1 * v1) + e0 * v0;
        double den = (e2 + e1) + e0;
        return num / (6.0 * den);
    }
    double a2 = 1.0 / ((kEpsWeno + b2) * (kEpsWeno + b2));
    double a1 = 6.0 * (1.0 / ((kEpsWeno + b1) * (kEpsWeno + b1)));
    double a0 = 3.0 * (1.0 / ((kEpsWeno + b0) * (kEpsWeno + b0)));
    double inv = 1.0 / ((a2 + a1) + a0);
    return ((1.0 / 6.0) * inv) * ((a2 * v2 + a1 * v1) + a0 * v0);
}

// Face value pair of the stencil s[0..5] = cells i-3 .. i+2 of face i:
// up = left-biased value (cells i-3..i+1), um = right-biased (cells i-2..i+2).
template <bool FAST>
__device__ __forceinline__ void weno_face(const double s[6], double& up, double& um) {
    up = weno_edge<false, FAST>(s[0], s[1], s[2], s[3], s[4]);
    um = weno_edge<true, FAST>(s[5], s[4], s[3], s[2], s[1]);
}

// AUSM+-up split functions (flux_schemes.H:107-181), beta = 1/8.  The
// supersonic branches of the pressure splits, (M + |M|)/(2M) and
// (M - |M|)/(2M), are exactly 1 or 0 (with a zero's sign that no later
// operation keeps), and those of the Mach splits, (M + |M|)/2 and
// (M - |M|)/2, exactly M or +0 (2M and its halving are exact), so all four
// are selects; the |M| <= 1 tests run on the integer pipe.
__device__ __forceinline__ double split_mach_p(double M) {
    return abs_le(M, 1.0) ? (0.25 * (M + 1.0)) * (M + 1.0) + (0.125 * (M * M - 1.0)) * (M * M - 1.0)
                          : (is_positive(M) ? M : 0.0);
}
__device__ __forceinline__ double split_mach_m(double M) {
    return abs_le(M, 1.0) ? (-0.25 * (M - 1.0)) * (M - 1.0) - (0.125 * (M * M - 1.0)) * (M * M - 1.0)
                          : (is_negative(M) ? M : 0.0);
}
__device__ __forceinline__ double split_pres_p(double M, double alpha) {
    return abs_le(M, 1.0)
               ? ((0.25 * (M + 1.0)) * (M + 1.0)) * (2.0 - M) + ((alpha * M) * (M * M - 1.0)) * (M * M - 1.0)
               : (is_positive(M) ? 1.0 : 0.0);
}
__device__ __forceinline__ double split_pres_m(double M, double alpha) {
    return abs_le(M, 1.0)
               ? ((0.25 * (M - 1.0)) * (M - 1.0)) * (2.0 + M) - ((alpha * M) * (M * M - 1.0)) * (M * M - 1.0)
               : (is_positive(M) ? 0.0 : 1.0);
}

// MUSCL state of component c with the Tatsumi-Martinelli-Jameson limiter
// (compute_flux_3d.H:33-65): uL + L/2 and uR - L/2 with
// L = psi (d1 + d2) / 2, psi = 1 - q^2, q = |d1 - d2| / (|d1| + |d2| + 1e-20),
// d1 = u_{i+1} - u_R, d2 = u_L - u_{i-2}.  In closed form L/2 = d1 d2 / (d1 + d2)
// when d1 and d2 have the same sign (then 1 - q^2 = 4 d1 d2 / (d1 + d2)^2) and
// 0 otherwise (q = 1): the reference's expression equals this up to rounding
// and terms of the order of its 1e-20 guard, and the closed form needs one
// reciprocal and four fewer FP64 operations.  The same-sign test is on the
// integer pipe (d1 d2 > 0).
__device__ __forceinline__ void muscl(double uim2, double uL, double uR, double uip1, double& uLh, double& uRh) {
    const double delt1 = uip1 - uR;
    const double delt2 = uL - uim2;
    const double p = delt1 * delt2;
    const double s = delt1 + delt2;
    // p > 0 implies s != 0; otherwise the reciprocal's value is not used
    const double half = is_positive(p) ? p * rcp_nonzero(s) : 0.0;
    uLh = uL + half;
    uRh = uR - half;
}

// ---------------------------------------------------------------------------
// prim_kernel: per-cell scalars over grow(bx, 3)
// ---------------------------------------------------------------------------
template <int NS>
__device__ __forceinline__ void prim_body(const RhsBox& B, int64_t t) {
    int lo[3], len[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = B.lo[d] - MFG_NGROW;
        len[d] = B.hi[d] - B.lo[d] + 1 + 2 * MFG_NGROW;
    }
    const int64_t n = (int64_t)len[0] * len[1] * len[2];
    if (t >= n) return;
    const Idx3 c = delinear(t, lo, len);
    const Fab& S = B.sb;
    const int64_t o = S.off(c.i, c.j, c.k);
    const double rho = S.p[o + RHO * S.ns];
    const double m0 = S.p[o + RHOU * S.ns], m1 = S.p[o + RHOV * S.ns], m2 = S.p[o + RHOW * S.ns];
    const double E = S.p[o + RHOE * S.ns];
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < c_P.nspec) ? S.p[o + (NFLO + s) * S.ns] : 0.0;
    // cons_to_prim (consprim_funcs.H:9-23); one Newton-refined reciprocal of
    // the density replaces the reference's five divisions by it
    const double irho = rcp_pos(rho);
    const double vx = m0 * irho, vy = m1 * irho, vz = m2 * irho;
    const double rhoe = E - (0.5 * rho) * ((vx * vx + vy * vy) + vz * vz);
    const double pf = thermo_p<NS>(rhoe, rho, spec);
    // get_max_eigenvalue's own-species terms (flux_schemes.H:21-43)
    const double reig = E - (0.5 * ((m0 * m0 + m1 * m1) + m2 * m2)) * irho;
    const double peig = thermo_p<NS>(reig, rho, spec);
    const double gam = thermo_gamma<NS>(rho, spec);
    const double aown = sqrt((gam * peig) * irho);
    const Fab& X = B.aux;
    const int64_t q = X.off(c.i, c.j, c.k);
    X.p[q + AUX_VX * X.ns] = vx;
    X.p[q + AUX_VY * X.ns] = vy;
    X.p[q + AUX_VZ * X.ns] = vz;
    X.p[q + AUX_PF * X.ns] = pf;
    X.p[q + AUX_REIG * X.ns] = reig;
    X.p[q + AUX_AOWN * X.ns] = aown;
    X.p[q + AUX_GAM * X.ns] = gam;
}

// ---------------------------------------------------------------------------
// face_kernel: per-face scalars for direction d
// ---------------------------------------------------------------------------
// Faces of direction d (growHi(bx, d, 1)).
__device__ __forceinline__ int64_t face_count(const RhsBox& B, int d) {
    int64_t nf = 1;
    for (int e = 0; e < 3; ++e) nf *= B.hi[e] - B.lo[e] + 1 + (e == d);
    return nf;
}

// Whether face f of direction d takes the flux branch of face_body
// (Navier-Stokes terms on and face volume fraction >= 1/2), by the same
// arithmetic.
__device__ __forceinline__ bool face_active(const RhsBox& B, int d, const Idx3& f) {
    const Fab& S = B.sb;
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t oR = S.off(f.i, f.j, f.k);
    const double* vf = S.p + VFRAC * S.ns;
    // 0.5 (a + b) >= 0.5 exactly when a + b >= 1 (the halving is exact)
    return c_P.do_ns && nonneg_ge(vf[oR - sd] + vf[oR], 1.0);
}

// Face f of direction d.  SOLID_SIDE: the caller knows the face is not
// active and the pass is the split form of orders 1/2 with Navier-Stokes
// terms (face_split_kernel); the flux branch and the first-order fallback
// test (used only by the flux branch and the stored face scalars of orders
// 4/5) are compiled out, the remaining arithmetic is the same.
template <int NS, bool SOLID_SIDE = false>
__device__ __forceinline__ void face_body_at(const RhsBox& B, int d, const Idx3& f) {
    const DevParams& P = c_P;
    const Fab& S = B.sb;
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
    const int64_t st1 = (t1 == 0) ? 1 : (t1 == 1) ? S.js : S.ks;
    const int64_t st2 = (t2 == 0) ? 1 : (t2 == 1) ? S.js : S.ks;
    const int64_t oR = S.off(f.i, f.j, f.k);  // right cell: face i separates i-1 and i
    const int64_t oL = oR - sd;
    const double* vf = S.p + VFRAC * S.ns;

    bool fallback = false;
    if (!SOLID_SIDE) {
#pragma unroll
        for (int q = -3; q <= 2; ++q) fallback |= below_one(vf[oR + q * sd]);
    }
    // face volume fraction 0.5 (a + b) >= 0.5, i.e. a + b >= 1 (the halving is exact)
    const bool active = !SOLID_SIDE && P.do_ns && nonneg_ge(vf[oL] + vf[oR], 1.0);

    double fs[NFS];
#pragma unroll
    for (int q = 0; q < NFS; ++q) fs[q] = 0.0;
    fs[FS_FLAGS] = __longlong_as_double((active ? 1 : 0) | ((P.do_ns && fallback) ? 2 : 0));  // bit pattern
    double uL[NCONS + NS], uR[NCONS + NS];  // AUSM+-up face states (orders 1, 2)
    double vise = 0.0;                      // viscous work of the energy flux (orders 1, 2)

    if (active) {
        const int ord = P.order_hyp;
        if (ord == 5 || ord == 4) {
            const Fab& X = B.aux;
            const int64_t qL = X.off(f.i, f.j, f.k) - ((d == 0) ? 1 : (d == 1) ? X.js : X.ks);
            const int64_t qR = X.off(f.i, f.j, f.k);
            const double* vd = X.p + (AUX_VX + d) * X.ns;
            const double veln = max_nonneg(fabs(vd[qL]), fabs(vd[qR]));
            const double aL = X.p[qL + AUX_AOWN * X.ns];
            double aR;
            if (ord == 5) {
                // presR is evaluated with the left cell's species (flux_schemes.H:33)
                double specL[NS];
#pragma unroll
                for (int s = 0; s < NS; ++s) specL[s] = (s < P.nspec) ? S.p[oL + (NFLO + s) * S.ns] : 0.0;
                const double rhoR = S.p[oR + RHO * S.ns];
                const double pR = thermo_p<NS>(X.p[qR + AUX_REIG * X.ns], rhoR, specL);
                aR = sqrt((X.p[qR + AUX_GAM * X.ns] * pR) / rhoR);
            } else {
                aR = X.p[qR + AUX_AOWN * X.ns];
            }
            fs[FS_LAMBDA] = max_nonneg(aL, aR) + veln;
        } else {
            // AUSM+-up (flux_schemes.H:185-310) on first- or second-order states
            const int nc = NCONS + P.nspec;
#pragma unroll
            for (int c = 0; c < NCONS + NS; ++c) {
                if (c >= nc) { uL[c] = uR[c] = 0.0; continue; }
                const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
                double ul = S.p[oL + sc * S.ns], ur = S.p[oR + sc * S.ns];
                if (ord == 2) {
                    double ulm1 = fallback ? ul : S.p[oL - sd + sc * S.ns];
                    double urp1 = fallback ? ur : S.p[oR + sd + sc * S.ns];
                    muscl(ulm1, ul, ur, urp1, uL[c], uR[c]);
                } else {
                    uL[c] = ul;
                    uR[c] = ur;
                }
            }
            const double rL = uL[RHO], rR = uR[RHO];
            const double irL = rcp_pos(rL), irR = rcp_pos(rR);
            // kinetic energy density |m|^2 / (2 rho) from the momenta and the
            // normal velocity (the transverse velocities are not needed)
            const double hkL = (0.5 * ((uL[RHOU] * uL[RHOU] + uL[RHOV] * uL[RHOV]) + uL[RHOW] * uL[RHOW])) * irL;
            const double hkR = (0.5 * ((uR[RHOU] * uR[RHOU] + uR[RHOV] * uR[RHOV]) + uR[RHOW] * uR[RHOW])) * irR;
            const double pL = thermo_p<NS>(uL[RHOE] - hkL, rL, uL + NCONS);
            const double pR = thermo_p<NS>(uR[RHOE] - hkR, rR, uR + NCONS);
            const double gL = thermo_gamma<NS>(rL, uL + NCONS), gR = thermo_gamma<NS>(rR, uR + NCONS);
            const double vL = ((d == 0) ? uL[RHOU] : (d == 1) ? uL[RHOV] : uL[RHOW]) * irL;
            const double vR = ((d == 0) ? uR[RHOU] : (d == 1) ? uR[RHOV] : uR[RHOW]) * irR;
            const bool cg = P.thermo_kind == MFG_THERMO_MASS_SINGLE;
            // gamma/(gamma-1) and 2(gamma-1)/(gamma+1): constants of the single-gas
            // family, else per face state with reciprocals of the positive gamma +- 1
            double gfL = P.g_gm1, gfR = P.g_gm1, afL = P.astar_fac, afR = P.astar_fac;
            if (!cg) {
                gfL = gL * rcp_pos(gL - 1.0);
                gfR = gR * rcp_pos(gR - 1.0);
                afL = (2.0 * (gL - 1.0)) * rcp_pos(gL + 1.0);
                afR = (2.0 * (gR - 1.0)) * rcp_pos(gR + 1.0);
            }
            // total enthalpy gamma/(gamma-1) p/rho + |v|^2/2 = (gf p + |m|^2/(2 rho)) / rho
            const double HL = fma(gfL, pL, hkL) * irL;
            const double HR = fma(gfR, pR, hkR) * irR;
            const double rsum = rL + rR;
            // a_hat = a*^2 / max(a*, |v|) per side, a_1/2 = min(a_hat_L, a_hat_R)
            // and its reciprocal.  On a subsonic side (a* >= |v|, tested as
            // a*^2 >= v^2) a_hat = a*, so when both sides are subsonic a_1/2 is
            // the square root of the smaller a*^2: a_1/2 = m rsqrt(m) and
            // 1/a_1/2 = rsqrt(m), one reciprocal square root and no reciprocal.
            // Otherwise each side as a* or a*^2/|v| (and |v|/a*^2), the smaller.
            const double as2L = afL * HL, as2R = afR * HR;
            double ah, iah;
            if (nonneg_ge(as2L, vL * vL) && nonneg_ge(as2R, vR * vR)) {
                const double m = min_nonneg(as2L, as2R);
                iah = rsqrt(m);
                ah = m * iah;
            } else {
                double irs = rsqrt(as2L);
                double ahL = as2L * irs, iahL = irs;
                if (!nonneg_ge(ahL, fabs(vL))) {
                    ahL = as2L * rcp_pos(fabs(vL));
                    iahL = fabs(vL) * rcp_pos(as2L);
                }
                irs = rsqrt(as2R);
                double ahR = as2R * irs, iahR = irs;
                if (!nonneg_ge(ahR, fabs(vR))) {
                    ahR = as2R * rcp_pos(fabs(vR));
                    iahR = fabs(vR) * rcp_pos(as2R);
                }
                const bool left = nonneg_le(ahL, ahR);
                ah = left ? ahL : ahR;
                iah = left ? iahL : iahR;
            }
            const double ML = vL * iah, MR = vR * iah;
            double Mh = split_mach_p(ML) + split_mach_m(MR);
            const double Mb2 = 0.5 * (ML * ML + MR * MR);
            // M_o = sqrt(min(1, max(Mb^2, 0.3^2))) as x rsqrt(x) on the clamped x
            const double xmo = min_nonneg(1.0, max_nonneg(Mb2, 0.3 * 0.3));
            const double Mo = xmo * rsqrt(xmo);
            const double fa = Mo * (2.0 - Mo);
            // pressure diffusion term (p_R - p_L) / (fa rho_1/2 a_1/2^2) / 4, rho_1/2 = (rho_L + rho_R) / 2
            Mh = Mh - ((pos_part(1.0 - Mb2) * (pR - pL)) * (iah * iah)) * (0.5 * rcp_pos(fa * rsum));
            double modM = fabs(Mh);
            if (nonneg_le(modM, 0.3)) modM = (Mh * Mh + 0.3 * 0.3) * (1.0 / (2.0 * 0.3));
            // alpha = 3/16 (-4 + 5 fa^2) as (15/16 fa) fa - 3/4
            const double alpha = fma((15.0 / 16.0) * fa, fa, -0.75);
            const double PLp = split_pres_p(ML, alpha), PRm = split_pres_m(MR, alpha);
            double ph = PLp * pL + PRm * pR;
            ph = ph - ((((0.75 * PLp) * PRm) * rsum) * (fa * ah)) * (vR - vL);
            fs[FS_LAMBDA] = ah;
            fs[FS_MH] = Mh;
            fs[FS_MODM] = modM;
            fs[FS_PH] = ph;
            fs[FS_PL] = pL;
            fs[FS_PR] = pR;
        }
        // viscous stress (compute_flux_3d.H:293-367); lagged primitive velocities
        const double* V0 = S.p + VELX * S.ns;
        const double* V1 = S.p + VELY * S.ns;
        const double* V2 = S.p + VELZ * S.ns;
        // transverse derivatives (0.5 (a + b) - 0.5 (c + d)) / (2 dx) formed as
        // ((a + b) - (c + d)) / (4 dx)
        const double ids = B.idx[d], iq1 = 0.25 * B.idx[t1], iq2 = 0.25 * B.idx[t2];
        // Only the stress row of the face normal is needed: tau_{d a} uses the
        // normal derivatives of all three velocities, the two transverse
        // derivatives of the normal velocity, and the divergence's two other
        // diagonal terms (7 of the 9 gradients, 3 of the 9 stresses).
        const double* Vd = (d == 0) ? V0 : (d == 1) ? V1 : V2;
        const double* Vt1 = (t1 == 0) ? V0 : (t1 == 1) ? V1 : V2;
        const double* Vt2 = (t2 == 0) ? V0 : (t2 == 1) ? V1 : V2;
        // normal differences; the derivative (x 1/dx) is formed only where the
        // divergence needs it, the shear terms fold the scale into an FMA
        const double dn[3] = {V0[oR] - V0[oL], V1[oR] - V1[oL], V2[oR] - V2[oL]};
        const double gnd = dn[d] * ids;
        const double d_t1 = ((Vd[oL + st1] + Vd[oR + st1]) - (Vd[oL - st1] + Vd[oR - st1])) * iq1;
        const double d_t2 = ((Vd[oL + st2] + Vd[oR + st2]) - (Vd[oL - st2] + Vd[oR - st2])) * iq2;
        // the divergence's two transverse diagonal terms, each scaled inside
        // the FMA that adds it: div V = dV_d/dx_d + dV_t1/dx_t1 + dV_t2/dx_t2
        const double s1 = (Vt1[oL + st1] + Vt1[oR + st1]) - (Vt1[oL - st1] + Vt1[oR - st1]);
        const double s2 = (Vt2[oL + st2] + Vt2[oR + st2]) - (Vt2[oL - st2] + Vt2[oR - st2]);
        // viscosity always from cells (i,j,k) and (i-1,j,k) (compute_flux_3d.H:179)
        const double mu = (P.visc_mode == MFG_TRANSPORT_CONST)
                              ? P.visc_hm
                              : harmonic_mean(blend(P.visc_mode, P.visc_gas, P.visc_solid, vf[oR]),
                                              blend(P.visc_mode, P.visc_gas, P.visc_solid, vf[oR - 1]));
        const double delu = fma(s2, iq2, fma(s1, iq1, gnd));
        // face velocities times 2 (the halving moves to the work sum)
        const double fv2[3] = {V0[oL] + V0[oR], V1[oL] + V1[oR], V2[oL] + V2[oR]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            // tau_{d a}: mu (2 dV_d/dx_d - 2/3 div V) on the diagonal, else
            // mu (dV_d/dx_a + dV_a/dx_d)
            const double tn = (a == d) ? mu * (2.0 * gnd - kTwo3rd * delu)
                                       : mu * fma(dn[a], ids, (a == t1) ? d_t1 : d_t2);
            fs[FS_VIS + a] = tn;
            if (ord >= 4) fs[FS_VISE + a] = tn * (0.5 * fv2[a]);
        }
        // orders 1, 2: the viscous work sum_a tau_{d a} v_a of the energy flux
        // with fused multiply-adds (the face thread assembles that flux itself)
        if (ord <= 2)
            vise = 0.5 * fma(fs[FS_VIS + 0], fv2[0], fma(fs[FS_VIS + 1], fv2[1], fs[FS_VIS + 2] * fv2[2]));
    }
    if (P.do_ns) {
        // heat conduction (compute_flux_3d.H:373-374), conductivity from (i,j,k),(i-1,j,k)
        const double kc = (P.cond_mode == MFG_TRANSPORT_CONST)
                              ? P.cond_hm
                              : harmonic_mean(blend(P.cond_mode, P.cond_gas, P.cond_solid, vf[oR]),
                                              blend(P.cond_mode, P.cond_gas, P.cond_solid, vf[oR - 1]));
        const double* T = S.p + TEMP * S.ns;
        fs[FS_THERM] = kc * ((T[oR] - T[oL]) * B.idx[d]);
    }
    if (SOLID_SIDE || (P.do_ns && P.order_hyp <= 2)) {
        // AUSM+-up: the face thread holds the face states and the scheme scalars,
        // so it writes every component's complete flux (no per-component pass).
        const Fab& O = B.flx[d];
        const int64_t qo = O.off(f.i, f.j, f.k);
        const Fab& U = B.uflux[d];
        const int64_t qu = U.p ? U.off(f.i, f.j, f.k) : 0;
        // AUSM+-up mass-flux weights of the face, the wave speed folded in:
        // fh = (M/2 (fL + fR) - |M|/2 (fR - fL)) a_half per component, as
        // wL fL + wR fR with wL = (M + |M|) a_half / 2, wR = (M - |M|) a_half / 2
        // (two FP64 operations per component instead of four)
        const double cmh = (0.5 * fs[FS_MH]) * fs[FS_LAMBDA], cmod = (0.5 * fs[FS_MODM]) * fs[FS_LAMBDA];
        const double wL = cmh + cmod, wR = cmh - cmod;
#pragma unroll
        for (int c = 0; c < NCONS + NS; ++c) {
            if (c >= NCONS + P.nspec) break;
            const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
            double F = 0.0;
            if (active) {
                double fL = uL[c], fR = uR[c];
                if (c == RHOE) {
                    fL = uL[c] + fs[FS_PL];
                    fR = uR[c] + fs[FS_PR];
                }
                double fh = fma(wR, fR, wL * fL);
                if (c == 1 + d) fh += fs[FS_PH];
                F = (c < NCONS) ? fh : P.advect_flag[c - NCONS] * fh;
                if (c >= RHOU && c <= RHOW) F -= fs[FS_VIS + c - 1];
                if (c == RHOE) F -= vise;
            }
            if (c == RHOE) F -= fs[FS_THERM];
            if (c >= NCONS) {
                const int s = c - NCONS;
                const double Dh = (P.diff_mode[s] == MFG_TRANSPORT_CONST)
                                      ? P.diff_hm[s]
                                      : harmonic_mean(blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oL]),
                                                      blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf[oR]));
                F -= (Dh * (S.p[oR + sc * S.ns] - S.p[oL + sc * S.ns])) * B.idx[d];
            }
            O.p[qo + c * O.ns] = F;
            if (U.p) U.p[qu + sc * U.ns] = F;
        }
        if (U.p)
            for (int z = NCONS; z < NFLO; ++z) U.p[qu + z * U.ns] = 0.0;
        return;
    }
    const Fab& F = B.fs[d];
    const int64_t q = F.off(f.i, f.j, f.k);
#pragma unroll
    for (int c = 0; c < NFS; ++c) F.p[q + c * F.ns] = fs[c];
}

// Face t (linear index over growHi(bx, d, 1)) of direction d.
template <int NS>
__device__ __forceinline__ void face_body(const RhsBox& B, int d, int64_t t) {
    int lo[3] = {B.lo[0], B.lo[1], B.lo[2]}, len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    const int64_t nf = (int64_t)len[0] * len[1] * len[2];
    if (t >= nf) return;
    face_body_at<NS>(B, d, delinear(t, lo, len));
}

// ---------------------------------------------------------------------------
// flux_kernel: per (face, component) along d
// ---------------------------------------------------------------------------
template <bool FAST>
__device__ __forceinline__ void flux_body(const RhsBox& B, int d, int c, int64_t t) {
    int lo[3] = {B.lo[0], B.lo[1], B.lo[2]}, len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    const int64_t nf = (int64_t)len[0] * len[1] * len[2];
    if (t >= nf) return;  // c: advected component 0..4, 5.. = species
    const Idx3 f = delinear(t, lo, len);
    const DevParams& P = c_P;
    const Fab& S = B.sb;
    const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);  // state component
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t oR = S.off(f.i, f.j, f.k);
    const int64_t oL = oR - sd;
    const Fab& FS = B.fs[d];
    const int64_t qf = FS.off(f.i, f.j, f.k);
    const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
    const bool active = flags & 1, fallback = flags & 2;
    const double* u = S.p + sc * S.ns;

    double F = 0.0;
    if (P.do_ns) {
        if (active) {
            const int ord = P.order_hyp;
            double fh;
            if (ord == 5 || ord == 4) {
                const Fab& X = B.aux;
                const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
                const int64_t xR = X.off(f.i, f.j, f.k);
                const double lam = FS.p[qf + FS_LAMBDA * FS.ns];
                double us[6], fl[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    int qq = q - 3;
                    if (fallback) qq = (q < 3) ? -1 : 0;  // first-order stencil (:233-249)
                    const int64_t os = oR + qq * sd, ox = xR + qq * xd;
                    us[q] = u[os];
                    const double rho = S.p[os + RHO * S.ns];
                    const double vd = X.p[ox + (AUX_VX + d) * X.ns];
                    const double va = (c >= 1 && c <= 3) ? X.p[ox + (AUX_VX + c - 1) * X.ns] : 0.0;
                    const double p = X.p[ox + AUX_PF * X.ns];
                    const double E = S.p[os + RHOE * S.ns];
                    fl[q] = euler_flux(c, d, us[q], rho, va, vd, p, E);
                }
                if (ord == 5) {
                    double fp, fm, up, um;
                    weno_face<FAST>(fl, fp, fm);
                    weno_face<FAST>(us, up, um);
                    fh = 0.5 * (fp + lam * up) + 0.5 * (fm - lam * um);
                } else {
                    // central_with_diss_flux(ul, ur, ulm1, urp1): uim1=ul, ui=ur, uim2=ulm1, uip1=urp1
                    fh = kTwelveth * (((7.0 * fl[3] + 7.0 * fl[2]) - fl[1]) - fl[4]);
                    fh -= ((kTwelveth * (((3.0 * us[3] - 3.0 * us[2]) - us[4]) + us[3])) * lam) * P.dissfactor;
                }
            } else {
                double ul = u[oL], ur = u[oR], uLh = ul, uRh = ur;
                if (ord == 2) {
                    const double ulm1 = fallback ? ul : u[oL - sd];
                    const double urp1 = fallback ? ur : u[oR + sd];
                    muscl(ulm1, ul, ur, urp1, uLh, uRh);
                }
                const double Mh = FS.p[qf + FS_MH * FS.ns];
                const double modM = FS.p[qf + FS_MODM * FS.ns];
                const double ah = FS.p[qf + FS_LAMBDA * FS.ns];
                double fL = uLh, fR = uRh;
                if (c == RHOE) {
                    fL = uLh + FS.p[qf + FS_PL * FS.ns];
                    fR = uRh + FS.p[qf + FS_PR * FS.ns];
                }
                fh = ((0.5 * Mh) * (fL + fR) - (0.5 * modM) * (fR - fL)) * ah;
                if (c == 1 + d) fh += FS.p[qf + FS_PH * FS.ns];
            }
            F = (c < NCONS) ? fh : P.advect_flag[c - NCONS] * fh;
            if (c >= RHOU && c <= RHOW) F -= FS.p[qf + (FS_VIS + c - 1) * FS.ns];
            if (c == RHOE) {
                F -= FS.p[qf + (FS_VISE + 0) * FS.ns];
                F -= FS.p[qf + (FS_VISE + 1) * FS.ns];
                F -= FS.p[qf + (FS_VISE + 2) * FS.ns];
            }
        }
        if (c == RHOE) F -= FS.p[qf + FS_THERM * FS.ns];
    } else if (c >= NCONS) {
        // species convection without Navier-Stokes (compute_flux_3d.H:382-421);
        // the limited states reduce to first order (by-value limiter, :69-83)
        const double* vfp = S.p + VFRAC * S.ns;
        const double* Vd = S.p + (VELX + d) * S.ns;
        double velface = 0.5 * (Vd[oL] + Vd[oR]);
        if (P.species_in_solid) {
            const double w = (vfp[oL] < 1.0) ? 0.0 : 1.0;  // both weights test the left cell (:410-411)
            velface = (w * Vd[oL] + w * Vd[oR]) / ((w + w) + kTiny);
        }
        F = P.advect_flag[c - NCONS] *
            ((0.5 * (velface + fabs(velface))) * u[oL] + (0.5 * (velface - fabs(velface))) * u[oR]);
    }
    if (c >= NCONS) {
        // species diffusion (compute_flux_3d.H:425-428)
        const int s = c - NCONS;
        const double* vfp = S.p + VFRAC * S.ns;
        const double Dh = (P.diff_mode[s] == MFG_TRANSPORT_CONST)
                              ? P.diff_hm[s]
                              : harmonic_mean(blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vfp[oL]),
                                              blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vfp[oR]));
        F -= (Dh * (u[oR] - u[oL])) * B.idx[d];
    }
    const Fab& O = B.flx[d];
    O.p[O.off(f.i, f.j, f.k) + c * O.ns] = F;
    if (B.uflux[d].p) {
        const Fab& U = B.uflux[d];
        const int64_t qu = U.off(f.i, f.j, f.k);
        U.p[qu + sc * U.ns] = F;
        if (c == 0)
            for (int z = NCONS; z < NFLO; ++z) U.p[qu + z * U.ns] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// update_kernel: per (cell, component): divergence, masking, RK stage
// ---------------------------------------------------------------------------
// One component n of the valid cell x (volume fraction vfrac): the body of
// both launch shapes below, so they round identically.
__device__ __forceinline__ void update_one(const RhsBox& B, int stage, double dt, int n, const Idx3& x,
                                           double vfrac) {
    const DevParams& P = c_P;
    const bool advected = (n < NCONS) || (n >= NFLO);
    if (!advected && is_finite_bits(dt) && __double_as_longlong(dt) >= 0) {
        // A component without a flux (velocities, pressure, temperature,
        // density, vfrac) has the rate +0 exactly, so for a finite dt >= +0
        // dt * ds = +0 and v + dt * ds = v + 0 (plus_zero): the same bits
        // without the two FP64 operations.  n and dt are uniform over a block, so this is a branch
        // of whole warps, not a predicated path.
        if (B.dsdt.p) B.dsdt(x.i, x.j, x.k, n) = 0.0;
        if (stage == 1) {
            B.snew(x.i, x.j, x.k, n) = plus_zero(B.sb(x.i, x.j, x.k, n));
        } else if (stage == 2) {
            double v = plus_zero(B.snew(x.i, x.j, x.k, n));
            v = add(v, mul(3.0, B.sold(x.i, x.j, x.k, n)));
            B.snew(x.i, x.j, x.k, n) = mul(v, 0.25);
        } else if (stage == 3) {
            double v = plus_zero(B.snew(x.i, x.j, x.k, n));
            v = add(B.sold(x.i, x.j, x.k, n), mul(2.0, v));
            B.snew(x.i, x.j, x.k, n) = mul(v, kThird);
        }
        return;
    }
    double ds = 0.0;
    if (advected) {
        const int c = (n < NCONS) ? n : n - (NFLO - NCONS);
        const Fab &Fx = B.flx[0], &Fy = B.flx[1], &Fz = B.flx[2];
        const int64_t ox = Fx.off(x.i, x.j, x.k) + c * Fx.ns;
        const int64_t oy = Fy.off(x.i, x.j, x.k) + c * Fy.ns;
        const int64_t oz = Fz.off(x.i, x.j, x.k) + c * Fz.ns;
        // explicit FMAs: every compiled copy of this body rounds the same way
        ds = __fma_rn(Fz.p[oz] - Fz.p[oz + Fz.ks], B.idx[2],
                      __fma_rn(Fy.p[oy] - Fy.p[oy + Fy.js], B.idx[1], mul(Fx.p[ox] - Fx.p[ox + 1], B.idx[0])));
        ds = plus_zero(ds);  // + source (compute_fluid_source is zero)
    }
    const int nnull = (P.species_in_solid == 1) ? NFLO : NFLO + P.nspec;
    // vfrac tests and the NaN test on the integer pipe
    if (n != RHOE) {
        if (n < nnull && below_one(vfrac)) ds = 0.0;
    } else if (!P.conj_ht) {
        if (below_one(vfrac)) ds = 0.0;
    } else if (is_positive(vfrac) && below_one(vfrac)) {
        ds = 0.0;
    }
    if (is_nan(ds)) raise_status(MFG_STATUS_NAN);
    if (B.dsdt.p) B.dsdt(x.i, x.j, x.k, n) = ds;
    // The stage algebra of the advected components with fused multiply-adds
    // (one rounding less per product than the reference's separate ones, 3
    // instead of 5 FP64 operations in stages 2 and 3); the components without
    // a flux above keep the reference's rounding, so the volume fraction and
    // the cut-cell classification it drives evolve exactly as there.
    if (stage == 1) {
        B.snew(x.i, x.j, x.k, n) = __fma_rn(dt, ds, B.sb(x.i, x.j, x.k, n));
    } else if (stage == 2) {
        double v = __fma_rn(dt, ds, B.snew(x.i, x.j, x.k, n));
        v = __fma_rn(3.0, B.sold(x.i, x.j, x.k, n), v);
        B.snew(x.i, x.j, x.k, n) = mul(v, 0.25);
    } else if (stage == 3) {
        double v = __fma_rn(dt, ds, B.snew(x.i, x.j, x.k, n));
        v = __fma_rn(2.0, v, B.sold(x.i, x.j, x.k, n));
        B.snew(x.i, x.j, x.k, n) = mul(v, kThird);
    }
}

__device__ __forceinline__ void update_body(const RhsBox& B, int stage, double dt, int n, int64_t t) {
    int lo[3] = {B.lo[0], B.lo[1], B.lo[2]}, len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1;
    const int64_t nc = (int64_t)len[0] * len[1] * len[2];
    if (t >= nc) return;  // n: state component
    const Idx3 x = delinear(t, lo, len);
    const bool advected = (n < NCONS) || (n >= NFLO);
    // the flux-less components' fast path reads no volume fraction
    update_one(B, stage, dt, n, x, advected ? B.sb(x.i, x.j, x.k, VFRAC) : 0.0);
}


// ---------------------------------------------------------------------------
// WENO5 column sweep (order 5 with Navier-Stokes terms, one-division mode):
// one thread walks a segment of faces along d for one component, keeping the
// per-cell parts of the reconstruction in registers.
//
// The six smoothness indicators and six candidate polynomials of a face's two
// WENO5-JS edges (flux_schemes.H:373-446) are functions of the three cells
// centred on f-2, f-1, f, f+1; per centre y with neighbours (x, y, z) there
// are three distinct indicators, K1 t^2 + A with t = x - 2y + z and
// A = (3x-4y+z)^2/4, (x-4y+3z)^2/4 or (x-z)^2/4, and four distinct
// polynomials.  Computing them once per cell instead of once per face use
// (six uses) and rebuilding each cell's Euler flux once instead of six times
// removes most of the per-face FP64 work; each face then only combines the
// nonlinear weights.  The left edge uses (B, C, A) at centres (f-2, f-1, f),
// the right edge (A, C, B) at (f+1, f, f-1).  Results differ from the
// per-face form by rounding only (the mirrored edge evaluates the same
// polynomials with operands in the other order).
// ---------------------------------------------------------------------------
constexpr int SWEEP_SEG = 32;  // longest face segment per thread (batched launches)

// Per stencil centre: the three smoothness indicators already in the form the
// weights use, (eps + beta)^2 (each is needed by one left and one right edge),
// and the candidate polynomials.
struct WenoCell {
    double dA, dB, dC, p1, p2, p3, p4;
};

// The sweep and the per-face form must round identically, so every operation
// of the per-cell and per-face parts is an explicit intrinsic (the compiler
// may neither contract nor reorder them differently in the two contexts).
__device__ __forceinline__ WenoCell weno_cell(double x, double y, double z) {
    WenoCell r;
    // t = x - 2y + z, tA = 3x - 4y + z, tB = x - 4y + 3z = 4t - tA, q = x - z
    const double t = __dadd_rn(__fma_rn(-2.0, y, x), z);
    const double m4y = __dmul_rn(-4.0, y);
    const double tA = __dadd_rn(__fma_rn(3.0, x, m4y), z);
    const double tB = __fma_rn(4.0, t, -tA);
    const double q = __dsub_rn(x, z);
    // eps + K1 t^2 + u^2/4 for the three u, with eps folded into the shared term
    const double kte = __fma_rn(__dmul_rn(13.0 / 12.0, t), t, kEpsWeno);
    const double sA = __fma_rn(__dmul_rn(0.25, tA), tA, kte);
    const double sB = __fma_rn(__dmul_rn(0.25, tB), tB, kte);
    const double sC = __fma_rn(__dmul_rn(0.25, q), q, kte);
    r.dA = __dmul_rn(sA, sA);
    r.dB = __dmul_rn(sB, sB);
    r.dC = __dmul_rn(sC, sC);
    // candidates (times 6): 2x - 7y + 11z, -x + 5y + 2z, 2x + 5y - z, 11x - 7y + 2z
    const double m7y = __dmul_rn(-7.0, y), y5 = __dmul_rn(5.0, y);
    r.p1 = __fma_rn(11.0, z, __fma_rn(2.0, x, m7y));
    r.p2 = __fma_rn(2.0, z, __dsub_rn(y5, x));
    r.p3 = __fma_rn(2.0, x, __dsub_rn(y5, z));
    r.p4 = __fma_rn(11.0, x, __fma_rn(2.0, z, m7y));
    return r;
}

// Nonlinear combination of one edge: (eps + beta)^2 of the three candidates
// d2, d1, d0 with linear weights 1, 6, 3 and candidates v2, v1, v0 (divided
// by 6).  The weight sum is a positive normal number, so a Newton-refined
// reciprocal replaces the division.
__device__ __forceinline__ double weno_comb(double d2, double d1, double d0, double v2, double v1, double v0) {
    const double e2 = __dmul_rn(d1, d0), e1 = __dmul_rn(6.0, __dmul_rn(d2, d0)), e0 = __dmul_rn(3.0, __dmul_rn(d2, d1));
    const double num = __fma_rn(e0, v0, __fma_rn(e1, v1, __dmul_rn(e2, v2)));
    const double den = __dadd_rn(__dadd_rn(e2, e1), e0);
    return __dmul_rn(num, rcp_pos(__dmul_rn(6.0, den)));
}

// Transverse directions of a sweep along d (the first one is x when d != 0,
// so consecutive threads read consecutive addresses).
__host__ __device__ __forceinline__ void sweep_dirs(int d, int& a, int& b) {
    a = (d == 0) ? 1 : 0;
    b = (d == 2) ? 1 : 2;
}

__host__ __device__ __forceinline__ int sweep_nseg(const RhsBox& B, int d, int seg) {
    const int nf = B.hi[d] - B.lo[d] + 2;
    return (nf + seg - 1) / seg;
}

__host__ __device__ __forceinline__ int64_t sweep_items(const RhsBox& B, int d, int seg = SWEEP_SEG) {
    int a, b;
    sweep_dirs(d, a, b);
    return (int64_t)(B.hi[a] - B.lo[a] + 1) * (B.hi[b] - B.lo[b] + 1) * sweep_nseg(B, d, seg);
}

// Raw values of one cell for component c: the state and its Euler flux along d.
__device__ __forceinline__ void sweep_raw(const RhsBox& B, int d, int c, int sc, int64_t os, int64_t ox, double& u,
                                          double& f) {
    const Fab& S = B.sb;
    const Fab& X = B.aux;
    u = S.p[os + sc * S.ns];
    const double va = (c >= 1 && c <= 3) ? X.p[ox + (AUX_VX + c - 1) * X.ns] : 0.0;
    f = euler_flux(c, d, u, S.p[os + RHO * S.ns], va, X.p[ox + (AUX_VX + d) * X.ns], X.p[ox + AUX_PF * X.ns],
                   S.p[os + RHOE * S.ns]);
}

// First-order stencil near the immersed boundary (compute_flux_3d.H:233-249):
// the six cells collapse to (L, L, L, R, R, R).  Both edges then have the
// indicators 0, (K1 + 1/4) D^2 and (K1 + 9/4) D^2 with D = R - L, hence the
// same nonlinear weights, and the candidates 6L, 4L + 2R, 2L + 4R (left edge)
// and their mirror images (right edge).
__device__ __forceinline__ void weno_collapsed(double L, double R, double& up, double& um) {
    const double D = __dsub_rn(R, L), D2 = __dmul_rn(D, D);
    const double s2 = kEpsWeno, s1 = __fma_rn(13.0 / 12.0 + 0.25, D2, kEpsWeno),
                 s0 = __fma_rn(13.0 / 12.0 + 2.25, D2, kEpsWeno);
    const double d2 = __dmul_rn(s2, s2), d1 = __dmul_rn(s1, s1), d0 = __dmul_rn(s0, s0);
    const double e2 = __dmul_rn(d1, d0), e1 = __dmul_rn(6.0, __dmul_rn(d2, d0)), e0 = __dmul_rn(3.0, __dmul_rn(d2, d1));
    const double r = rcp_pos(__dmul_rn(6.0, __dadd_rn(__dadd_rn(e2, e1), e0)));
    const double vl1 = __fma_rn(2.0, R, __dmul_rn(4.0, L)), vl0 = __fma_rn(4.0, R, __dmul_rn(2.0, L));
    const double vr1 = __fma_rn(2.0, L, __dmul_rn(4.0, R)), vr0 = __fma_rn(4.0, L, __dmul_rn(2.0, R));
    up = __dmul_rn(__fma_rn(e0, vl0, __fma_rn(e1, vl1, __dmul_rn(e2, __dmul_rn(6.0, L)))), r);
    um = __dmul_rn(__fma_rn(e0, vr0, __fma_rn(e1, vr1, __dmul_rn(e2, __dmul_rn(6.0, R)))), r);
}

// The four cells of a face's stencil (centres f-2 .. f+1) for the state and
// for the Euler flux of one component.
struct WenoWindow {
    WenoCell u0, u1, u2, u3, f0, f1, f2, f3;
};

// Flux of component c through one face (the sweep and the per-face form share
// it, so they agree bitwise): uL/uR and fL/fR are the state and Euler flux of
// the two cells next to the face, vfL/vfR their volume fractions.
__device__ __forceinline__ double flux5_face(const RhsBox& B, int d, int c, const Fab& FS, int64_t qf,
                                             const WenoWindow& w, double uL, double uR, double fL, double fR,
                                             double vfL, double vfR, bool hyper = true) {
    const DevParams& P = c_P;
    const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
    double F = 0.0;
    if (hyper && (flags & 1)) {
        const double lam = FS.p[qf + FS_LAMBDA * FS.ns];
        double fp, fm, up, um;
        if (!(flags & 2)) {
            fp = weno_comb(w.f0.dB, w.f1.dC, w.f2.dA, w.f0.p1, w.f1.p2, w.f2.p3);
            fm = weno_comb(w.f3.dA, w.f2.dC, w.f1.dB, w.f3.p4, w.f2.p3, w.f1.p2);
            up = weno_comb(w.u0.dB, w.u1.dC, w.u2.dA, w.u0.p1, w.u1.p2, w.u2.p3);
            um = weno_comb(w.u3.dA, w.u2.dC, w.u1.dB, w.u3.p4, w.u2.p3, w.u1.p2);
        } else {
            weno_collapsed(fL, fR, fp, fm);
            weno_collapsed(uL, uR, up, um);
        }
        const double fh = __fma_rn(0.5, __fma_rn(lam, up, fp), __dmul_rn(0.5, __fma_rn(-lam, um, fm)));
        F = (c < NCONS) ? fh : __dmul_rn(P.advect_flag[c - NCONS], fh);
        if (c >= RHOU && c <= RHOW) F = __dsub_rn(F, FS.p[qf + (FS_VIS + c - 1) * FS.ns]);
        if (c == RHOE) {
            F = __dsub_rn(F, FS.p[qf + (FS_VISE + 0) * FS.ns]);
            F = __dsub_rn(F, FS.p[qf + (FS_VISE + 1) * FS.ns]);
            F = __dsub_rn(F, FS.p[qf + (FS_VISE + 2) * FS.ns]);
        }
    }
    if (c == RHOE) F = __dsub_rn(F, FS.p[qf + FS_THERM * FS.ns]);
    if (c >= NCONS) {  // species diffusion (compute_flux_3d.H:425-428)
        const int s = c - NCONS;
        double Dh = P.diff_hm[s];
        if (P.diff_mode[s] != MFG_TRANSPORT_CONST) {  // harmonic mean of gas vf + solid (1 - vf)
            const double g = P.diff_gas[s], so = P.diff_solid[s];
            const double dl = __fma_rn(g, vfL, __dmul_rn(so, __dsub_rn(1.0, vfL)));
            const double dr = __fma_rn(g, vfR, __dmul_rn(so, __dsub_rn(1.0, vfR)));
            Dh = __ddiv_rn(__dmul_rn(__dmul_rn(2.0, dl), dr), __dadd_rn(__dadd_rn(dl, dr), 1e-30));
        }
        F = __fma_rn(-__dmul_rn(Dh, __dsub_rn(uR, uL)), B.idx[d], F);
    }
    return F;
}

__device__ __forceinline__ void flux5_store(const RhsBox& B, int d, int c, int sc, const Idx3& f, double F) {
    const Fab& O = B.flx[d];
    O.p[O.off(f.i, f.j, f.k) + c * O.ns] = F;
    if (B.uflux[d].p) {
        const Fab& U = B.uflux[d];
        const int64_t qu = U.off(f.i, f.j, f.k);
        U.p[qu + sc * U.ns] = F;
        if (c == 0)
            for (int z = NCONS; z < NFLO; ++z) U.p[qu + z * U.ns] = 0.0;
    }
}

// Per-face form (for launches too small to fill the GPU with column
// segments): one thread per (face, component) builds the four cells itself.
__device__ __forceinline__ void flux5_face_body(const RhsBox& B, int d, int c, int64_t t) {
    int len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    if (t >= (int64_t)len[0] * len[1] * len[2]) return;
    const Idx3 f = delinear(t, B.lo, len);
    const Fab& S = B.sb;
    const Fab& X = B.aux;
    const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
    const int64_t oR = S.off(f.i, f.j, f.k), xR = X.off(f.i, f.j, f.k);
    const double* vfp = S.p + VFRAC * S.ns;
    const Fab& FS = B.fs[d];
    if (c >= NCONS && c_P.advect_flag[c - NCONS] == 0.0) {  // not advected: diffusion only
        const WenoWindow w0 = {};
        const double F = flux5_face(B, d, c, FS, FS.off(f.i, f.j, f.k), w0, S.p[oR - sd + sc * S.ns],
                                    S.p[oR + sc * S.ns], 0.0, 0.0, vfp[oR - sd], vfp[oR], false);
        flux5_store(B, d, c, sc, f, F);
        return;
    }
    double ru[6], rf[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) sweep_raw(B, d, c, sc, oR + (q - 3) * sd, xR + (q - 3) * xd, ru[q], rf[q]);
    WenoWindow w;
    w.u0 = weno_cell(ru[0], ru[1], ru[2]);
    w.u1 = weno_cell(ru[1], ru[2], ru[3]);
    w.u2 = weno_cell(ru[2], ru[3], ru[4]);
    w.u3 = weno_cell(ru[3], ru[4], ru[5]);
    w.f0 = weno_cell(rf[0], rf[1], rf[2]);
    w.f1 = weno_cell(rf[1], rf[2], rf[3]);
    w.f2 = weno_cell(rf[2], rf[3], rf[4]);
    w.f3 = weno_cell(rf[3], rf[4], rf[5]);
    const double F = flux5_face(B, d, c, FS, FS.off(f.i, f.j, f.k), w, ru[2], ru[3], rf[2], rf[3], vfp[oR - sd],
                                vfp[oR]);
    flux5_store(B, d, c, sc, f, F);
}

__device__ __forceinline__ void flux5_sweep_body(const RhsBox& B, int d, int c, int64_t t, int seglen = SWEEP_SEG) {
    if (t >= sweep_items(B, d, seglen)) return;
    int ta, tb;
    sweep_dirs(d, ta, tb);
    const int na = B.hi[ta] - B.lo[ta] + 1, nb = B.hi[tb] - B.lo[tb] + 1;
    const int64_t ncol = (int64_t)na * nb;
    const int seg = (int)(t / ncol);
    const int64_t col = t - (int64_t)seg * ncol;
    const int nf = B.hi[d] - B.lo[d] + 2;
    const int nseg = sweep_nseg(B, d, seglen);
    const int per = (nf + nseg - 1) / nseg;
    const int f0 = B.lo[d] + seg * per;
    const int f1 = min(B.lo[d] + nf - 1, f0 + per - 1);
    if (f0 > f1) return;
    int iv[3];
    iv[ta] = B.lo[ta] + (int)(col % na);
    iv[tb] = B.lo[tb] + (int)(col / na);
    iv[d] = f0;
    const Fab& S = B.sb;
    const Fab& X = B.aux;
    const Fab& FS = B.fs[d];
    const int sc = (c < NCONS) ? c : c + (NFLO - NCONS);
    const int64_t sd = (d == 0) ? 1 : (d == 1) ? S.js : S.ks;
    const int64_t xd = (d == 0) ? 1 : (d == 1) ? X.js : X.ks;
    const int64_t fd = (d == 0) ? 1 : (d == 1) ? FS.js : FS.ks;
    int64_t oR = S.off(iv[0], iv[1], iv[2]);  // right cell of the current face
    int64_t xR = X.off(iv[0], iv[1], iv[2]);
    int64_t qf = FS.off(iv[0], iv[1], iv[2]);
    const double* vfp = S.p + VFRAC * S.ns;
    if (c >= NCONS && c_P.advect_flag[c - NCONS] == 0.0) {  // not advected: diffusion only
        const WenoWindow w0 = {};
        for (int f = f0; f <= f1; ++f, oR += sd, qf += fd, ++iv[d]) {
            const double F = flux5_face(B, d, c, FS, qf, w0, S.p[oR - sd + sc * S.ns], S.p[oR + sc * S.ns], 0.0, 0.0,
                                        vfp[oR - sd], vfp[oR], false);
            Idx3 fi;
            fi.i = iv[0];
            fi.j = iv[1];
            fi.k = iv[2];
            flux5_store(B, d, c, sc, fi, F);
        }
        return;
    }
    // raw values of cells f-3 .. f+2; the per-cell WENO parts of the four
    // stencil centres f-2 .. f+1 are built only when a face needs them: faces
    // on the solid side of the immersed boundary (no hyperbolic flux) and
    // first-order fallback faces use the raw values alone, so columns through
    // solid regions skip the reconstruction's per-cell work (bitwise the same
    // numbers: each centre is the same weno_cell of the same three values)
    double ru[6], rf[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) sweep_raw(B, d, c, sc, oR + (q - 3) * sd, xR + (q - 3) * xd, ru[q], rf[q]);
    WenoWindow w;
    unsigned have = 0;  // bit q: centre f-2+q built
    for (int f = f0;; ++f) {
        const int flags = (int)__double_as_longlong(FS.p[qf + FS_FLAGS * FS.ns]);
        if ((flags & 3) == 1) {
            if (!(have & 1u)) {
                w.u0 = weno_cell(ru[0], ru[1], ru[2]);
                w.f0 = weno_cell(rf[0], rf[1], rf[2]);
            }
            if (!(have & 2u)) {
                w.u1 = weno_cell(ru[1], ru[2], ru[3]);
                w.f1 = weno_cell(rf[1], rf[2], rf[3]);
            }
            if (!(have & 4u)) {
                w.u2 = weno_cell(ru[2], ru[3], ru[4]);
                w.f2 = weno_cell(rf[2], rf[3], rf[4]);
            }
            if (!(have & 8u)) {
                w.u3 = weno_cell(ru[3], ru[4], ru[5]);
                w.f3 = weno_cell(rf[3], rf[4], rf[5]);
            }
            have = 15u;
        }
        const double F = flux5_face(B, d, c, FS, qf, w, ru[2], ru[3], rf[2], rf[3], vfp[oR - sd], vfp[oR]);
        Idx3 fi;
        fi.i = iv[0];
        fi.j = iv[1];
        fi.k = iv[2];
        flux5_store(B, d, c, sc, fi, F);
        if (f == f1) break;
        // advance one face: load cell f+3, shift the window
        ++iv[d];
        oR += sd;
        xR += xd;
        qf += fd;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            ru[q] = ru[q + 1];
            rf[q] = rf[q + 1];
        }
        sweep_raw(B, d, c, sc, oR + 2 * sd, xR + 2 * xd, ru[5], rf[5]);
        w.u0 = w.u1;
        w.u1 = w.u2;
        w.u2 = w.u3;
        w.f0 = w.f1;
        w.f1 = w.f2;
        w.f2 = w.f3;
        have = (have >> 1) & 7u;
    }
}

// Work items of each phase for one box.
__host__ __device__ __forceinline__ int64_t prim_items(const RhsBox& B) {
    return (int64_t)(B.hi[0] - B.lo[0] + 7) * (B.hi[1] - B.lo[1] + 7) * (B.hi[2] - B.lo[2] + 7);
}
__host__ __device__ __forceinline__ int64_t face_items(const RhsBox& B, int d) {
    return (int64_t)(B.hi[0] - B.lo[0] + 1 + (d == 0)) * (B.hi[1] - B.lo[1] + 1 + (d == 1)) *
           (B.hi[2] - B.lo[2] + 1 + (d == 2));
}
__host__ __device__ __forceinline__ int64_t cell_items(const RhsBox& B) {
    return (int64_t)(B.hi[0] - B.lo[0] + 1) * (B.hi[1] - B.lo[1] + 1) * (B.hi[2] - B.lo[2] + 1);
}

}  // namespace
}  // namespace mfg
