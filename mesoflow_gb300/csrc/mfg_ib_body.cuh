// Per-cut-cell body of the immersed-boundary ghost treatment (update_cutcells,
// Source/Src_3d/ib_utils.H:272-436), shared by the per-box launches
// (mfg_ib.cu) and the batched launches over all boxes (mfg_batch.cu).
//
// Two forms of the same arithmetic: cutcell_one computes the inverse-distance
// weights of the 5^3 neighbourhood on the fly; cut_weights_one stores them
// (fluid-neighbour mask, 1/den, 1/sum w, the 125 weights) and cutcell_cached
// applies stored weights.  Both accumulate in the same neighbour order and
// finish with the same multiplications, so they give bitwise equal results.
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {

// Dirichlet IDW weights by neighbour offset (defined in mfg_ib.cu)
extern __constant__ double c_wdir[125];

namespace {

constexpr int SG = 2;  // STENCILGROW
constexpr int SW = 2 * SG + 1;
constexpr int CUT_SLOTS = 128;  // stored weights per cut cell (125 used)


struct CutBox {
    int lo[3], len[3];
    int64_t n;
    Fab S;
    double dx[3];
    double dxmin;
    double* tcht;  // conjugate-heat-transfer temperature average per valid cell (or null)
};

// Stored weights of the cut cells of one box (list position w).
struct CutCacheView {
    const unsigned long long* mask;  // 2 per cut cell: fluid-neighbour bits by slot
    const double* scal;              // 2 per cut cell: 1/den of the velocity weights (0: zero velocity), 1/sum w
    const double* wn;                // CUT_SLOTS per cut cell: IDW weight by slot
};

__device__ __forceinline__ void cell_of(const CutBox& c, int64_t t, int& i, int& j, int& k) {
    split3(t, c.len[0], c.len[1], i, j, k);
    i += c.lo[0];
    j += c.lo[1];
    k += c.lo[2];
}

// Level-set normal from the central differences of vfrac, the distance to the
// vfrac = 1/2 surface and the surface point in units of dxmin.
__device__ __forceinline__ void cut_geometry(const CutBox& c, int64_t o, double& dist, double xpn[3], double dxnd[3]) {
    const Fab& S = c.S;
    const double* V = S.p + VFRAC * S.ns;
    const double vf = V[o];
    const double hx = 0.5 / c.dx[0], hy = 0.5 / c.dx[1], hz = 0.5 / c.dx[2];
    const double gx = add(mul(V[o - 1], -hx), mul(V[o + 1], hx));
    const double gy = add(mul(V[o - S.js], -hy), mul(V[o + S.js], hy));
    const double gz = add(mul(V[o - S.ks], -hz), mul(V[o + S.ks], hz));
    const double mag = sqrt((gx * gx + gy * gy) + gz * gz);
    double xp[3] = {0.0, 0.0, 0.0};
    dist = 0.0;
    if (mag > kTiny) {
        dist = (vf - 0.5) / mag;
        xp[0] = -dist * (gx / mag);
        xp[1] = -dist * (gy / mag);
        xp[2] = -dist * (gz / mag);
    }
    for (int d = 0; d < 3; ++d) {
        dxnd[d] = c.dx[d] / c.dxmin;
        xpn[d] = xp[d] / c.dxmin;
    }
}

// 1/den of the velocity weights: den = sum wd + 1/dn^2 (the surface point),
// zero when the cell centre lies on the surface (velocity set to zero).
__device__ __forceinline__ double vel_iden(const CutBox& c, double dist, double swd) {
    if (fabs(dist) < c.dxmin * 1e-5) return 0.0;
    const double dn = fabs(dist) / c.dxmin;
    return 1.0 / (swd + 1.0 / (dn * dn));
}

// Writes the primitives and conserved variables of cut cell (o, t) from the
// weighted sums (prim_to_cons, consprim_funcs.H:26-44).
template <int NS>
__device__ __forceinline__ void cut_finish(const CutBox& c, int64_t t, int64_t o, double iden, bool have, double iswn,
                                           const double sv[3], double sp, double st, double sr, const double* ss) {
    const Fab& S = c.S;
    const DevParams& P = c_P;
    const bool interp_spec = !P.species_in_solid;
    double vel[3];
    // the surface value is zero: its term adds 0/(dn*dn) to each sum
    for (int a = 0; a < 3; ++a) vel[a] = (iden == 0.0) ? 0.0 : (sv[a] + 0.0) * iden;
    const double pres = have ? sp * iswn : S.p[o + PRES * S.ns];
    double temp;
    if (P.conj_ht)
        temp = c.tcht[t];
    else
        temp = have ? st * iswn : S.p[o + TEMP * S.ns];
    const double dens = have ? sr * iswn : S.p[o + DENS * S.ns];
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= P.nspec) {
            spec[s] = 0.0;
            continue;
        }
        spec[s] = (interp_spec && have) ? ss[s] * iswn : S.p[o + (NFLO + s) * S.ns];
    }
    S.p[o + VELX * S.ns] = vel[0];
    S.p[o + VELY * S.ns] = vel[1];
    S.p[o + VELZ * S.ns] = vel[2];
    S.p[o + PRES * S.ns] = pres;
    S.p[o + TEMP * S.ns] = temp;
    S.p[o + DENS * S.ns] = dens;
    if (interp_spec) {
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.nspec) S.p[o + (NFLO + s) * S.ns] = spec[s];
    }
    const double e = thermo_e<NS>(dens, pres, spec);
    const double ke = add(add(mul(vel[0], vel[0]), mul(vel[1], vel[1])), mul(vel[2], vel[2]));
    S.p[o + RHO * S.ns] = dens;
    S.p[o + RHOU * S.ns] = mul(dens, vel[0]);
    S.p[o + RHOV * S.ns] = mul(dens, vel[1]);
    S.p[o + RHOW * S.ns] = mul(dens, vel[2]);
    S.p[o + RHOE * S.ns] = add(mul(dens, e), mul(mul(0.5, dens), ke));
}

// On-the-fly form: velocity by inverse-distance weighting with a zero
// Dirichlet value at the surface point; pressure, temperature, density and
// species by inverse-distance weighting about the surface point (zero normal
// gradient), over the vfrac == 1 cells of the 5^3 neighbourhood.
template <int NS>
__device__ __forceinline__ void cutcell_one(const CutBox& c, int64_t t) {
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const DevParams& P = c_P;
    const double* V = S.p + VFRAC * S.ns;
    double dist, xpn[3], dxnd[3];
    cut_geometry(c, o, dist, xpn, dxnd);
    double sv[3] = {0.0, 0.0, 0.0}, swd = 0.0;
    double sp = 0.0, st = 0.0, sr = 0.0, ss[NS], swn = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s) ss[s] = 0.0;
    const bool interp_spec = !P.species_in_solid;
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const int64_t q = o + l + m * S.js + n * S.ks;
                if (!is_one(V[q])) continue;
                const int w = (l + SG) + SW * ((m + SG) + SW * (n + SG));
                if (!(l == 0 && m == 0 && n == 0)) {
                    const double wd = c_wdir[w];
                    sv[0] += S.p[q + VELX * S.ns] * wd;
                    sv[1] += S.p[q + VELY * S.ns] * wd;
                    sv[2] += S.p[q + VELZ * S.ns] * wd;
                    swd += wd;
                }
                const double a = l * dxnd[0] - xpn[0], b = m * dxnd[1] - xpn[1], e = n * dxnd[2] - xpn[2];
                const double wn = rcp_pos(((a * a + b * b) + e * e) + kTiny2);
                sp += S.p[q + PRES * S.ns] * wn;
                st += S.p[q + TEMP * S.ns] * wn;
                sr += S.p[q + DENS * S.ns] * wn;
                if (interp_spec) {
#pragma unroll
                    for (int s = 0; s < NS; ++s)
                        if (s < P.nspec) ss[s] += S.p[q + (NFLO + s) * S.ns] * wn;
                }
                swn += wn;
            }
    const bool have = swn > 0.0;
    cut_finish<NS>(c, t, o, vel_iden(c, dist, swd), have, have ? 1.0 / swn : 0.0, sv, sp, st, sr, ss);
}

// Stores the weights of cut cell t of the box at list position w.
__device__ __forceinline__ void cut_weights_one(const CutBox& c, int64_t t, int w, unsigned long long* mask,
                                                double* scal, double* wnp) {
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const double* V = S.p + VFRAC * S.ns;
    double dist, xpn[3], dxnd[3];
    cut_geometry(c, o, dist, xpn, dxnd);
    unsigned long long m0 = 0, m1 = 0;
    double swd = 0.0, swn = 0.0;
    double* W = wnp + (int64_t)w * CUT_SLOTS;
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const int64_t q = o + l + m * S.js + n * S.ks;
                if (!is_one(V[q])) continue;
                const int slot = (l + SG) + SW * ((m + SG) + SW * (n + SG));
                if (slot < 64)
                    m0 |= 1ull << slot;
                else
                    m1 |= 1ull << (slot - 64);
                if (!(l == 0 && m == 0 && n == 0)) swd += c_wdir[slot];
                const double a = l * dxnd[0] - xpn[0], b = m * dxnd[1] - xpn[1], e = n * dxnd[2] - xpn[2];
                const double wn = rcp_pos(((a * a + b * b) + e * e) + kTiny2);
                W[slot] = wn;
                swn += wn;
            }
    mask[2 * (int64_t)w] = m0;
    mask[2 * (int64_t)w + 1] = m1;
    scal[2 * (int64_t)w] = vel_iden(c, dist, swd);
    scal[2 * (int64_t)w + 1] = swn > 0.0 ? 1.0 / swn : 0.0;
}

// Cached form: the stored weights applied in the on-the-fly order.
template <int NS>
__device__ __forceinline__ void cutcell_cached(const CutBox& c, int64_t t, int w, const CutCacheView& cc) {
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const DevParams& P = c_P;
    const bool interp_spec = !P.species_in_solid;
    const double* W = cc.wn + (int64_t)w * CUT_SLOTS;
    double sv[3] = {0.0, 0.0, 0.0};
    double sp = 0.0, st = 0.0, sr = 0.0, ss[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) ss[s] = 0.0;
    const unsigned long long mk[2] = {cc.mask[2 * (int64_t)w], cc.mask[2 * (int64_t)w + 1]};
    for (int h = 0; h < 2; ++h) {
        unsigned long long bits = mk[h];
        while (bits) {
            const int slot = h * 64 + __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const int l = slot % SW - SG, m = (slot / SW) % SW - SG, n = slot / (SW * SW) - SG;
            const int64_t q = o + l + m * S.js + n * S.ks;
            if (slot != (SW * SW * SW) / 2) {
                const double wd = c_wdir[slot];
                sv[0] += S.p[q + VELX * S.ns] * wd;
                sv[1] += S.p[q + VELY * S.ns] * wd;
                sv[2] += S.p[q + VELZ * S.ns] * wd;
            }
            const double wn = W[slot];
            sp += S.p[q + PRES * S.ns] * wn;
            st += S.p[q + TEMP * S.ns] * wn;
            sr += S.p[q + DENS * S.ns] * wn;
            if (interp_spec) {
#pragma unroll
                for (int s = 0; s < NS; ++s)
                    if (s < P.nspec) ss[s] += S.p[q + (NFLO + s) * S.ns] * wn;
            }
        }
    }
    const bool have = (mk[0] | mk[1]) != 0;
    cut_finish<NS>(c, t, o, cc.scal[2 * (int64_t)w], have, cc.scal[2 * (int64_t)w + 1], sv, sp, st, sr, ss);
}

}  // namespace
}  // namespace mfg
