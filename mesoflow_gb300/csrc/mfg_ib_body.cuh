// Per-cut-cell body of the immersed-boundary ghost treatment (update_cutcells,
// Source/Src_3d/ib_utils.H:272-436), shared by the per-box launches
// (mfg_ib.cu) and the batched launches over all boxes (mfg_batch.cu).
//
// Two forms of the same arithmetic: cutcell_one computes the inverse-distance
// weights of the 5^3 neighbourhood on the fly; cut_entries_one stores, for
// each fluid neighbour in neighbourhood order, its offset and both weights
// (plus 1/den and 1/sum w per cut cell) and cutcell_cached applies them.
// Both accumulate in the same neighbour order and finish with the same
// multiplications, so they give bitwise equal results.
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {

// Dirichlet IDW weights by neighbour offset (defined in mfg_ib.cu)
extern __constant__ double c_wdir[125];

namespace {

constexpr int SG = 2;  // STENCILGROW
constexpr int SW = 2 * SG + 1;
constexpr int CUT_BATCH = 4;  // neighbour entries whose gathers are issued together


struct CutBox {
    int lo[3], len[3];
    int64_t n;
    Fab S;
    double dx[3];
    double dxmin;
    double* tcht;  // conjugate-heat-transfer temperature average per valid cell (or null)
};

// Stored entries of the cut cells of one box.  Cut cells sit in the list in
// decreasing order of their fluid-neighbour count, so the 32 cells of a warp
// loop about as often; entry e of list position w lives at
// base[w / 32] + 32 e + w % 32, so a warp's loads of entry e are contiguous.
struct CutCacheView {
    const int* list;       // cell index by list position
    const int* kc;         // fluid neighbours by list position
    const int64_t* base;   // first entry of each group of 32 list positions
    const int* off;        // offset of the neighbour from the cell in Sborder
    const double* wn;      // inverse-distance weight about the surface point
    const double* wd;      // Dirichlet velocity weight
    const double* scal;    // 2 per list position: 1/den (0: zero velocity), 1/sum wn
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

// Number of vfrac == 1 cells in the 5^3 neighbourhood of cut cell t.
__device__ __forceinline__ int cut_count_one(const CutBox& c, int64_t t) {
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const double* V = S.p + VFRAC * S.ns;
    int cnt = 0;
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) cnt += is_one(V[o + l + m * S.js + n * S.ks]) ? 1 : 0;
    return cnt;
}

// Stores the entries of the cut cell at list position w (cell cc.list[w]).
__device__ __forceinline__ void cut_entries_one(const CutBox& c, int w, const CutCacheView& cc, int* offp,
                                                double* wnp, double* wdp, double* scal) {
    int i, j, k;
    cell_of(c, cc.list[w], i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const double* V = S.p + VFRAC * S.ns;
    double dist, xpn[3], dxnd[3];
    cut_geometry(c, o, dist, xpn, dxnd);
    double swd = 0.0, swn = 0.0;
    int64_t ix = cc.base[w >> 5] + (w & 31);
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const int64_t q = l + m * S.js + n * S.ks;
                if (!is_one(V[o + q])) continue;
                const int slot = (l + SG) + SW * ((m + SG) + SW * (n + SG));
                const bool centre = l == 0 && m == 0 && n == 0;
                if (!centre) swd += c_wdir[slot];
                const double a = l * dxnd[0] - xpn[0], b = m * dxnd[1] - xpn[1], e = n * dxnd[2] - xpn[2];
                const double wn = rcp_pos(((a * a + b * b) + e * e) + kTiny2);
                offp[ix] = (int)q;
                wnp[ix] = wn;
                wdp[ix] = centre ? 0.0 : c_wdir[slot];
                ix += 32;
                swn += wn;
            }
    scal[2 * (int64_t)w] = vel_iden(c, dist, swd);
    scal[2 * (int64_t)w + 1] = swn > 0.0 ? 1.0 / swn : 0.0;
}

// Cached form: the stored entries applied in the on-the-fly order.  A cut
// cell is never its own fluid neighbour (its vfrac is below one), so every
// entry carries a velocity weight, as in the on-the-fly loop.
template <int NS>
__device__ __forceinline__ void cutcell_cached(const CutBox& c, int w, const CutCacheView& cc) {
    const int64_t t = cc.list[w];
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const DevParams& P = c_P;
    const bool interp_spec = !P.species_in_solid;
    double sv[3] = {0.0, 0.0, 0.0};
    double sp = 0.0, st = 0.0, sr = 0.0, ss[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) ss[s] = 0.0;
    const int kn = cc.kc[w];
    int64_t ix = cc.base[w >> 5] + (w & 31);
    // batches of CUT_BATCH entries: all gathers of a batch are issued before
    // its sums, which then run in neighbour order
    int e = 0;
    for (; e + CUT_BATCH <= kn; e += CUT_BATCH, ix += 32 * CUT_BATCH) {
        int64_t q[CUT_BATCH];
        double wd[CUT_BATCH], wn[CUT_BATCH], v[CUT_BATCH][6];
#pragma unroll
        for (int u = 0; u < CUT_BATCH; ++u) {
            q[u] = o + cc.off[ix + 32 * u];
            wd[u] = cc.wd[ix + 32 * u];
            wn[u] = cc.wn[ix + 32 * u];
        }
#pragma unroll
        for (int u = 0; u < CUT_BATCH; ++u) {
            v[u][0] = S.p[q[u] + VELX * S.ns];
            v[u][1] = S.p[q[u] + VELY * S.ns];
            v[u][2] = S.p[q[u] + VELZ * S.ns];
            v[u][3] = S.p[q[u] + PRES * S.ns];
            v[u][4] = S.p[q[u] + TEMP * S.ns];
            v[u][5] = S.p[q[u] + DENS * S.ns];
        }
#pragma unroll
        for (int u = 0; u < CUT_BATCH; ++u) {
            sv[0] += v[u][0] * wd[u];
            sv[1] += v[u][1] * wd[u];
            sv[2] += v[u][2] * wd[u];
            sp += v[u][3] * wn[u];
            st += v[u][4] * wn[u];
            sr += v[u][5] * wn[u];
            if (interp_spec) {
#pragma unroll
                for (int s = 0; s < NS; ++s)
                    if (s < P.nspec) ss[s] += S.p[q[u] + (NFLO + s) * S.ns] * wn[u];
            }
        }
    }
    for (; e < kn; ++e, ix += 32) {
        const int64_t q = o + cc.off[ix];
        const double wd = cc.wd[ix], wn = cc.wn[ix];
        sv[0] += S.p[q + VELX * S.ns] * wd;
        sv[1] += S.p[q + VELY * S.ns] * wd;
        sv[2] += S.p[q + VELZ * S.ns] * wd;
        sp += S.p[q + PRES * S.ns] * wn;
        st += S.p[q + TEMP * S.ns] * wn;
        sr += S.p[q + DENS * S.ns] * wn;
        if (interp_spec) {
#pragma unroll
            for (int s = 0; s < NS; ++s)
                if (s < P.nspec) ss[s] += S.p[q + (NFLO + s) * S.ns] * wn;
        }
    }
    cut_finish<NS>(c, t, o, cc.scal[2 * (int64_t)w], kn > 0, cc.scal[2 * (int64_t)w + 1], sv, sp, st, sr, ss);
}

}  // namespace
}  // namespace mfg
