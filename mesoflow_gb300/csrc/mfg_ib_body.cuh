// Per-cut-cell body of the immersed-boundary ghost treatment (update_cutcells,
// Source/Src_3d/ib_utils.H:272-436), shared by the per-box launches
// (mfg_ib.cu) and the batched launches over all boxes (mfg_batch.cu).
#pragma once
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {

// Dirichlet IDW weights by neighbour offset (defined in mfg_ib.cu)
extern __constant__ double c_wdir[125];

namespace {

constexpr int SG = 2;  // STENCILGROW
constexpr int SW = 2 * SG + 1;


struct CutBox {
    int lo[3], len[3];
    int64_t n;
    Fab S;
    double dx[3];
    double dxmin;
    double* tcht;  // conjugate-heat-transfer temperature average per valid cell (or null)
};

__device__ __forceinline__ void cell_of(const CutBox& c, int64_t t, int& i, int& j, int& k) {
    int64_t a = t / c.len[0];
    i = c.lo[0] + (int)(t - a * c.len[0]);
    k = c.lo[2] + (int)(a / c.len[1]);
    j = c.lo[1] + (int)(a - (int64_t)(k - c.lo[2]) * c.len[1]);
}

template <int NS>
__device__ __forceinline__ void cutcell_one(const CutBox& c, int64_t t) {
    int i, j, k;
    cell_of(c, t, i, j, k);
    const Fab& S = c.S;
    const int64_t o = S.off(i, j, k);
    const double vf = S.p[o + VFRAC * S.ns];
    const DevParams& P = c_P;
    const double* V = S.p + VFRAC * S.ns;

    // level-set gradient
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

    // Dirichlet (velocity, zero at the surface point) and hom-Neumann sums
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
    double vel[3];
    if (fabs(dist) < c.dxmin * 1e-5) {
        vel[0] = vel[1] = vel[2] = 0.0;
    } else {
        const double dn = fabs(dist) / c.dxmin;
        const double wsurf = 1.0 / (dn * dn);
        const double den = swd + wsurf;
        // the surface value is zero: its term adds 0/(dn*dn) to each sum
        vel[0] = (sv[0] + 0.0) / den;
        vel[1] = (sv[1] + 0.0) / den;
        vel[2] = (sv[2] + 0.0) / den;
    }
    const bool have = swn > 0.0;
    const double pres = have ? sp / swn : S.p[o + PRES * S.ns];
    double temp;
    if (P.conj_ht)
        temp = c.tcht[t];
    else
        temp = have ? st / swn : S.p[o + TEMP * S.ns];
    const double dens = have ? sr / swn : S.p[o + DENS * S.ns];
    double spec[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= P.nspec) {
            spec[s] = 0.0;
            continue;
        }
        spec[s] = (interp_spec && have) ? ss[s] / swn : S.p[o + (NFLO + s) * S.ns];
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
    // prim_to_cons (consprim_funcs.H:26-44)
    const double e = thermo_e<NS>(dens, pres, spec);
    const double ke = add(add(mul(vel[0], vel[0]), mul(vel[1], vel[1])), mul(vel[2], vel[2]));
    S.p[o + RHO * S.ns] = dens;
    S.p[o + RHOU * S.ns] = mul(dens, vel[0]);
    S.p[o + RHOV * S.ns] = mul(dens, vel[1]);
    S.p[o + RHOW * S.ns] = mul(dens, vel[2]);
    S.p[o + RHOE * S.ns] = add(mul(dens, e), mul(mul(0.5, dens), ke));
}


}  // namespace
}  // namespace mfg
