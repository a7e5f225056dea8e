// Immersed-boundary cut-cell ghost treatment (update_cutcells,
// Source/Src_3d/ib_utils.H:272-436), in place on Sborder's valid cells.
//
// For a cell with 0 < vfrac < 1: the level-set normal from the central
// differences of vfrac (the quadratic basis of ib_utils.H:14-96 evaluated at
// the cell centre reduces to them), the distance to the vfrac = 1/2 surface,
// velocity by inverse-distance weighting with a zero Dirichlet value at the
// surface point, and pressure, temperature, density and species by
// inverse-distance weighting about the surface point (zero normal gradient),
// all over the vfrac == 1 cells of the 5^3 neighbourhood; the conserved
// variables are then re-derived from the primitives.
//
// Work layout: a compaction pass lists the box's cut cells (one atomic per
// warp), then a fixed grid of threads walks the list, one cut cell per thread,
// so no lane idles on pure fluid or solid cells.  Each neighbour's weight
// 1/(d^2 + 1e-40) is computed once (Newton-refined reciprocal) and shared by
// all interpolated components (the reference divides per component); the
// Dirichlet weights depend only on the grid and come from a constant table.
#include <algorithm>

#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {
namespace {

constexpr int TPB = 128;
constexpr int SG = 2;  // STENCILGROW
constexpr int SW = 2 * SG + 1;

__constant__ double c_wdir[SW * SW * SW];  // Dirichlet IDW weights by offset

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

// Conjugate heat transfer: mean temperature of the 26 neighbours, read before
// any cut cell is updated (ib_utils.H:345-364).
__global__ void cht_avg_kernel(CutBox c) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.n) return;
    int i, j, k;
    cell_of(c, t, i, j, k);
    const double vf = c.S(i, j, k, VFRAC);
    if (!(vf > 0.0 && vf < 1.0)) return;
    double sum = 0.0;
    for (int n = -1; n <= 1; ++n)
        for (int m = -1; m <= 1; ++m)
            for (int l = -1; l <= 1; ++l)
                if (!(l == 0 && m == 0 && n == 0)) sum += c.S(i + l, j + m, k + n, TEMP);
    c.tcht[t] = sum / 26.0;
}

// Appends the linear index of every cut cell (0 < vfrac < 1) of the box to list.
__global__ void cut_list_kernel(CutBox c, int* __restrict__ list, unsigned* __restrict__ count) {
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
__device__ void cutcell_one(const CutBox& c, int64_t t);

template <int NS>
__global__ void __launch_bounds__(TPB) cutcell_kernel(CutBox c, const int* __restrict__ list,
                                                      const unsigned* __restrict__ count) {
    const unsigned n = *count;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
        cutcell_one<NS>(c, list[w]);
}

template <int NS>
__device__ void cutcell_one(const CutBox& c, int64_t t) {
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

double g_wdir_dx[3] = {-1.0, -1.0, -1.0};

}  // namespace

cudaError_t launch_cutcells_box(const mfg_box& b, const mfg_geom& g, double* tcht_scratch, int* list,
                                unsigned* count, cudaStream_t st) {
    CutBox c;
    c.n = 1;
    for (int d = 0; d < 3; ++d) {
        c.lo[d] = b.lo[d];
        c.len[d] = b.hi[d] - b.lo[d] + 1;
        c.n *= c.len[d];
        c.dx[d] = g.dx[d];
    }
    c.S = make_fab(b.sborder);
    c.dxmin = fmin(g.dx[0], fmin(g.dx[1], g.dx[2]));
    c.tcht = tcht_scratch;
    if (g.dx[0] != g_wdir_dx[0] || g.dx[1] != g_wdir_dx[1] || g.dx[2] != g_wdir_dx[2]) {
        // Dirichlet weights: 1/((l dx_nd)^2 + (m dy_nd)^2 + (n dz_nd)^2 + 1e-40), centre unused
        double w[SW * SW * SW];
        const double dn[3] = {g.dx[0] / c.dxmin, g.dx[1] / c.dxmin, g.dx[2] / c.dxmin};
        for (int n = -SG; n <= SG; ++n)
            for (int m = -SG; m <= SG; ++m)
                for (int l = -SG; l <= SG; ++l) {
                    const double a = l * dn[0], bb = m * dn[1], e = n * dn[2];
                    const double d2 = (a * a + bb * bb) + e * e;
                    w[(l + SG) + SW * ((m + SG) + SW * (n + SG))] = (l == 0 && m == 0 && n == 0) ? 0.0 : 1.0 / (d2 + kTiny2);
                }
        cudaError_t e = cudaMemcpyToSymbolAsync(c_wdir, w, sizeof(w), 0, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
        cudaStreamSynchronize(st);
        for (int d = 0; d < 3; ++d) g_wdir_dx[d] = g.dx[d];
    }
    const unsigned nb = (unsigned)((c.n + TPB - 1) / TPB);
    ProfScope ps(K_CUT, st);
    if (c_host_params().conj_ht) cht_avg_kernel<<<nb, TPB, 0, st>>>(c);
    cudaMemsetAsync(count, 0, sizeof(unsigned), st);
    cut_list_kernel<<<nb, TPB, 0, st>>>(c, list, count);
    // a fixed grid walks the list (its length stays on the device)
    const unsigned ng = (unsigned)std::min<int64_t>(nb, 152 * 8);
    const int ns = c_host_params().nspec;
    if (ns <= 1) cutcell_kernel<1><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 2) cutcell_kernel<2><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 4) cutcell_kernel<4><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 8) cutcell_kernel<8><<<ng, TPB, 0, st>>>(c, list, count);
    else cutcell_kernel<16><<<ng, TPB, 0, st>>>(c, list, count);
    return cudaGetLastError();
}

}  // namespace mfg
