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

#include "mfg_ib_body.cuh"

namespace mfg {

__constant__ double c_wdir[125];

namespace {

constexpr int TPB = 128;

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
__global__ void __launch_bounds__(TPB) cutcell_kernel(CutBox c, const int* __restrict__ list,
                                                      const unsigned* __restrict__ count) {
    const unsigned n = *count;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
        cutcell_one<NS>(c, list[w]);
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
    // the table depends on the cell aspect ratios only (dx / dxmin), the same on every level
    const double dnk[3] = {g.dx[0] / c.dxmin, g.dx[1] / c.dxmin, g.dx[2] / c.dxmin};
    if (dnk[0] != g_wdir_dx[0] || dnk[1] != g_wdir_dx[1] || dnk[2] != g_wdir_dx[2]) {
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
        for (int d = 0; d < 3; ++d) g_wdir_dx[d] = dnk[d];
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
