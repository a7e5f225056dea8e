// Batched AMR form: every box of every level advanced together.
//
// The box list (all levels, uneven box sizes) is uploaded once into device
// tables.  Each phase of a step (ghost fill, cut-cell list, cut cells,
// per-cell primitives, face scalars, face fluxes, update, chemistry, primitive
// refresh, clipping) is one launch over a tile list spanning all boxes: a
// tile is a contiguous run of work items (cells, faces or (face, component)
// pairs) of one box, and a fixed grid of blocks walks the tiles
// (persistent-style), so small boxes no longer leave most SMs idle.  Tile size
// and grid size per phase come from a measured search (mfg_boxlist_autotune).
// The whole step -- copy to phi_old, three stages of fill + cut cells + RHS +
// stage algebra, chemistry sub-step, primitive refresh, clipping -- can be
// captured into one CUDA graph and replayed.
//
// Levels advance with one common dt (no subcycling).  Ghost cells of level L
// are filled from level L boxes (periodic images included), then from the
// coarser level by piecewise-constant injection where level L has no data,
// then by the physical boundary rules.  The same kernels serve the plain mode,
// which launches per box (RHS, cut cells, bookends) and per level (fill).
#include <algorithm>
#include <array>
#include <cmath>
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

constexpr int BT = 256;

struct Tile {
    int box;
    int part;  // direction, component, or direction*32 + component
    long long start, end;
};

struct MBox {
    int lo[3], hi[3];
    int level;
    Fab sb, sold, snew;
    Fab cp;               // level > 0: coarse patch (coarse data around the grown box, for interpolation)
    int cplo[3], cphi[3];
};

// Coarse data at one fill time: 0 old, 1 new, 2 a*old + b*new.
struct TCoef {
    int kind;
    double a, b;
};

// One flux-register cell of a coarse-fine interface: the coarse face between
// coarse cell cc (owned by coarse box cb, outside fine box fb) and the fine
// box's side `side` of direction d; cf is that face in cb's face indexing,
// ff the first of the ratio^2 fine faces in fb's.
struct RegEnt {
    int fb, cb, d, side;
    int cc[3], cf[3], ff[3];
};

struct LevelG {
    int dlo[3], dhi[3], per[3];
    int gran, mlen[3];
    long long owner_off;  // offset of this level's owner map in the concatenated map
    int ratio;            // refinement ratio to the coarser level
    double dx[3];
};

// Device-resident state of mfg_boxlist_evolve's loop.
constexpr int RUN_MAXLEV = 16;
struct RunState {
    double t, dt_prev, dt;
    double final_time, stop_time, cfl;
    int istep, max_step, nlev;
    double acc[2 * RUN_MAXLEV];  // per level: max wave speed, max species diffusivity
    // subcycled loop: per-level dt of this step and of the previous one
    double dtl[RUN_MAXLEV], dtl_prev[RUN_MAXLEV];
};

enum Phase { PH_GROWN = 0, PH_VALID, PH_FACE, PH_FLUX, PH_UPDATE, PH_COUNT };
// per-level phases of the multi-level step: coarse-patch cells, coarsened cells of fine boxes
enum { PH_CP = PH_COUNT, PH_AVG, PH_ALL };

struct PhaseTiles {
    Tile* d = nullptr;
    int n = 0;
    int grid = 0;
    int tile_items = 4096;
    int grid_cap = 0;  // 0: one block per tile
};

// ---- kernels -------------------------------------------------------------------
#define TILE_LOOP                                                       \
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {           \
        const Tile tl = tiles[ti];                                      \
        for (long long t = tl.start + threadIdx.x; t < tl.end; t += blockDim.x) {
#define TILE_END \
    }            \
    }

__device__ __forceinline__ void grown_of(const MBox& b, long long t, int& i, int& j, int& k) {
    const int l0 = b.hi[0] - b.lo[0] + 1 + 2 * MFG_NGROW, l1 = b.hi[1] - b.lo[1] + 1 + 2 * MFG_NGROW;
    split3(t, l0, l1, i, j, k);
    i += b.lo[0] - MFG_NGROW;
    j += b.lo[1] - MFG_NGROW;
    k += b.lo[2] - MFG_NGROW;
}

__device__ __forceinline__ int owner_at(const LevelG& G, const int* owner, const int w[3]) {
    const int m0 = (w[0] - G.dlo[0]) / G.gran, m1 = (w[1] - G.dlo[1]) / G.gran, m2 = (w[2] - G.dlo[2]) / G.gran;
    return owner[G.owner_off + m0 + (long long)G.mlen[0] * (m1 + (long long)G.mlen[1] * m2)];
}

__device__ __forceinline__ int floor_div(int a, int r) { return a >= 0 ? a / r : -((-a + r - 1) / r); }
__device__ __forceinline__ double dmin_(double a, double b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ double dmax_(double a, double b) { return (a < b) ? b : a; }  // std::max

// cell_cons_interp (AMReX CellConservativeLinear without cross-component
// limiting) from the coarse patch u of a box of level l (coarse level geometry
// Gc, ratio r), for coarse cell ic and component c: MC-limited central slopes,
// the one-sided 4-point slope at an ext_dir face of the coarse domain, and one
// factor alpha per coarse cell keeping every fine value within the 27 coarse
// neighbours' bounds; returns u0 and the three slopes times alpha.  A fine
// child f of ic then gets u0 + sum_d off_d slope_d.  Explicit roundings: the
// same operations in the same order as the CPU restatement.
__device__ double cc_slopes(const MBox& b, const LevelG& Gc, int r, const int ic[3], int c, double sa[3]) {
    const DevParams& P = c_P;
    const Fab& u = b.cp;
    const int64_t q0 = u.off(ic[0], ic[1], ic[2]) + (int64_t)c * u.ns;
    const int64_t st[3] = {1, u.js, u.ks};
    const double u0 = u.p[q0];
    double sl[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double um = u.p[q0 - st[d]], up = u.p[q0 + st[d]];
        double dc = __dmul_rn(0.5, __dsub_rn(up, um));
        if (!Gc.per[d] && ic[d] == Gc.dlo[d] && P.bc_lo[d] == MFG_BC_EXT_DIR) {
            if (ic[d] + 2 <= b.cphi[d])
                dc = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(-16. / 15., um), __dmul_rn(0.5, u0)),
                                         __dmul_rn(2. / 3., up)),
                               __dmul_rn(0.1, u.p[q0 + 2 * st[d]]));
            else
                dc = __dmul_rn(0.25, __dsub_rn(__dadd_rn(up, __dmul_rn(5., u0)), __dmul_rn(6., um)));
        }
        if (!Gc.per[d] && ic[d] == Gc.dhi[d] && P.bc_hi[d] == MFG_BC_EXT_DIR) {
            if (ic[d] - 2 >= b.cplo[d])
                dc = __dadd_rn(__dsub_rn(__dsub_rn(__dmul_rn(16. / 15., up), __dmul_rn(0.5, u0)),
                                         __dmul_rn(2. / 3., um)),
                               __dmul_rn(0.1, u.p[q0 - 2 * st[d]]));
            else
                dc = __dmul_rn(-0.25, __dsub_rn(__dadd_rn(um, __dmul_rn(5., u0)), __dmul_rn(6., up)));
        }
        const double df = __dmul_rn(2.0, __dsub_rn(up, u0));
        const double db = __dmul_rn(2.0, __dsub_rn(u0, um));
        double sx = (__dmul_rn(df, db) >= 0.0) ? dmin_(fabs(df), fabs(db)) : 0.0;
        sx = __dmul_rn(copysign(1.0, dc), dmin_(sx, fabs(dc)));
        sl[d] = sx;
    }
    double alpha = 1.0;
    if (sl[0] != 0.0 || sl[1] != 0.0 || sl[2] != 0.0) {
        // (|s| (r-1)) / (2r); for r a power of two the division is the exact
        // multiplication by 1/(2r)
        const double f = (double)(r - 1), g = (double)(2 * r);
        const bool pow2 = (r & (r - 1)) == 0;
        const double ig = 1.0 / g;
        double t[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double x = __dmul_rn(fabs(sl[d]), f);
            t[d] = pow2 ? __dmul_rn(x, ig) : __ddiv_rn(x, g);
        }
        const double dumax = __dadd_rn(__dadd_rn(t[0], t[1]), t[2]);
        double umax = u0, umin = u0;
        for (int kk = -1; kk <= 1; ++kk)
            for (int jj = -1; jj <= 1; ++jj)
#pragma unroll
                for (int ii = -1; ii <= 1; ++ii) {
                    const double x = u.p[q0 + ii + jj * u.js + kk * u.ks];
                    umin = dmin_(umin, x);
                    umax = dmax_(umax, x);
                }
        if (__dmul_rn(dumax, alpha) > __dsub_rn(umax, u0)) alpha = __ddiv_rn(__dsub_rn(umax, u0), dumax);
        if (__dmul_rn(dumax, alpha) > __dsub_rn(u0, umin)) alpha = __ddiv_rn(__dsub_rn(u0, umin), dumax);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) sa[d] = __dmul_rn(sl[d], alpha);
    return u0;
}

// One coarse cell of a fine box's coarsened grown box with at least one
// child to interpolate (a ghost cell of the box inside the periodically
// extended fine domain that no fine box covers); bit m of mask = child
// (m % r, (m / r) % r, m / r^2).  The hierarchy is fixed, so the list is
// built once.
struct IEnt {
    int box, i, j, k;
    unsigned long long mask;
};

// Ghost cells of the fine boxes that the fine level does not cover, by
// cell_cons_interp: one thread per (listed coarse cell, component) computes the
// slopes once and writes the masked children.
__global__ void __launch_bounds__(BT) bk_cp_interp(const IEnt* __restrict__ ent, int ne,
                                                   const MBox* __restrict__ boxes, const LevelG* __restrict__ lev) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int c = blockIdx.y;
    const IEnt E = ent[e];
    const MBox& b = boxes[E.box];
    const int r = lev[b.level].ratio;
    const int ic[3] = {E.i, E.j, E.k};
    double sa[3];
    const double u0 = cc_slopes(b, lev[b.level - 1], r, ic, c, sa);
    // child offsets ((m + 0.5) / r - 0.5, m = 0..r-1; the division is exact as
    // a multiplication for r a power of two)
    double offs[4];
    const bool pow2 = (r & (r - 1)) == 0;
    for (int m = 0; m < r && m < 4; ++m) {
        const double x = (double)m + 0.5;
        offs[m] = __dsub_rn(pow2 ? __dmul_rn(x, 1.0 / (double)r) : __ddiv_rn(x, (double)r), 0.5);
    }
    unsigned long long mask = E.mask;
    while (mask) {
        const int m = __ffsll((long long)mask) - 1;
        mask &= mask - 1;
        const int mi = m % r, mj = (m / r) % r, mk = m / (r * r);
        double v = __dadd_rn(u0, __dmul_rn(offs[mi], sa[0]));
        v = __dadd_rn(v, __dmul_rn(offs[mj], sa[1]));
        v = __dadd_rn(v, __dmul_rn(offs[mk], sa[2]));
        b.sb(ic[0] * r + mi, ic[1] * r + mj, ic[2] * r + mk, c) = v;
    }
}

// copy of valid data (own level, periodic images); where the own level has
// none, from the coarser level: left to bk_cp_interp (interp = 1, the
// multi-level step) or piecewise-constant injection (interp = 0)
__global__ void __launch_bounds__(BT) bk_fill_copy(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                   const int* __restrict__ owner, const Tile* __restrict__ tiles,
                                                   int ntiles, int src, int nc, int interp) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    int i, j, k;
    grown_of(b, t, i, j, k);
    const LevelG& G = lev[b.level];
    int w[3] = {i, j, k};
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
        const int len = G.dhi[d] - G.dlo[d] + 1;
        if (G.per[d]) {
            while (w[d] < G.dlo[d]) w[d] += len;
            while (w[d] > G.dhi[d]) w[d] -= len;
        } else if (w[d] < G.dlo[d] || w[d] > G.dhi[d]) {
            inside = false;
        }
    }
    if (!inside) continue;
    int ob = owner_at(G, owner, w);
    int cw[3] = {w[0], w[1], w[2]};
    if (ob < 0 && b.level > 0 && interp) continue;
    if (ob < 0 && b.level > 0) {
        const LevelG& Gc = lev[b.level - 1];
        for (int d = 0; d < 3; ++d) cw[d] = Gc.dlo[d] + (w[d] - G.dlo[d]) / G.ratio;
        ob = owner_at(Gc, owner, cw);
    }
    if (ob < 0) continue;
    const MBox& o = boxes[ob];
    const Fab& S = src ? o.snew : o.sold;
    copy_comps(b.sb.p + b.sb.off(i, j, k), b.sb.ns, S.p + S.off(cw[0], cw[1], cw[2]), S.ns, nc);
    TILE_END
}

// Physical boundary of one cell (i, j, k) of the array S outside the domain of
// G in `stage` non-periodic directions (faces 1, edges 2, corners 3), from S
// itself.
template <int NS>
__device__ __forceinline__ void bc_cell(const Fab& S, const LevelG& G, int i, int j, int k, int stage, int nc) {
    const int iv[3] = {i, j, k};
    bool out[3];
    int nout = 0;
    for (int d = 0; d < 3; ++d) {
        out[d] = !G.per[d] && (iv[d] < G.dlo[d] || iv[d] > G.dhi[d]);
        nout += out[d];
    }
    if (nout != stage) return;
    const DevParams& P = c_P;
    int dext = -1, dlast = -1;
    for (int d = 0; d < 3; ++d) {
        if (!out[d]) continue;
        dlast = d;
        const int kind = (iv[d] < G.dlo[d]) ? P.bc_lo[d] : P.bc_hi[d];
        if (kind == MFG_BC_EXT_DIR) dext = d;
    }
    const int ds = (dext >= 0) ? dext : dlast;
    const bool lo = iv[ds] < G.dlo[ds];
    const int kind = lo ? P.bc_lo[ds] : P.bc_hi[ds];
    int sv[3] = {i, j, k};
    const long long qd = S.off(i, j, k);
    if (dext >= 0) {
        sv[ds] = lo ? G.dlo[ds] : G.dhi[ds];
        const long long qs = S.off(sv[0], sv[1], sv[2]);
        double s_int[NFLO + MAXS], s_ext[NFLO + MAXS];
        for (int c = 0; c < nc; ++c) s_int[c] = S.p[qs + c * S.ns];
        external_state<NS>(lo ? P.ext_lo[ds] : P.ext_hi[ds], ds, s_int, s_ext, nc);
        for (int c = 0; c < nc; ++c) S.p[qd + c * S.ns] = s_ext[c];
    } else if (kind == MFG_BC_FOEXTRAP) {
        sv[ds] = lo ? G.dlo[ds] : G.dhi[ds];
        const long long qs = S.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < nc; ++c) S.p[qd + c * S.ns] = S.p[qs + c * S.ns];
    } else {
        sv[ds] = lo ? (2 * G.dlo[ds] - iv[ds] - 1) : (2 * G.dhi[ds] - iv[ds] + 1);
        const long long qs = S.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < nc; ++c) {
            const double x = S.p[qs + c * S.ns];
            S.p[qd + c * S.ns] = odd_at_wall(c) ? -x : x;
        }
    }
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_fill_bc(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                 const Tile* __restrict__ tiles, int ntiles, int stage, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    int i, j, k;
    grown_of(b, t, i, j, k);
    bc_cell<NS>(b.sb, lev[b.level], i, j, k, stage, nc);
    TILE_END
}

__device__ __forceinline__ void cp_of(const MBox& b, long long t, int& i, int& j, int& k) {
    split3(t, b.cphi[0] - b.cplo[0] + 1, b.cphi[1] - b.cplo[1] + 1, i, j, k);
    i += b.cplo[0];
    j += b.cplo[1];
    k += b.cplo[2];
}

// Coarse patch of a fine box from its coarser level at one fill time (the
// coarse half of FillPatchTwoLevels): cells inside the coarse domain (periodic
// images included) from the owning coarse box's old / new data or their
// linear combination; the rest by bk_cp_bc.
__global__ void __launch_bounds__(BT) bk_cp_fill(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                 const int* __restrict__ owner, const Tile* __restrict__ tiles,
                                                 int ntiles, const TCoef* __restrict__ coef, int ev, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    int i, j, k;
    cp_of(b, t, i, j, k);
    const LevelG& G = lev[b.level - 1];
    int w[3] = {i, j, k};
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
        const int len = G.dhi[d] - G.dlo[d] + 1;
        if (G.per[d]) {
            while (w[d] < G.dlo[d]) w[d] += len;
            while (w[d] > G.dhi[d]) w[d] -= len;
        } else if (w[d] < G.dlo[d] || w[d] > G.dhi[d]) {
            inside = false;
        }
    }
    if (!inside) continue;
    const int ob = owner_at(G, owner, w);
    if (ob < 0) continue;  // excluded by the nesting check at creation
    const MBox& o = boxes[ob];
    const TCoef cf = coef[ev];
    const long long q0 = o.sold.off(w[0], w[1], w[2]), q1 = o.snew.off(w[0], w[1], w[2]);
    const long long qd = b.cp.off(i, j, k);
    for (int c = 0; c < nc; ++c) {
        const double x0 = o.sold.p[q0 + c * o.sold.ns], x1 = o.snew.p[q1 + c * o.snew.ns];
        b.cp.p[qd + c * b.cp.ns] =
            cf.kind == 0 ? x0 : cf.kind == 1 ? x1 : __dadd_rn(__dmul_rn(cf.a, x0), __dmul_rn(cf.b, x1));
    }
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_cp_bc(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                               const Tile* __restrict__ tiles, int ntiles, int stage, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    int i, j, k;
    cp_of(b, t, i, j, k);
    bc_cell<NS>(b.cp, lev[b.level - 1], i, j, k, stage, nc);
    TILE_END
}

// Flux registers (AMReX FluxRegister).  One thread per (register cell, advected
// component c); registers are stored component-major, reg[c * ne + e].
// CrseInit(ADD): reg += F_coarse * scale_d
// With dtp (device dt of the level), scale_d = ((sgn dt) dA_d) w instead of s_d.
struct RegScale {
    double s[3];       // scales for a host dt
    double dA[3], w;   // face areas and stage weight, for a device dt
    double sgn;        // -1 CrseInit, +1 FineAdd
};
__device__ __forceinline__ double reg_scale(const RegScale& S, const double* dtp, int d) {
    return dtp ? __dmul_rn(__dmul_rn(S.sgn * (*dtp), S.dA[d]), S.w) : S.s[d];
}

__global__ void __launch_bounds__(BT) bk_reg_crse(const RegEnt* __restrict__ ent, int ne,
                                                  const RhsBox* __restrict__ rhs, double* __restrict__ reg,
                                                  RegScale S, const double* __restrict__ dtp) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int c = blockIdx.y;
    const RegEnt E = ent[e];
    const Fab& F = rhs[E.cb].flx[E.d];
    const double scale = reg_scale(S, dtp, E.d);
    double& r = reg[(size_t)c * ne + e];
    r = __dadd_rn(r, __dmul_rn(F.p[F.off(E.cf[0], E.cf[1], E.cf[2]) + c * F.ns], scale));
}

// FineAdd: reg += scale_d * F_fine over the ratio^2 fine faces, the higher
// transverse direction outer
__global__ void __launch_bounds__(BT) bk_reg_fine(const RegEnt* __restrict__ ent, int ne,
                                                  const RhsBox* __restrict__ rhs, double* __restrict__ reg,
                                                  RegScale S, const double* __restrict__ dtp, int ratio) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int c = blockIdx.y;
    const RegEnt E = ent[e];
    const Fab& F = rhs[E.fb].flx[E.d];
    const double scale = reg_scale(S, dtp, E.d);
    const int t1 = E.d == 0 ? 1 : 0, t2 = E.d == 2 ? 1 : 2;
    const int64_t st[3] = {1, F.js, F.ks};
    const int64_t q = F.off(E.ff[0], E.ff[1], E.ff[2]) + c * F.ns;
    double v = reg[(size_t)c * ne + e];
    for (int o2 = 0; o2 < ratio; ++o2)
        for (int o1 = 0; o1 < ratio; ++o1) v = __dadd_rn(v, __dmul_rn(scale, F.p[q + o1 * st[t1] + o2 * st[t2]]));
    reg[(size_t)c * ne + e] = v;
}

// Reflux of one orientation (entries e0..e1): the coarse cell outside the fine
// box gets -reg/vol (low side) or +reg/vol (high side), every state component
// (zero register for the non-advected ones).
__global__ void __launch_bounds__(BT) bk_reflux(const RegEnt* __restrict__ ent, int e0, int e1, int ne,
                                                const MBox* __restrict__ boxes, const double* __restrict__ reg,
                                                double vol) {
    const int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= e1) return;
    const int n = blockIdx.y;
    const RegEnt E = ent[e];
    int c = -1;
    if (n < NCONS) c = n;
    else if (n >= NFLO) c = n - (NFLO - NCONS);
    const double f = c >= 0 ? reg[(size_t)c * ne + e] : 0.0;
    double& x = boxes[E.cb].snew(E.cc[0], E.cc[1], E.cc[2], n);
    x = __dadd_rn(x, E.side ? __ddiv_rn(f, vol) : __ddiv_rn(-f, vol));
}

__device__ __forceinline__ void avg_of(const MBox& b, int r, long long t, int& i, int& j, int& k) {
    const int a0 = floor_div(b.lo[0], r), a1 = floor_div(b.lo[1], r), a2 = floor_div(b.lo[2], r);
    split3(t, floor_div(b.hi[0] + 1, r) - a0, floor_div(b.hi[1] + 1, r) - a1, i, j, k);
    i += a0;
    j += a1;
    k += a2;
}

// average_down of a fine box onto the coarse cells it covers, every component:
// crse = (1/r^3) * sum of the fine cells (k, j, i order, from 0)
__global__ void __launch_bounds__(BT) bk_avgdown(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                 const int* __restrict__ owner, const Tile* __restrict__ tiles,
                                                 int ntiles, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    const int r = lev[b.level].ratio;
    int i, j, k;
    avg_of(b, r, t, i, j, k);
    const int w[3] = {i, j, k};
    const int ob = owner_at(lev[b.level - 1], owner, w);
    if (ob < 0) continue;
    const Fab& C = boxes[ob].snew;
    const Fab& F = b.snew;
    const double volfrac = 1.0 / (double)(r * r * r);
    for (int n = 0; n < nc; ++n) {
        double acc = 0.0;
        for (int kr = 0; kr < r; ++kr)
            for (int jr = 0; jr < r; ++jr)
                for (int ir = 0; ir < r; ++ir) acc = __dadd_rn(acc, F(i * r + ir, j * r + jr, k * r + kr, n));
        C(i, j, k, n) = __dmul_rn(volfrac, acc);
    }
    TILE_END
}

__global__ void __launch_bounds__(BT) bk_cut_list(const CutBox* __restrict__ cb, const Tile* __restrict__ tiles,
                                                  int ntiles, int2* __restrict__ list, unsigned* __restrict__ count) {
    TILE_LOOP
    const CutBox& c = cb[tl.box];
    int i, j, k;
    cell_of(c, t, i, j, k);
    const double vf = c.S(i, j, k, VFRAC);
    const bool cut = vf > 0.0 && vf < 1.0;
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, cut);
    if (m) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
        base = __shfl_sync(act, base, leader);
        if (cut) list[base + __popc(m & ((1u << lane) - 1u))] = make_int2(tl.box, (int)t);
    }
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_cut(const CutBox* __restrict__ cb, const int2* __restrict__ list,
                                             const unsigned* __restrict__ count) {
    const unsigned n = *count;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x) {
        const int2 e = list[w];
        cutcell_one<NS>(cb[e.x], e.y);
    }
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_prim(const RhsBox* __restrict__ B, const Tile* __restrict__ tiles, int ntiles) {
    TILE_LOOP
    prim_body<NS>(B[tl.box], t);
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_face(const RhsBox* __restrict__ B, const Tile* __restrict__ tiles, int ntiles) {
    TILE_LOOP
    face_body<NS>(B[tl.box], tl.part, t);
    TILE_END
}

template <bool FAST>
__global__ void __launch_bounds__(BT) bk_flux(const RhsBox* __restrict__ B, const Tile* __restrict__ tiles, int ntiles) {
    TILE_LOOP
    flux_body<FAST>(B[tl.box], tl.part >> 5, tl.part & 31, t);
    TILE_END
}

constexpr int SWEEP_BT = 128;
__global__ void __launch_bounds__(SWEEP_BT, 2) bk_flux_sweep(const RhsBox* __restrict__ B,
                                                             const Tile* __restrict__ tiles, int ntiles) {
    TILE_LOOP
    flux5_sweep_body(B[tl.box], tl.part >> 5, tl.part & 31, t);
    TILE_END
}
__global__ void __launch_bounds__(SWEEP_BT, 2) bk_flux5_face(const RhsBox* __restrict__ B,
                                                             const Tile* __restrict__ tiles, int ntiles) {
    TILE_LOOP
    flux5_face_body(B[tl.box], tl.part >> 5, tl.part & 31, t);
    TILE_END
}

// WENO5 with Navier-Stokes terms in the one-division mode: column sweep or
// per-face form of the same arithmetic (bitwise equal; the autotuner picks).
bool flux_sweep_mode() {
    return c_host_params().order_hyp == 5 && c_host_params().do_ns && weno_fast_mode();
}

__global__ void __launch_bounds__(BT) bk_update(const RhsBox* __restrict__ B, const Tile* __restrict__ tiles,
                                                int ntiles, int stage, double dt, const double* __restrict__ dtp) {
    if (dtp) dt = *dtp;
    TILE_LOOP
    update_body(B[tl.box], stage, dt, tl.part, t);
    TILE_END
}

__device__ __forceinline__ Valid valid_mbox(const MBox& b) {
    Valid v;
    v.n = 1;
    for (int d = 0; d < 3; ++d) {
        v.lo[d] = b.lo[d];
        v.len[d] = b.hi[d] - b.lo[d] + 1;
        v.n *= v.len[d];
    }
    return v;
}

// phi_old <- phi_new, all components
__global__ void __launch_bounds__(BT) bk_copy_old(const MBox* __restrict__ boxes, const Tile* __restrict__ tiles,
                                                  int ntiles, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    const Valid v = valid_mbox(b);
    int i, j, k;
    cell_of(v, t, i, j, k);
    copy_comps(&b.sold(i, j, k, 0), b.sold.ns, &b.snew(i, j, k, 0), b.snew.ns, nc);
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_chem(const MBox* __restrict__ boxes, const Tile* __restrict__ tiles,
                                              int ntiles, double dt, int nc, const double* __restrict__ dtp) {
    if (dtp) dt = *dtp;
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    chem_substep_body<NS>(valid_mbox(b), b.sold, b.snew, dt, nc, t);
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_prims(const MBox* __restrict__ boxes, const Tile* __restrict__ tiles,
                                               int ntiles, int nspec, int clip) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    const Valid v = valid_mbox(b);
    prims_body<NS>(v, b.snew, t);
    if (clip) clip_body(v, b.snew, nspec, t);
    TILE_END
}

// EstTimeStep over the tile list of valid cells: per level, the maxima of the
// wave speed and of the species diffusivity (one atomic per warp and tile).
template <int NS>
__global__ void __launch_bounds__(BT) bk_timestep(const MBox* __restrict__ boxes, const Tile* __restrict__ tiles,
                                                  int ntiles, RunState* __restrict__ R) {
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
        const Tile tl = tiles[ti];
        const MBox& b = boxes[tl.box];
        const Valid v = valid_mbox(b);
        double ws = 0.0, md = 0.0;
        for (long long t = tl.start + threadIdx.x; t < tl.end; t += blockDim.x) {
            int i, j, k;
            cell_of(v, t, i, j, k);
            double w1, m1;
            timestep_cell<NS>(b.snew, i, j, k, w1, m1);
            ws = fmax(ws, w1);
            md = fmax(md, m1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            ws = fmax(ws, __shfl_down_sync(0xffffffffu, ws, o));
            md = fmax(md, __shfl_down_sync(0xffffffffu, md, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomic_max_nonneg(&R->acc[2 * b.level], ws);
            atomic_max_nonneg(&R->acc[2 * b.level + 1], md);
        }
    }
}

// ComputeDt with one dt for every level (Source/mflo_timestep.cpp:18-50 with
// no subcycling): per level EstTimeStep (:136-153) times cfl, capped at 1.1 x
// the previous dt, the minimum over levels, clamped to stop_time.  The same
// operations in the same order as the host path (mfg_est_timestep and the
// driver's compute_dt).
__global__ void bk_compute_dt(const LevelG* __restrict__ lev, RunState* __restrict__ R) {
    double dt0 = 1.7976931348623157e308;
    for (int l = 0; l < R->nlev; ++l) {
        const double h0 = R->acc[2 * l], h1 = R->acc[2 * l + 1];
        double est = 1.7976931348623157e308;
        if (h0 > 0)
            for (int d = 0; d < 3; ++d) est = dmin_(est, __ddiv_rn(lev[l].dx[d], h0));
        if (h1 > 0)
            for (int d = 0; d < 3; ++d)
                est = dmin_(est, __ddiv_rn(__ddiv_rn(__dmul_rn(__dmul_rn(0.5, lev[l].dx[d]), lev[l].dx[d]), h1), 3.0));
        est = __dmul_rn(est, R->cfl);
        const double cap = __dmul_rn(1.1, R->dt_prev);
        const double dtl = (cap < est) ? cap : est;
        dt0 = dmin_(dt0, dtl);
    }
    const double eps = __dmul_rn(1e-3, dt0);
    if (__dadd_rn(R->t, dt0) > __dsub_rn(R->stop_time, eps)) dt0 = __dsub_rn(R->stop_time, R->t);
    R->dt = dt0;
}

// Loop condition of mfg_boxlist_evolve (mflo::EvolveAMR, Source/mflo_evolve.cpp:
// 21-88): step count and final time, the stop-time break, and the status bits
// where the reference aborts (NaN, negative pressure).
__device__ __forceinline__ unsigned run_continue(const RunState* R) {
    const unsigned bad = g_status & (MFG_STATUS_NAN | MFG_STATUS_NEG_PRESSURE);
    return (R->istep < R->max_step && R->t < R->final_time && !bad) ? 1u : 0u;
}

__global__ void bk_run_init(RunState* __restrict__ R, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, run_continue(R));
}

__global__ void bk_run_advance(RunState* __restrict__ R, cudaGraphConditionalHandle h) {
    const double dt = R->dt;
    R->t = __dadd_rn(R->t, dt);
    R->istep += 1;
    R->dt_prev = dt;
    for (int q = 0; q < 2 * RUN_MAXLEV; ++q) R->acc[q] = 0.0;
    unsigned c = run_continue(R);
    if (R->t >= __dsub_rn(R->stop_time, __dmul_rn(1e-6, dt))) c = 0u;
    cudaGraphSetConditional(h, c);
}

// ComputeDt of the subcycled hierarchy (Source/mflo_timestep.cpp:18-50):
// per level EstTimeStep x cfl capped at 1.1 x the level's previous dt,
// dt_0 = min over levels of (product of ratios up to l) x that, the stop-time
// clamp, then dt_l = dt_{l-1} / ratio_l.
__global__ void bk_compute_dt_amr(const LevelG* __restrict__ lev, RunState* __restrict__ R) {
    double tmp[RUN_MAXLEV];
    for (int l = 0; l < R->nlev; ++l) {
        const double h0 = R->acc[2 * l], h1 = R->acc[2 * l + 1];
        double est = 1.7976931348623157e308;
        if (h0 > 0)
            for (int d = 0; d < 3; ++d) est = dmin_(est, __ddiv_rn(lev[l].dx[d], h0));
        if (h1 > 0)
            for (int d = 0; d < 3; ++d)
                est = dmin_(est, __ddiv_rn(__ddiv_rn(__dmul_rn(__dmul_rn(0.5, lev[l].dx[d]), lev[l].dx[d]), h1), 3.0));
        tmp[l] = __dmul_rn(est, R->cfl);
    }
    double dt0 = tmp[0];
    int nf = 1;
    for (int l = 0; l < R->nlev; ++l) {
        tmp[l] = dmin_(tmp[l], __dmul_rn(1.1, R->dtl_prev[l]));
        nf *= (l > 0) ? lev[l].ratio : 1;
        dt0 = dmin_(dt0, __dmul_rn((double)nf, tmp[l]));
    }
    const double eps = __dmul_rn(1e-3, dt0);
    if (__dadd_rn(R->t, dt0) > __dsub_rn(R->stop_time, eps)) dt0 = __dsub_rn(R->stop_time, R->t);
    R->dtl[0] = dt0;
    for (int l = 1; l < R->nlev; ++l) R->dtl[l] = __ddiv_rn(R->dtl[l - 1], (double)lev[l].ratio);
}

// The coarse-data coefficients of every fill of one coarse step, in the order
// of the host recursion (amr_time_step): level l advancing from `time` sets
// t_old = t_new, t_new += dt_l, and its three stages read level l-1 at time,
// time + dt_l, time + dt_l (mflo::GetData); the substeps of level l+1 start at
// time + (i-1) dt_{l+1}.
__global__ void bk_amr_plan(const LevelG* __restrict__ lev, const RunState* __restrict__ R,
                            TCoef* __restrict__ coef) {
    const int nlev = R->nlev;
    double t_old[RUN_MAXLEV], t_new[RUN_MAXLEV], ftime[RUN_MAXLEV];
    int fnext[RUN_MAXLEV];
    for (int l = 0; l < nlev; ++l) t_old[l] = t_new[l] = R->t;
    int ev = 0;
    // level 0: no coarser data
    t_old[0] = t_new[0];
    t_new[0] = __dadd_rn(t_new[0], R->dtl[0]);
    ftime[0] = R->t;
    fnext[0] = 1;
    int depth = 0;
    while (depth >= 0) {
        const int lc = depth;
        if (lc + 1 < nlev && fnext[lc] <= lev[lc + 1].ratio) {
            const int i = fnext[lc]++;
            const int lf = lc + 1;
            const double dtf = R->dtl[lf];
            const double time = __fma_rn((double)(i - 1), dtf, ftime[lc]);
            t_old[lf] = t_new[lf];
            t_new[lf] = __dadd_rn(t_new[lf], dtf);
            for (int stage = 1; stage <= 3; ++stage) {
                const double T = stage == 1 ? time : __dadd_rn(time, dtf);
                const int l = lf - 1;
                TCoef c{0, 0.0, 0.0};
                const double teps = __dmul_rn(__dsub_rn(t_new[l], t_old[l]), 1.e-3);
                if (T > __dsub_rn(t_new[l], teps) && T < __dadd_rn(t_new[l], teps)) {
                    c.kind = 1;
                } else if (T > __dsub_rn(t_old[l], teps) && T < __dadd_rn(t_old[l], teps)) {
                    c.kind = 0;
                } else {
                    c.kind = 2;
                    c.a = __ddiv_rn(__dsub_rn(t_new[l], T), __dsub_rn(t_new[l], t_old[l]));
                    c.b = __ddiv_rn(__dsub_rn(T, t_old[l]), __dsub_rn(t_new[l], t_old[l]));
                }
                coef[ev++] = c;
            }
            ftime[lf] = time;
            fnext[lf] = 1;
            depth = lf;
        } else {
            --depth;
        }
    }
}

__global__ void bk_run_advance_amr(RunState* __restrict__ R, cudaGraphConditionalHandle h) {
    const double dt = R->dtl[0];
    R->t = __dadd_rn(R->t, dt);
    R->istep += 1;
    for (int l = 0; l < R->nlev; ++l) R->dtl_prev[l] = R->dtl[l];
    for (int q = 0; q < 2 * RUN_MAXLEV; ++q) R->acc[q] = 0.0;
    unsigned c = run_continue(R);
    if (R->t >= __dsub_rn(R->stop_time, __dmul_rn(1e-6, dt))) c = 0u;
    cudaGraphSetConditional(h, c);
}

#undef TILE_LOOP
#undef TILE_END

int igcd(int a, int b) {
    a = a < 0 ? -a : a;
    b = b < 0 ? -b : b;
    while (b) {
        int t = a % b;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace
}  // namespace mfg

using namespace mfg;

struct mfg_boxlist {
    int nbox = 0, nlev = 0;
    std::vector<mfg_box> boxes;
    std::vector<mfg_geom> geoms;
    std::vector<RhsBox> rhs;
    std::vector<CutBox> cut;
    std::vector<MBox> mbox;
    std::vector<LevelG> levg;
    RhsBox* d_rhs = nullptr;
    CutBox* d_cut = nullptr;
    MBox* d_mbox = nullptr;
    LevelG* d_lev = nullptr;
    int* d_owner = nullptr;
    double* d_scratch = nullptr;
    int2* d_cutlist = nullptr;
    unsigned* d_count = nullptr;  // [0]: batched cut count, [1]: plain per-box count
    int* d_plainlist = nullptr;
    PhaseTiles ph[PH_COUNT];
    std::vector<PhaseTiles> level_grown;  // per-level tiles of grown cells (plain-mode fill)
    int cut_grid = 0;
    int flux_form = 2;          // with flux_sweep_mode(): 2 column sweep, 1 per-face form
    int flux_tiles_kind = -1;   // flux_kind() the flux tiles were built for
    cudaGraphExec_t gexec = nullptr;
    double gdt = 0.0;
    long long cells = 0;
    // multi-level step (mfg_boxlist_step_amr)
    int amr_rc = MFG_ERR_STATE;            // MFG_OK when the hierarchy is aligned and properly nested
    double* d_cp = nullptr;                // coarse patches of the boxes of levels > 0
    std::vector<PhaseTiles> lt;            // per level and phase (level * PH_ALL + phase)
    int lt_version = -1;                   // tile_version the per-level lists were built for
    int tile_version = 0;                  // bumped whenever the all-box tile lists change
    std::vector<RegEnt*> d_ent;            // [l]: register cells of the l / l-1 interface
    std::vector<IEnt*> d_ient;             // [l]: coarse cells with fine ghost children to interpolate
    std::vector<int> nient;
    std::vector<double*> d_reg;
    std::vector<int> nent;
    std::vector<std::array<int, 7>> eoff;  // [l]: first entry of each orientation (x-lo, y-lo, z-lo, x-hi, ...)
    TCoef* d_coef = nullptr;
    std::vector<TCoef> hcoef;
    int nevents = 0;
    cudaGraphExec_t gexec_amr = nullptr;
    double gdt_amr = 0.0;
    int lt_flux_kind = -1;
    std::vector<int> h_owner;              // host copy of the owner maps
    // device-resident time loop (mfg_boxlist_evolve)
    RunState* d_run = nullptr;
    cudaGraphExec_t gexec_run = nullptr;
    cudaGraphExec_t gexec_run_amr = nullptr;
};

namespace {

// Flux-phase kernel: 0 flux_body, 1 WENO5 per-face form, 2 WENO5 column sweep.
int flux_kind(const mfg_boxlist& L) { return flux_sweep_mode() ? L.flux_form : 0; }

void free_tiles(PhaseTiles& p) {
    if (p.d) cudaFree(p.d);
    p.d = nullptr;
    p.n = 0;
}

long long items_of(const mfg_boxlist& L, int ph, int b, int part) {
    const mfg_box& x = L.boxes[b];
    long long n[3];
    for (int d = 0; d < 3; ++d) n[d] = x.hi[d] - x.lo[d] + 1;
    switch (ph) {
        case PH_GROWN: return (n[0] + 6) * (n[1] + 6) * (n[2] + 6);
        case PH_VALID:
        case PH_UPDATE: return n[0] * n[1] * n[2];
        case PH_FACE: return (n[0] + (part == 0)) * (n[1] + (part == 1)) * (n[2] + (part == 2));
        case PH_FLUX: {
            const int d = part >> 5;
            if (flux_kind(L) == 2) return sweep_items(L.rhs[b], d);
            return (n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
        }
        case PH_CP: {
            if (x.level == 0) return 0;
            const MBox& m = L.mbox[b];
            return (long long)(m.cphi[0] - m.cplo[0] + 1) * (m.cphi[1] - m.cplo[1] + 1) * (m.cphi[2] - m.cplo[2] + 1);
        }
        case PH_AVG: {
            if (x.level == 0) return 0;
            const long long r = L.levg[x.level].ratio;
            return (n[0] / r) * (n[1] / r) * (n[2] / r);
        }
    }
    return 0;
}

std::vector<int> parts_of(int ph) {
    const int ns = c_host_params().nspec;
    std::vector<int> p;
    if (ph == PH_FACE)
        p = {0, 1, 2};
    else if (ph == PH_FLUX) {
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < NCONS + ns; ++c) p.push_back(d * 32 + c);
    } else if (ph == PH_UPDATE) {
        for (int c = 0; c < NFLO + ns; ++c) p.push_back(c);
    } else {
        p = {0};
    }
    return p;
}

cudaError_t build_tiles(mfg_boxlist& L, PhaseTiles& P, int ph, int tile_items, int level) {
    std::vector<Tile> t;
    for (int b = 0; b < L.nbox; ++b) {
        if (level >= 0 && L.boxes[b].level != level) continue;
        for (int part : parts_of(ph)) {
            const long long n = items_of(L, ph, b, part);
            for (long long s = 0; s < n; s += tile_items) t.push_back({b, part, s, std::min(n, s + tile_items)});
        }
    }
    free_tiles(P);
    if (ph == PH_FLUX && level < 0) L.flux_tiles_kind = flux_kind(L);
    if (level < 0) ++L.tile_version;
    P.tile_items = tile_items;
    P.n = (int)t.size();
    P.grid = P.grid_cap > 0 ? std::min(P.n, P.grid_cap) : P.n;
    if (P.n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&P.d, t.size() * sizeof(Tile));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(P.d, t.data(), t.size() * sizeof(Tile), cudaMemcpyHostToDevice);
}

int ns_bucket(int ns) { return ns <= 1 ? 1 : ns <= 2 ? 2 : ns <= 4 ? 4 : ns <= 8 ? 8 : 16; }

#define MFG_UNPACK(...) __VA_ARGS__
// KER<NS-bucket><<<CFG>>>ARGS for the current species count
#define NS_DISPATCH(KER, CFG, ARGS)                                   \
    switch (ns_bucket(c_host_params().nspec)) {                        \
        case 1: KER<1><<<MFG_UNPACK CFG>>> ARGS; break;                 \
        case 2: KER<2><<<MFG_UNPACK CFG>>> ARGS; break;                 \
        case 4: KER<4><<<MFG_UNPACK CFG>>> ARGS; break;                 \
        case 8: KER<8><<<MFG_UNPACK CFG>>> ARGS; break;                 \
        default: KER<16><<<MFG_UNPACK CFG>>> ARGS; break;               \
    }

// ---- batched phases --------------------------------------------------------------
// The tile lists a phase runs over: every box, or the boxes of one level.
struct TSet {
    const PhaseTiles* t[PH_ALL];
    const PhaseTiles& operator[](int p) const { return *t[p]; }
};
TSet all_tiles(const mfg_boxlist& L) {
    TSet s;
    for (int p = 0; p < PH_ALL; ++p) s.t[p] = p < PH_COUNT ? &L.ph[p] : nullptr;
    return s;
}
TSet level_tiles(const mfg_boxlist& L, int l) {
    TSet s;
    for (int p = 0; p < PH_ALL; ++p) s.t[p] = &L.lt[(size_t)l * PH_ALL + p];
    return s;
}

void b_fill(mfg_boxlist& L, const PhaseTiles& T, int src, cudaStream_t st, int interp = 0) {
    if (!T.n) return;
    const int nc = NFLO + c_host_params().nspec;
    {
        ProfScope ps(K_FILL_COPY, st);
        bk_fill_copy<<<T.grid, BT, 0, st>>>(L.d_mbox, L.d_lev, L.d_owner, T.d, T.n, src, nc, interp);
    }
    for (int s = 1; s <= 3; ++s) {
        ProfScope ps(K_FILL_BC, st);
        NS_DISPATCH(bk_fill_bc, (T.grid, BT, 0, st), (L.d_mbox, L.d_lev, T.d, T.n, s, nc));
    }
}

void b_cutcells(mfg_boxlist& L, const PhaseTiles& T, cudaStream_t st) {
    ProfScope ps(K_CUT, st);
    cudaMemsetAsync(L.d_count, 0, sizeof(unsigned), st);
    bk_cut_list<<<T.grid, BT, 0, st>>>(L.d_cut, T.d, T.n, L.d_cutlist, L.d_count);
    NS_DISPATCH(bk_cut, (L.cut_grid, BT, 0, st), (L.d_cut, L.d_cutlist, L.d_count));
}

void b_rhs(mfg_boxlist& L, const TSet& TS, int stage, double dt, cudaStream_t st, const double* dtp = nullptr) {
    const int ord = c_host_params().order_hyp;
    if (ord >= 4) {
        const PhaseTiles& T = TS[PH_GROWN];
        ProfScope ps(K_PRIM, st);
        NS_DISPATCH(bk_prim, (T.grid, BT, 0, st), (L.d_rhs, T.d, T.n));
    }
    {
        const PhaseTiles& T = TS[PH_FACE];
        ProfScope ps(K_FACE, st);
        NS_DISPATCH(bk_face, (T.grid, BT, 0, st), (L.d_rhs, T.d, T.n));
    }
    if (!(c_host_params().do_ns && ord <= 2)) {
        const PhaseTiles& T = TS[PH_FLUX];
        ProfScope ps(K_FLUX, st);
        if (flux_kind(L) == 2)
            bk_flux_sweep<<<T.grid, SWEEP_BT, 0, st>>>(L.d_rhs, T.d, T.n);
        else if (flux_kind(L) == 1)
            bk_flux5_face<<<T.grid, SWEEP_BT, 0, st>>>(L.d_rhs, T.d, T.n);
        else if (weno_fast_mode())
            bk_flux<true><<<T.grid, BT, 0, st>>>(L.d_rhs, T.d, T.n);
        else
            bk_flux<false><<<T.grid, BT, 0, st>>>(L.d_rhs, T.d, T.n);
    }
    {
        const PhaseTiles& T = TS[PH_UPDATE];
        ProfScope ps(K_UPDATE, st);
        bk_update<<<T.grid, BT, 0, st>>>(L.d_rhs, T.d, T.n, stage, dt, dtp);
    }
}

// dtp (optional): device address of dt (mfg_boxlist_evolve's loop).
void step_batched(mfg_boxlist& L, double dt, cudaStream_t st, const double* dtp = nullptr) {
    const int nc = NFLO + c_host_params().nspec;
    const PhaseTiles& V = L.ph[PH_VALID];
    {
        ProfScope ps(K_COPY, st);
        bk_copy_old<<<V.grid, BT, 0, st>>>(L.d_mbox, V.d, V.n, nc);
    }
    const TSet T = all_tiles(L);
    for (int stage = 1; stage <= 3; ++stage) {
        b_fill(L, L.ph[PH_GROWN], stage == 1 ? 0 : 1, st);
        b_cutcells(L, L.ph[PH_VALID], st);
        b_rhs(L, T, stage, dt, st, dtp);
    }
    {
        ProfScope ps(K_COPY, st);
        bk_copy_old<<<V.grid, BT, 0, st>>>(L.d_mbox, V.d, V.n, nc);
    }
    {
        ProfScope ps(K_CHEM, st);
        NS_DISPATCH(bk_chem, (V.grid, BT, 0, st), (L.d_mbox, V.d, V.n, dt, nc, dtp));
    }
    {
        ProfScope ps(K_PRIMS, st);
        NS_DISPATCH(bk_prims, (V.grid, BT, 0, st), (L.d_mbox, V.d, V.n, c_host_params().nspec, 1));
    }
}

// Plain form: the same kernels launched once per box (RHS, cut cells, bookends)
// and once per level (fill), as an MFIter loop would.
int step_plain(mfg_boxlist& L, double dt, cudaStream_t st) {
    const int nc = NFLO + c_host_params().nspec;
    Fab none;
    memset(&none, 0, sizeof(none));
    for (int b = 0; b < L.nbox; ++b)
        if (launch_axpy_valid(L.boxes[b], make_fab(L.boxes[b].s_old), none, 0.0, true, make_fab(L.boxes[b].s_new), nc,
                              st) != cudaSuccess)
            return MFG_ERR_CUDA;
    for (int stage = 1; stage <= 3; ++stage) {
        for (int l = 0; l < L.nlev; ++l) b_fill(L, L.level_grown[l], stage == 1 ? 0 : 1, st);
        for (int b = 0; b < L.nbox; ++b)
            if (launch_cutcells_box(L.boxes[b], L.geoms[L.boxes[b].level], nullptr, L.d_plainlist, L.d_count + 1, st) !=
                cudaSuccess)
                return MFG_ERR_CUDA;
        for (int b = 0; b < L.nbox; ++b)
            if (launch_rhs_box(L.rhs[b], stage, dt, weno_fast_mode(), st) != cudaSuccess) return MFG_ERR_CUDA;
    }
    for (int b = 0; b < L.nbox; ++b) {
        if (launch_axpy_valid(L.boxes[b], make_fab(L.boxes[b].s_old), none, 0.0, true, make_fab(L.boxes[b].s_new), nc,
                              st) != cudaSuccess)
            return MFG_ERR_CUDA;
        if (launch_chem_substep(L.boxes[b], dt, st) != cudaSuccess) return MFG_ERR_CUDA;
        if (launch_update_prims(L.boxes[b], nullptr, st) != cudaSuccess) return MFG_ERR_CUDA;
        if (launch_clip_species(L.boxes[b], st) != cudaSuccess) return MFG_ERR_CUDA;
    }
    return MFG_OK;
}

void drop_graph(mfg_boxlist& L) {
    if (L.gexec) cudaGraphExecDestroy(L.gexec);
    L.gexec = nullptr;
    if (L.gexec_amr) cudaGraphExecDestroy(L.gexec_amr);
    L.gexec_amr = nullptr;
    if (L.gexec_run) cudaGraphExecDestroy(L.gexec_run);
    L.gexec_run = nullptr;
    if (L.gexec_run_amr) cudaGraphExecDestroy(L.gexec_run_amr);
    L.gexec_run_amr = nullptr;
}

// ---- multi-level step -------------------------------------------------------------
// mflo::timeStep (Source/mflo_evolve.cpp:174-247) over the whole hierarchy:
// level l advances with dt_l = dt_{l-1} / ratio_l (ratio_l substeps per step
// of level l-1).  Each stage fills the level's ghost cells (FillPatch,
// Source/mflo_gridwork.cpp:135-173: for l > 0 the coarse patch of each box
// from level l-1 at the stage time, its physical boundaries, then
// cell_cons_interp where level l has no data), runs cut cells and the RHS
// with the stage update, and adds the stage's face fluxes to the flux
// registers (CrseInit on the finer interface with -dt dA w, FineAdd on the
// coarser one with dt dA w; w = 1/6, 1/6, 2/3, Source/mflo_evolve.cpp:
// 655-681); then the chemistry sub-step.  After the substeps of level l+1,
// level l is refluxed and level l+1 averaged down onto it; after the coarse
// step, primitive refresh and clipping of every box.
constexpr double kTwo3rd = 0.6666666666666666667;  // Source/mflo_constants.H two3rd, sixth
constexpr double kSixth = kTwo3rd * 0.5 * 0.5;

int hfloor_div(int a, int r) { return a >= 0 ? a / r : -((-a + r - 1) / r); }

bool hwrap(const LevelG& G, const int iv[3], int w[3]) {
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
        const int len = G.dhi[d] - G.dlo[d] + 1;
        w[d] = iv[d];
        if (G.per[d]) {
            while (w[d] < G.dlo[d]) w[d] += len;
            while (w[d] > G.dhi[d]) w[d] -= len;
        } else if (w[d] < G.dlo[d] || w[d] > G.dhi[d]) {
            inside = false;
        }
    }
    return inside;
}

int howner(const mfg_boxlist& L, int l, const int w[3]) {
    const LevelG& G = L.levg[l];
    const int m0 = (w[0] - G.dlo[0]) / G.gran, m1 = (w[1] - G.dlo[1]) / G.gran, m2 = (w[2] - G.dlo[2]) / G.gran;
    return L.h_owner[G.owner_off + m0 + (long long)G.mlen[0] * (m1 + (long long)G.mlen[1] * m2)];
}

// Coarse patches, nesting and alignment checks, flux registers.  A hierarchy
// that fails a check keeps amr_rc = MFG_ERR_ARG (the common-dt step still works).
cudaError_t setup_amr(mfg_boxlist& L) {
    const int nlev = L.nlev, nc = NFLO + c_host_params().nspec, C = NCONS + c_host_params().nspec;
    int rc = MFG_OK;
    for (int l = 1; l < nlev; ++l) {
        const int r = L.levg[l].ratio;
        const mfg_geom &gc = L.geoms[l - 1], &gf = L.geoms[l];
        if (r < 2 || r > 4) rc = MFG_ERR_ARG;  // refinement ratios 2, 3, 4
        for (int d = 0; d < 3 && !rc; ++d) {
            if (gf.domain_lo[d] != gc.domain_lo[d] * r || gf.domain_hi[d] + 1 != (gc.domain_hi[d] + 1) * r ||
                gf.is_periodic[d] != gc.is_periodic[d] || std::fabs(gc.dx[d] / gf.dx[d] - r) > 1e-9 * r)
                rc = MFG_ERR_ARG;
        }
    }
    // coarse patches
    size_t tot = 0;
    std::vector<size_t> off(L.nbox, 0);
    for (int b = 0; b < L.nbox && !rc; ++b) {
        MBox& m = L.mbox[b];
        if (m.level == 0) continue;
        const int r = L.levg[m.level].ratio;
        size_t n = 1;
        for (int d = 0; d < 3; ++d) {
            if (hfloor_div(m.lo[d], r) * r != m.lo[d] || hfloor_div(m.hi[d] + 1, r) * r != m.hi[d] + 1) rc = MFG_ERR_ARG;
            m.cplo[d] = hfloor_div(m.lo[d] - MFG_NGROW, r) - 1;
            m.cphi[d] = hfloor_div(m.hi[d] + MFG_NGROW, r) + 1;
            n *= (size_t)(m.cphi[d] - m.cplo[d] + 1);
            // a reflecting boundary mirrors the patch's outside layers onto its inside ones
            const LevelG& G = L.levg[m.level - 1];
            if (!G.per[d]) {
                const int inside = std::min(m.cphi[d], G.dhi[d]) - std::max(m.cplo[d], G.dlo[d]) + 1;
                if (inside < std::max(G.dlo[d] - m.cplo[d], m.cphi[d] - G.dhi[d])) rc = MFG_ERR_ARG;
            }
        }
        off[b] = tot;
        tot += n;
    }
    // nesting: every coarse-patch cell inside the coarse domain lies on the coarse level
    for (int b = 0; b < L.nbox && !rc; ++b) {
        const MBox& m = L.mbox[b];
        if (m.level == 0) continue;
        for (int k = m.cplo[2]; k <= m.cphi[2] && !rc; ++k)
            for (int j = m.cplo[1]; j <= m.cphi[1] && !rc; ++j)
                for (int i = m.cplo[0]; i <= m.cphi[0] && !rc; ++i) {
                    const int iv[3] = {i, j, k};
                    int w[3];
                    if (hwrap(L.levg[m.level - 1], iv, w) && howner(L, m.level - 1, w) < 0) rc = MFG_ERR_ARG;
                }
    }
    // coarse cells with fine ghost children to interpolate, per level
    std::vector<std::vector<IEnt>> ients(nlev);
    for (int b = 0; b < L.nbox && !rc; ++b) {
        const MBox& m = L.mbox[b];
        if (m.level == 0) continue;
        const int l = m.level, r = L.levg[l].ratio;
        const LevelG& G = L.levg[l];
        for (int k = m.cplo[2] + 1; k < m.cphi[2]; ++k)
            for (int j = m.cplo[1] + 1; j < m.cphi[1]; ++j)
                for (int i = m.cplo[0] + 1; i < m.cphi[0]; ++i) {
                    unsigned long long mask = 0;
                    for (int mk = 0; mk < r; ++mk)
                        for (int mj = 0; mj < r; ++mj)
                            for (int mi = 0; mi < r; ++mi) {
                                const int fv[3] = {i * r + mi, j * r + mj, k * r + mk};
                                bool ghost = false, grown = true;
                                for (int d = 0; d < 3; ++d) {
                                    ghost |= fv[d] < m.lo[d] || fv[d] > m.hi[d];
                                    grown &= fv[d] >= m.lo[d] - MFG_NGROW && fv[d] <= m.hi[d] + MFG_NGROW;
                                }
                                int w[3];
                                if (!ghost || !grown || !hwrap(G, fv, w) || howner(L, l, w) >= 0) continue;
                                mask |= 1ull << (mi + r * (mj + r * mk));
                            }
                    if (mask) ients[l].push_back(IEnt{b, i, j, k, mask});
                }
    }
    // flux registers, in the order x-lo, y-lo, z-lo, x-hi, y-hi, z-hi
    L.d_ent.assign(nlev, nullptr);
    L.d_reg.assign(nlev, nullptr);
    L.nent.assign(nlev, 0);
    L.eoff.assign(nlev, std::array<int, 7>{});
    std::vector<std::vector<RegEnt>> ents(nlev);
    for (int l = 1; l < nlev && !rc; ++l) {
        const int r = L.levg[l].ratio;
        for (int side = 0; side < 2; ++side)
            for (int d = 0; d < 3; ++d) {
                L.eoff[l][d + 3 * side] = (int)ents[l].size();
                for (int fb = 0; fb < L.nbox && !rc; ++fb) {
                    const MBox& m = L.mbox[fb];
                    if (m.level != l) continue;
                    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
                    const int fface = side ? m.hi[d] + 1 : m.lo[d];
                    const int cface = hfloor_div(fface, r);
                    for (int q2 = hfloor_div(m.lo[t2], r); q2 <= hfloor_div(m.hi[t2] + 1, r) - 1; ++q2)
                        for (int q1 = hfloor_div(m.lo[t1], r); q1 <= hfloor_div(m.hi[t1] + 1, r) - 1; ++q1) {
                            int cc[3];
                            cc[d] = side ? cface : cface - 1;
                            cc[t1] = q1;
                            cc[t2] = q2;
                            int w[3];
                            if (!hwrap(L.levg[l - 1], cc, w)) continue;
                            const int fw[3] = {w[0] * r, w[1] * r, w[2] * r};
                            if (howner(L, l, fw) >= 0) continue;  // covered: average_down overwrites it
                            const int cb = howner(L, l - 1, w);
                            if (cb < 0) {
                                rc = MFG_ERR_ARG;
                                break;
                            }
                            RegEnt e;
                            e.fb = fb;
                            e.cb = cb;
                            e.d = d;
                            e.side = side;
                            for (int q = 0; q < 3; ++q) e.cc[q] = e.cf[q] = w[q];
                            e.cf[d] = side ? w[d] : w[d] + 1;
                            e.ff[d] = fface;
                            e.ff[t1] = q1 * r;
                            e.ff[t2] = q2 * r;
                            ents[l].push_back(e);
                        }
                }
            }
        L.eoff[l][6] = (int)ents[l].size();
    }
    L.amr_rc = rc;
    if (rc) return cudaSuccess;
    cudaError_t e;
    if ((e = cudaMalloc(&L.d_cp, std::max<size_t>(tot * nc, 1) * sizeof(double))) != cudaSuccess) return e;
    cudaMemsetAsync(L.d_cp, 0, std::max<size_t>(tot * nc, 1) * sizeof(double));
    for (int b = 0; b < L.nbox; ++b) {
        MBox& m = L.mbox[b];
        if (m.level == 0) continue;
        int len[3];
        for (int d = 0; d < 3; ++d) len[d] = m.cphi[d] - m.cplo[d] + 1;
        m.cp = dense_fab(L.d_cp + off[b] * nc, m.cplo, len);
    }
    if ((e = cudaMemcpy(L.d_mbox, L.mbox.data(), L.nbox * sizeof(MBox), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    L.d_ient.assign(nlev, nullptr);
    L.nient.assign(nlev, 0);
    for (int l = 1; l < nlev; ++l) {
        const size_t ni = ients[l].size();
        L.nient[l] = (int)ni;
        if ((e = cudaMalloc(&L.d_ient[l], std::max<size_t>(ni, 1) * sizeof(IEnt))) != cudaSuccess) return e;
        if (ni && (e = cudaMemcpy(L.d_ient[l], ients[l].data(), ni * sizeof(IEnt), cudaMemcpyHostToDevice)) !=
                      cudaSuccess)
            return e;
    }
    for (int l = 1; l < nlev; ++l) {
        const size_t ne = ents[l].size();
        L.nent[l] = (int)ne;
        if ((e = cudaMalloc(&L.d_ent[l], std::max<size_t>(ne, 1) * sizeof(RegEnt))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&L.d_reg[l], std::max<size_t>(ne * C, 1) * sizeof(double))) != cudaSuccess) return e;
        if (ne && (e = cudaMemcpy(L.d_ent[l], ents[l].data(), ne * sizeof(RegEnt), cudaMemcpyHostToDevice)) !=
                      cudaSuccess)
            return e;
    }
    int nev = 0, sub = 1;
    for (int l = 1; l < nlev; ++l) {
        sub *= L.levg[l].ratio;
        nev += 3 * sub;
    }
    L.nevents = nev;
    L.hcoef.assign(std::max(nev, 1), TCoef{0, 0.0, 0.0});
    return cudaMalloc(&L.d_coef, std::max(nev, 1) * sizeof(TCoef));
}

// Per-level tile lists with the settings of the all-box lists.
cudaError_t build_level_tiles(mfg_boxlist& L) {
    L.lt.resize((size_t)L.nlev * PH_ALL);
    for (int l = 0; l < L.nlev; ++l)
        for (int p = 0; p < PH_ALL; ++p) {
            const PhaseTiles& src = L.ph[p < PH_COUNT ? p : PH_GROWN];
            PhaseTiles& P = L.lt[(size_t)l * PH_ALL + p];
            P.grid_cap = src.grid_cap;
            cudaError_t e = build_tiles(L, P, p, src.tile_items, l);
            if (e != cudaSuccess) return e;
        }
    L.lt_version = L.tile_version;
    L.lt_flux_kind = flux_kind(L);
    return cudaSuccess;
}

struct AmrRun {
    std::vector<double> t_old, t_new, dt;
    int ev = 0;
    bool launch = false;
    int mode = 1;
    cudaStream_t st = nullptr;
    int rc = MFG_OK;
    const double* ddt = nullptr;  // device per-level dt (mfg_boxlist_evolve_amr), batched mode only
};

// Coarse data of level l at time T (mflo::GetData, Source/mflo.cpp:310-330):
// new / old within 1e-3 dt of t_new / t_old, else their linear combination.
int amr_coef(mfg_boxlist& L, AmrRun& R, int l, double T) {
    TCoef c{0, 0.0, 0.0};
    const double teps = (R.t_new[l] - R.t_old[l]) * 1.e-3;
    if (T > R.t_new[l] - teps && T < R.t_new[l] + teps) {
        c.kind = 1;
    } else if (T > R.t_old[l] - teps && T < R.t_old[l] + teps) {
        c.kind = 0;
    } else {
        const double t0 = R.t_old[l], t1 = R.t_new[l];
        c.kind = 2;
        c.a = (t1 - T) / (t1 - t0);
        c.b = (T - t0) / (t1 - t0);
    }
    L.hcoef[R.ev] = c;
    return R.ev++;
}

void amr_note(AmrRun& R, cudaError_t e) {
    if (e != cudaSuccess && R.rc == MFG_OK) R.rc = MFG_ERR_CUDA;
}

void amr_fill(mfg_boxlist& L, AmrRun& R, int l, int src, int ev) {
    const TSet T = level_tiles(L, l);
    const int nc = NFLO + c_host_params().nspec;
    cudaStream_t st = R.st;
    if (l > 0 && T[PH_CP].n) {
        const PhaseTiles& C = T[PH_CP];
        {
            ProfScope ps(K_AMR_PATCH, st);
            bk_cp_fill<<<C.grid, BT, 0, st>>>(L.d_mbox, L.d_lev, L.d_owner, C.d, C.n, L.d_coef, ev, nc);
        }
        for (int s = 1; s <= 3; ++s) {
            ProfScope ps(K_AMR_PATCH, st);
            NS_DISPATCH(bk_cp_bc, (C.grid, BT, 0, st), (L.d_mbox, L.d_lev, C.d, C.n, s, nc));
        }
        const int ni = L.nient[l];
        ProfScope ps(K_AMR_INTERP, st);
        if (ni) bk_cp_interp<<<dim3((ni + BT - 1) / BT, nc), BT, 0, st>>>(L.d_ient[l], ni, L.d_mbox, L.d_lev);
    }
    b_fill(L, T[PH_GROWN], src, st, 1);
}

void amr_copy_old(mfg_boxlist& L, AmrRun& R, int l) {
    const int nc = NFLO + c_host_params().nspec;
    if (R.mode == 0) {
        Fab none;
        memset(&none, 0, sizeof(none));
        for (int b = 0; b < L.nbox; ++b)
            if (L.boxes[b].level == l)
                amr_note(R, launch_axpy_valid(L.boxes[b], make_fab(L.boxes[b].s_old), none, 0.0, true,
                                              make_fab(L.boxes[b].s_new), nc, R.st));
        return;
    }
    const PhaseTiles& V = level_tiles(L, l)[PH_VALID];
    if (!V.n) return;
    ProfScope ps(K_COPY, R.st);
    bk_copy_old<<<V.grid, BT, 0, R.st>>>(L.d_mbox, V.d, V.n, nc);
}

void amr_stage(mfg_boxlist& L, AmrRun& R, int l, int stage, double dtl) {
    cudaStream_t st = R.st;
    if (R.mode == 0) {
        for (int b = 0; b < L.nbox; ++b)
            if (L.boxes[b].level == l)
                amr_note(R, launch_cutcells_box(L.boxes[b], L.geoms[l], nullptr, L.d_plainlist, L.d_count + 1, st));
        for (int b = 0; b < L.nbox; ++b)
            if (L.boxes[b].level == l) amr_note(R, launch_rhs_box(L.rhs[b], stage, dtl, weno_fast_mode(), st));
    } else {
        const TSet T = level_tiles(L, l);
        if (T[PH_VALID].n) {
            b_cutcells(L, T[PH_VALID], st);
            b_rhs(L, T, stage, dtl, st, R.ddt ? R.ddt + l : nullptr);
        }
    }
    // flux registers
    const int C = NCONS + c_host_params().nspec;
    const double ff = stage < 3 ? kSixth : kTwo3rd;
    const double* dx = L.geoms[l].dx;
    const double dA[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
    const double* dtp = R.ddt ? R.ddt + l : nullptr;
    ProfScope ps(K_AMR_SYNC, st);
    if (l + 1 < L.nlev && L.nent[l + 1]) {
        const int ne = L.nent[l + 1];
        const RegScale S = {{-dtl * dA[0] * ff, -dtl * dA[1] * ff, -dtl * dA[2] * ff}, {dA[0], dA[1], dA[2]}, ff, -1.0};
        bk_reg_crse<<<dim3((ne + BT - 1) / BT, C), BT, 0, st>>>(L.d_ent[l + 1], ne, L.d_rhs, L.d_reg[l + 1], S, dtp);
    }
    if (l > 0 && L.nent[l]) {
        const int ne = L.nent[l];
        const RegScale S = {{dtl * dA[0] * ff, dtl * dA[1] * ff, dtl * dA[2] * ff}, {dA[0], dA[1], dA[2]}, ff, 1.0};
        bk_reg_fine<<<dim3((ne + BT - 1) / BT, C), BT, 0, st>>>(L.d_ent[l], ne, L.d_rhs, L.d_reg[l], S, dtp,
                                                               L.levg[l].ratio);
    }
}

void amr_chem(mfg_boxlist& L, AmrRun& R, int l, double dtl) {
    const int nc = NFLO + c_host_params().nspec;
    if (R.mode == 0) {
        for (int b = 0; b < L.nbox; ++b)
            if (L.boxes[b].level == l) amr_note(R, launch_chem_substep(L.boxes[b], dtl, R.st));
        return;
    }
    const PhaseTiles& V = level_tiles(L, l)[PH_VALID];
    if (!V.n) return;
    ProfScope ps(K_CHEM, R.st);
    NS_DISPATCH(bk_chem, (V.grid, BT, 0, R.st), (L.d_mbox, V.d, V.n, dtl, nc, R.ddt ? R.ddt + l : nullptr));
}

void amr_sync(mfg_boxlist& L, AmrRun& R, int l) {  // reflux of level l, average_down of l+1 onto l
    cudaStream_t st = R.st;
    const int nc = NFLO + c_host_params().nspec;
    ProfScope ps(K_AMR_SYNC, st);
    const double* dx = L.geoms[l].dx;
    const double vol = dx[0] * dx[1] * dx[2];
    const int ne = L.nent[l + 1];
    for (int o = 0; o < 6; ++o) {
        const int e0 = L.eoff[l + 1][o], e1 = L.eoff[l + 1][o + 1];
        if (e1 > e0)
            bk_reflux<<<dim3((e1 - e0 + BT - 1) / BT, nc), BT, 0, st>>>(L.d_ent[l + 1], e0, e1, ne, L.d_mbox,
                                                                      L.d_reg[l + 1], vol);
    }
    const PhaseTiles& A = level_tiles(L, l + 1)[PH_AVG];
    if (A.n) bk_avgdown<<<A.grid, BT, 0, st>>>(L.d_mbox, L.d_lev, L.d_owner, A.d, A.n, nc);
}

void amr_advance(mfg_boxlist& L, AmrRun& R, int l, double time, double dtl) {
    if (R.launch) amr_copy_old(L, R, l);
    R.t_old[l] = R.t_new[l];
    R.t_new[l] += dtl;
    if (R.launch && l + 1 < L.nlev && L.nent[l + 1])
        amr_note(R, cudaMemsetAsync(L.d_reg[l + 1], 0,
                                    (size_t)L.nent[l + 1] * (NCONS + c_host_params().nspec) * sizeof(double), R.st));
    for (int stage = 1; stage <= 3; ++stage) {
        const double T = stage == 1 ? time : time + dtl;
        const int ev = l > 0 ? amr_coef(L, R, l - 1, T) : -1;
        if (!R.launch) continue;
        amr_fill(L, R, l, stage == 1 ? 0 : 1, ev);
        amr_stage(L, R, l, stage, dtl);
    }
    if (R.launch) {
        amr_copy_old(L, R, l);
        amr_chem(L, R, l, dtl);
    }
}

void amr_time_step(mfg_boxlist& L, AmrRun& R, int l, double time) {
    amr_advance(L, R, l, time, R.dt[l]);
    if (l + 1 < L.nlev) {
        // time + (i-1) dt_{l+1} as one rounding, as the device plan computes it
        for (int i = 1; i <= L.levg[l + 1].ratio; ++i)
            amr_time_step(L, R, l + 1, std::fma((double)(i - 1), R.dt[l + 1], time));
        if (R.launch) amr_sync(L, R, l);
    }
}

int amr_run(mfg_boxlist& L, double time, double dt0, bool launch, int mode, cudaStream_t st,
            const double* ddt = nullptr) {
    AmrRun R;
    R.launch = launch;
    R.mode = mode;
    R.st = st;
    R.ddt = ddt;
    R.t_old.assign(L.nlev, time);
    R.t_new.assign(L.nlev, time);
    R.dt.assign(L.nlev, dt0);
    for (int l = 1; l < L.nlev; ++l) R.dt[l] = R.dt[l - 1] / L.levg[l].ratio;
    amr_time_step(L, R, 0, time);
    if (!launch) return MFG_OK;
    if (mode == 0) {
        for (int b = 0; b < L.nbox; ++b) {
            amr_note(R, launch_update_prims(L.boxes[b], nullptr, st));
            amr_note(R, launch_clip_species(L.boxes[b], st));
        }
    } else {
        const PhaseTiles& V = L.ph[PH_VALID];
        ProfScope ps(K_PRIMS, st);
        NS_DISPATCH(bk_prims, (V.grid, BT, 0, st), (L.d_mbox, V.d, V.n, c_host_params().nspec, 1));
    }
    amr_note(R, cudaGetLastError());
    return R.rc;
}

// The device time loop as one graph: an init kernel setting the loop
// condition, then a WHILE node whose body is one step with its ComputeDt
// (common dt, or the subcycled hierarchy with the fill plan) and the kernel
// that advances the time and sets the condition again.
bool build_run_graph(mfg_boxlist& L, cudaStream_t st, bool amr) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t n0, wn;
    cudaKernelNodeParams kp;
    memset(&kp, 0, sizeof(kp));
    RunState* R = L.d_run;
    void* args[] = {&R, &h};
    kp.func = (void*)bk_run_init;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = args;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    bool ok = cudaGraphConditionalHandleCreate(&h, g, 0, 0) == cudaSuccess &&
              cudaGraphAddKernelNode(&n0, g, nullptr, 0, &kp) == cudaSuccess;
    if (ok) {
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        ok = cudaGraphAddNode(&wn, g, &n0, nullptr, 1, &cp) == cudaSuccess;
    }
    if (ok) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
             cudaSuccess;
        if (ok) {
            const PhaseTiles& V = L.ph[PH_VALID];
            NS_DISPATCH(bk_timestep, (V.grid, BT, 0, st), (L.d_mbox, V.d, V.n, R));
            if (amr) {
                bk_compute_dt_amr<<<1, 1, 0, st>>>(L.d_lev, R);
                bk_amr_plan<<<1, 1, 0, st>>>(L.d_lev, R, L.d_coef);
                const int rc = amr_run(L, 0.0, 0.0, true, 1, st, R->dtl);
                ok = rc == MFG_OK;
                bk_run_advance_amr<<<1, 1, 0, st>>>(R, h);
            } else {
                bk_compute_dt<<<1, 1, 0, st>>>(L.d_lev, R);
                step_batched(L, 0.0, st, &R->dt);
                bk_run_advance<<<1, 1, 0, st>>>(R, h);
            }
            ok = (cudaStreamEndCapture(st, &body) == cudaSuccess) && ok;
        }
    }
    cudaGraphExec_t& ex = amr ? L.gexec_run_amr : L.gexec_run;
    if (ok) ok = cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    cudaGraphDestroy(g);
    if (!ok) {
        ex = nullptr;
        note_cuda_error(cudaGetLastError(), "building the device time loop");
    }
    return ok;
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

extern "C" {

int mfg_boxlist_create(const mfg_box* boxes, int nbox, const mfg_geom* geoms, int nlev, mfg_boxlist** out) {
    if (!out || nlev < 1 || nlev > 16) return MFG_ERR_ARG;
    *out = nullptr;
    int rc = validate_boxes(boxes, nbox, true, false, true, true);
    if (rc) return rc;
    if (c_host_params().conj_ht) return MFG_ERR_STATE;  // the batched cut cells have no CHT pre-pass
    for (int b = 0; b < nbox; ++b)
        if (boxes[b].level < 0 || boxes[b].level >= nlev) return MFG_ERR_ARG;
    // one Dirichlet weight table serves every level: cell aspect ratios must agree
    for (int l = 1; l < nlev; ++l)
        for (int d = 0; d < 3; ++d)
            if (geoms[l].dx[d] * geoms[0].dx[(d + 1) % 3] != geoms[0].dx[d] * geoms[l].dx[(d + 1) % 3]) return MFG_ERR_ARG;
    mfg_boxlist* L = new mfg_boxlist();
    L->nbox = nbox;
    L->nlev = nlev;
    L->boxes.assign(boxes, boxes + nbox);
    L->geoms.assign(geoms, geoms + nlev);
    cudaError_t e = cudaSuccess;
    // per-box RHS scratch, all boxes resident at once
    std::vector<size_t> off(nbox);
    size_t tot = 0, maxcells = 0;
    for (int b = 0; b < nbox; ++b) {
        int n[3];
        for (int d = 0; d < 3; ++d) n[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
        off[b] = tot;
        tot += (rhs_box_scratch_doubles(n) + 31) / 32 * 32;
        maxcells = std::max(maxcells, (size_t)n[0] * n[1] * n[2]);
        L->cells += (long long)n[0] * n[1] * n[2];
    }
    if ((e = cudaMalloc(&L->d_scratch, std::max<size_t>(tot, 1) * sizeof(double))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_cutlist, std::max<size_t>(L->cells, 1) * sizeof(int2))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_count, 2 * sizeof(unsigned))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_plainlist, std::max<size_t>(maxcells, 1) * sizeof(int))) != cudaSuccess) goto fail;
    L->rhs.resize(nbox);
    L->cut.resize(nbox);
    L->mbox.resize(nbox);
    for (int b = 0; b < nbox; ++b) {
        const mfg_box& x = boxes[b];
        const mfg_geom& g = geoms[x.level];
        L->rhs[b] = layout_rhs_box(x, g, L->d_scratch + off[b]);
        CutBox& c = L->cut[b];
        memset(&c, 0, sizeof(c));
        c.n = 1;
        for (int d = 0; d < 3; ++d) {
            c.lo[d] = x.lo[d];
            c.len[d] = x.hi[d] - x.lo[d] + 1;
            c.n *= c.len[d];
            c.dx[d] = g.dx[d];
        }
        c.S = make_fab(x.sborder);
        c.dxmin = std::min(g.dx[0], std::min(g.dx[1], g.dx[2]));
        c.tcht = nullptr;
        MBox& m = L->mbox[b];
        memset(&m, 0, sizeof(m));
        for (int d = 0; d < 3; ++d) {
            m.lo[d] = x.lo[d];
            m.hi[d] = x.hi[d];
        }
        m.level = x.level;
        m.sb = make_fab(x.sborder);
        m.sold = make_fab(x.s_old);
        m.snew = make_fab(x.s_new);
    }
    {
        // per-level owner maps, concatenated; indices are global box numbers
        std::vector<int> own;
        L->levg.resize(nlev);
        for (int l = 0; l < nlev; ++l) {
            const mfg_geom& g = geoms[l];
            int gr = 0;
            for (int d = 0; d < 3; ++d) gr = igcd(gr, g.domain_hi[d] - g.domain_lo[d] + 1);
            for (int b = 0; b < nbox; ++b) {
                if (boxes[b].level != l) continue;
                for (int d = 0; d < 3; ++d) {
                    gr = igcd(gr, boxes[b].lo[d] - g.domain_lo[d]);
                    gr = igcd(gr, boxes[b].hi[d] + 1 - g.domain_lo[d]);
                }
            }
            if (gr <= 0) gr = 1;
            LevelG& G = L->levg[l];
            memset(&G, 0, sizeof(G));
            for (int d = 0; d < 3; ++d) {
                G.dlo[d] = g.domain_lo[d];
                G.dhi[d] = g.domain_hi[d];
                G.per[d] = g.is_periodic[d];
                G.mlen[d] = (g.domain_hi[d] - g.domain_lo[d] + 1) / gr;
            }
            G.gran = gr;
            for (int d = 0; d < 3; ++d) G.dx[d] = g.dx[d];
            G.owner_off = (long long)own.size();
            G.ratio = (l > 0) ? (int)((geoms[l - 1].dx[0] / g.dx[0]) + 0.5) : 1;
            const size_t base = own.size();
            own.resize(base + (size_t)G.mlen[0] * G.mlen[1] * G.mlen[2], -1);
            for (int b = 0; b < nbox; ++b) {
                if (boxes[b].level != l) continue;
                int a[3], z[3];
                for (int d = 0; d < 3; ++d) {
                    a[d] = (boxes[b].lo[d] - g.domain_lo[d]) / gr;
                    z[d] = (boxes[b].hi[d] + 1 - g.domain_lo[d]) / gr;
                }
                for (int q2 = a[2]; q2 < z[2]; ++q2)
                    for (int q1 = a[1]; q1 < z[1]; ++q1)
                        for (int q0 = a[0]; q0 < z[0]; ++q0)
                            own[base + q0 + (size_t)G.mlen[0] * (q1 + (size_t)G.mlen[1] * q2)] = b;
            }
        }
        if ((e = cudaMalloc(&L->d_owner, std::max<size_t>(own.size(), 1) * sizeof(int))) != cudaSuccess) goto fail;
        if ((e = cudaMemcpy(L->d_owner, own.data(), own.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
            goto fail;
        L->h_owner.swap(own);
    }
    if ((e = cudaMalloc(&L->d_rhs, nbox * sizeof(RhsBox))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_cut, nbox * sizeof(CutBox))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_mbox, nbox * sizeof(MBox))) != cudaSuccess) goto fail;
    if ((e = cudaMalloc(&L->d_lev, nlev * sizeof(LevelG))) != cudaSuccess) goto fail;
    cudaMemcpy(L->d_rhs, L->rhs.data(), nbox * sizeof(RhsBox), cudaMemcpyHostToDevice);
    cudaMemcpy(L->d_cut, L->cut.data(), nbox * sizeof(CutBox), cudaMemcpyHostToDevice);
    cudaMemcpy(L->d_mbox, L->mbox.data(), nbox * sizeof(MBox), cudaMemcpyHostToDevice);
    cudaMemcpy(L->d_lev, L->levg.data(), nlev * sizeof(LevelG), cudaMemcpyHostToDevice);
    for (int p = 0; p < PH_COUNT; ++p)
        if ((e = build_tiles(*L, L->ph[p], p, 4096, -1)) != cudaSuccess) goto fail;
    L->level_grown.resize(nlev);
    for (int l = 0; l < nlev; ++l)
        if ((e = build_tiles(*L, L->level_grown[l], PH_GROWN, 4096, l)) != cudaSuccess) goto fail;
    L->cut_grid = sm_count() * 8;
    // the Dirichlet weight table of the cut cells (shared with the per-box path)
    {
        double w[125];
        const double dxmin = std::min(geoms[0].dx[0], std::min(geoms[0].dx[1], geoms[0].dx[2]));
        const double dn[3] = {geoms[0].dx[0] / dxmin, geoms[0].dx[1] / dxmin, geoms[0].dx[2] / dxmin};
        for (int n = -2; n <= 2; ++n)
            for (int m = -2; m <= 2; ++m)
                for (int l = -2; l <= 2; ++l) {
                    const double a = l * dn[0], bb = m * dn[1], ee = n * dn[2];
                    const double d2 = (a * a + bb * bb) + ee * ee;
                    w[(l + 2) + 5 * ((m + 2) + 5 * (n + 2))] = (l == 0 && m == 0 && n == 0) ? 0.0 : 1.0 / (d2 + kTiny2);
                }
        if ((e = cudaMemcpyToSymbol(c_wdir, w, sizeof(w))) != cudaSuccess) goto fail;
    }
    if ((e = setup_amr(*L)) != cudaSuccess) goto fail;
    *out = L;
    return MFG_OK;
fail:
    mfg_boxlist_destroy(L);
    return MFG_ERR_CUDA;
}

int mfg_boxlist_destroy(mfg_boxlist* L) {
    if (!L) return MFG_OK;
    drop_graph(*L);
    for (int p = 0; p < PH_COUNT; ++p) free_tiles(L->ph[p]);
    for (auto& t : L->level_grown) free_tiles(t);
    for (auto& t : L->lt) free_tiles(t);
    for (double* r : L->d_reg) cudaFree(r);
    for (IEnt* r : L->d_ient) cudaFree(r);
    for (RegEnt* r : L->d_ent) cudaFree(r);
    cudaFree(L->d_cp);
    cudaFree(L->d_coef);
    cudaFree(L->d_run);
    cudaFree(L->d_rhs);
    cudaFree(L->d_cut);
    cudaFree(L->d_mbox);
    cudaFree(L->d_lev);
    cudaFree(L->d_owner);
    cudaFree(L->d_scratch);
    cudaFree(L->d_cutlist);
    cudaFree(L->d_count);
    cudaFree(L->d_plainlist);
    delete L;
    return MFG_OK;
}

// mode 0: plain per-box launches; 1: batched launches; 2: batched step replayed
// from a CUDA graph (captured on first use and whenever dt changes).
int mfg_boxlist_step(mfg_boxlist* L, double time, double dt, int mode, void* stream) {
    (void)time;
    if (!L) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (L->flux_tiles_kind != flux_kind(*L)) {  // the WENO mode changed since the tiles were built
        drop_graph(*L);
        if (build_tiles(*L, L->ph[PH_FLUX], PH_FLUX, L->ph[PH_FLUX].tile_items, -1) != cudaSuccess)
            return MFG_ERR_CUDA;
    }
    if (mode == 0) return step_plain(*L, dt, st);
    if (mode == 1) {
        step_batched(*L, dt, st);
        return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
    }
    if (mode != 2) return MFG_ERR_ARG;
    if (!L->gexec || L->gdt != dt) {
        drop_graph(*L);
        if (!st) return MFG_ERR_ARG;  // capture needs a non-default stream
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return MFG_ERR_CUDA;
        step_batched(*L, dt, st);
        if (cudaStreamEndCapture(st, &g) != cudaSuccess || !g) return MFG_ERR_CUDA;
        cudaError_t e = cudaGraphInstantiate(&L->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            L->gexec = nullptr;
            return MFG_ERR_CUDA;
        }
        L->gdt = dt;
    }
    return cudaGraphLaunch(L->gexec, st) == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

// mflo::EvolveAMR's loop on the device for the common-dt step: one CUDA graph
// whose WHILE node repeats {EstTimeStep, ComputeDt, step, time += dt} while a
// kernel-set condition holds, so no step waits for the host.
int mfg_boxlist_evolve(mfg_boxlist* L, double final_time, double stop_time, int max_step, double* time, double* dt,
                       int* istep, void* stream) {
    if (!L || !time || !dt || !istep || !stream) return MFG_ERR_ARG;
    if (L->nlev > RUN_MAXLEV) return MFG_ERR_ARG;
    if (profile_enabled()) return MFG_ERR_STATE;  // event records cannot live in a conditional body
    cudaStream_t st = (cudaStream_t)stream;
    if (L->flux_tiles_kind != flux_kind(*L)) {
        drop_graph(*L);
        if (build_tiles(*L, L->ph[PH_FLUX], PH_FLUX, L->ph[PH_FLUX].tile_items, -1) != cudaSuccess)
            return MFG_ERR_CUDA;
    }
    if (!L->d_run && cudaMalloc(&L->d_run, sizeof(RunState)) != cudaSuccess) return MFG_ERR_CUDA;
    if (!L->gexec_run && !build_run_graph(*L, st, false)) return MFG_ERR_CUDA;
    RunState hs;
    memset(&hs, 0, sizeof(hs));
    hs.t = *time;
    hs.dt_prev = *dt;
    hs.final_time = final_time;
    hs.stop_time = stop_time;
    hs.cfl = c_host_params().cfl;
    hs.istep = *istep;
    hs.max_step = max_step;
    hs.nlev = L->nlev;
    if (cudaMemcpyAsync(L->d_run, &hs, sizeof(hs), cudaMemcpyHostToDevice, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaGraphLaunch(L->gexec_run, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaMemcpyAsync(&hs, L->d_run, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MFG_ERR_CUDA;
    *time = hs.t;
    *dt = hs.dt_prev;
    *istep = hs.istep;
    unsigned v = 0;
    if (read_status(&v, false) != cudaSuccess) return MFG_ERR_CUDA;
    if (v & MFG_STATUS_NAN) return MFG_ERR_NAN;
    if (v & MFG_STATUS_NEG_PRESSURE) return MFG_ERR_NEG_PRESSURE;
    return MFG_OK;
}

// mflo::EvolveAMR's loop for the subcycled hierarchy, on the device.
int mfg_boxlist_evolve_amr(mfg_boxlist* L, double final_time, double stop_time, int max_step, double* time,
                           double* dt, int* istep, void* stream) {
    if (!L || !time || !dt || !istep || !stream) return MFG_ERR_ARG;
    if (L->amr_rc) return L->amr_rc;
    if (L->nlev > RUN_MAXLEV) return MFG_ERR_ARG;
    if (profile_enabled()) return MFG_ERR_STATE;
    cudaStream_t st = (cudaStream_t)stream;
    if (L->flux_tiles_kind != flux_kind(*L)) {
        drop_graph(*L);
        if (build_tiles(*L, L->ph[PH_FLUX], PH_FLUX, L->ph[PH_FLUX].tile_items, -1) != cudaSuccess)
            return MFG_ERR_CUDA;
    }
    if (L->lt_version != L->tile_version || L->lt_flux_kind != flux_kind(*L)) {
        drop_graph(*L);
        if (build_level_tiles(*L) != cudaSuccess) return MFG_ERR_CUDA;
    }
    if (!L->d_run && cudaMalloc(&L->d_run, sizeof(RunState)) != cudaSuccess) return MFG_ERR_CUDA;
    if (!L->gexec_run_amr && !build_run_graph(*L, st, true)) return MFG_ERR_CUDA;
    RunState hs;
    memset(&hs, 0, sizeof(hs));
    hs.t = *time;
    hs.final_time = final_time;
    hs.stop_time = stop_time;
    hs.cfl = c_host_params().cfl;
    hs.istep = *istep;
    hs.max_step = max_step;
    hs.nlev = L->nlev;
    for (int l = 0; l < L->nlev; ++l) hs.dtl_prev[l] = dt[l];
    if (cudaMemcpyAsync(L->d_run, &hs, sizeof(hs), cudaMemcpyHostToDevice, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaGraphLaunch(L->gexec_run_amr, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaMemcpyAsync(&hs, L->d_run, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MFG_ERR_CUDA;
    *time = hs.t;
    for (int l = 0; l < L->nlev; ++l) dt[l] = hs.dtl_prev[l];
    *istep = hs.istep;
    unsigned v = 0;
    if (read_status(&v, false) != cudaSuccess) return MFG_ERR_CUDA;
    if (v & MFG_STATUS_NAN) return MFG_ERR_NAN;
    if (v & MFG_STATUS_NEG_PRESSURE) return MFG_ERR_NEG_PRESSURE;
    return MFG_OK;
}

// The reference's multi-level step (subcycling, two-level fill with
// conservative interpolation, flux registers, reflux, average_down).
int mfg_boxlist_step_amr(mfg_boxlist* L, double time, double dt0, int mode, void* stream) {
    if (!L || mode < 0 || mode > 2) return MFG_ERR_ARG;
    if (L->amr_rc) return L->amr_rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (L->flux_tiles_kind != flux_kind(*L)) {
        drop_graph(*L);
        if (build_tiles(*L, L->ph[PH_FLUX], PH_FLUX, L->ph[PH_FLUX].tile_items, -1) != cudaSuccess)
            return MFG_ERR_CUDA;
    }
    if (L->lt_version != L->tile_version || L->lt_flux_kind != flux_kind(*L)) {
        drop_graph(*L);
        if (build_level_tiles(*L) != cudaSuccess) return MFG_ERR_CUDA;
    }
    // coarse-data coefficients of this step's fills (host pass, then one upload;
    // the kernels, and a captured graph, read them from device memory)
    amr_run(*L, time, dt0, false, mode, st);
    if (L->nevents &&
        cudaMemcpyAsync(L->d_coef, L->hcoef.data(), L->nevents * sizeof(TCoef), cudaMemcpyHostToDevice, st) !=
            cudaSuccess)
        return MFG_ERR_CUDA;
    if (mode < 2) return amr_run(*L, time, dt0, true, mode, st);
    if (!L->gexec_amr || L->gdt_amr != dt0) {
        if (L->gexec_amr) cudaGraphExecDestroy(L->gexec_amr);
        L->gexec_amr = nullptr;
        if (!st) return MFG_ERR_ARG;  // capture needs a non-default stream
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return MFG_ERR_CUDA;
        const int rc = amr_run(*L, time, dt0, true, 1, st);
        if (cudaStreamEndCapture(st, &g) != cudaSuccess || !g) return MFG_ERR_CUDA;
        if (rc) {
            cudaGraphDestroy(g);
            return rc;
        }
        cudaError_t e = cudaGraphInstantiate(&L->gexec_amr, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            L->gexec_amr = nullptr;
            return MFG_ERR_CUDA;
        }
        L->gdt_amr = dt0;
    }
    return cudaGraphLaunch(L->gexec_amr, st) == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

// Measured search over tile size and grid size for each batched phase: every
// candidate runs the phase alone (the phases are idempotent on their inputs:
// fill, cut cells, face scalars, fluxes, and the update with stage 0, which only
// recomputes dsdt) and the fastest by CUDA events is kept.  results[] (optional,
// 3 doubles per phase: tile items, grid blocks, ms) reports the choice.
int mfg_boxlist_autotune(mfg_boxlist* L, double dt, double* results, void* stream) {
    if (!L) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int sms = sm_count();
    const int tiles_c[] = {1024, 4096, 16384};
    const int grids_c[] = {0, 2, 4, 8};  // 0: one block per tile, else x SMs
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int ord = c_host_params().order_hyp;
    for (int p = 0; p < PH_COUNT; ++p) {
        if (p == PH_FLUX && c_host_params().do_ns && ord <= 2) continue;
        float best = 1e30f;
        int bt = L->ph[p].tile_items, bg = L->ph[p].grid_cap, bf = L->flux_form;
        const int nforms = (p == PH_FLUX && flux_sweep_mode()) ? 2 : 1;
        for (int form = 0; form < nforms; ++form)
        for (int ti : tiles_c)
            for (int gc : grids_c) {
                if (nforms == 2) L->flux_form = 2 - form;
                PhaseTiles& P = L->ph[p];
                P.grid_cap = gc ? gc * sms : 0;
                if (build_tiles(*L, P, p, ti, -1) != cudaSuccess) return MFG_ERR_CUDA;
                float ms_min = 1e30f;
                for (int rep = 0; rep < 3; ++rep) {
                    cudaEventRecord(e0, st);
                    switch (p) {
                        case PH_GROWN: b_fill(*L, P, 1, st); break;
                        case PH_VALID: b_cutcells(*L, P, st); break;
                        case PH_FACE: {
                            NS_DISPATCH(bk_face, (P.grid, BT, 0, st), (L->d_rhs, P.d, P.n));
                            break;
                        }
                        case PH_FLUX:
                            if (flux_kind(*L) == 2)
                                bk_flux_sweep<<<P.grid, SWEEP_BT, 0, st>>>(L->d_rhs, P.d, P.n);
                            else if (flux_kind(*L) == 1)
                                bk_flux5_face<<<P.grid, SWEEP_BT, 0, st>>>(L->d_rhs, P.d, P.n);
                            else
                                bk_flux<true><<<P.grid, BT, 0, st>>>(L->d_rhs, P.d, P.n);
                            break;
                        case PH_UPDATE: bk_update<<<P.grid, BT, 0, st>>>(L->d_rhs, P.d, P.n, 0, dt, nullptr); break;
                    }
                    cudaEventRecord(e1, st);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    ms_min = std::min(ms_min, ms);
                }
                if (ms_min < best) {
                    best = ms_min;
                    bt = ti;
                    bg = P.grid_cap;
                    bf = L->flux_form;
                }
            }
        L->flux_form = bf;
        L->ph[p].grid_cap = bg;
        if (build_tiles(*L, L->ph[p], p, bt, -1) != cudaSuccess) return MFG_ERR_CUDA;
        if (results) {
            results[3 * p + 0] = bt;
            results[3 * p + 1] = L->ph[p].grid;
            results[3 * p + 2] = best;
            if (p == PH_FLUX) results[3 * PH_COUNT] = flux_kind(*L);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    drop_graph(*L);
    return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

long long mfg_boxlist_cells(const mfg_boxlist* L) { return L ? L->cells : 0; }

}  // extern "C"
