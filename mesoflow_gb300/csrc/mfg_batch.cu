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
};

struct LevelG {
    int dlo[3], dhi[3], per[3];
    int gran, mlen[3];
    long long owner_off;  // offset of this level's owner map in the concatenated map
    int ratio;            // refinement ratio to the coarser level
};

enum Phase { PH_GROWN = 0, PH_VALID, PH_FACE, PH_FLUX, PH_UPDATE, PH_COUNT };

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

// copy of valid data (own level, periodic images), else coarse-level injection
__global__ void __launch_bounds__(BT) bk_fill_copy(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                   const int* __restrict__ owner, const Tile* __restrict__ tiles,
                                                   int ntiles, int src, int nc) {
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
    if (ob < 0 && b.level > 0) {
        const LevelG& Gc = lev[b.level - 1];
        for (int d = 0; d < 3; ++d) cw[d] = Gc.dlo[d] + (w[d] - G.dlo[d]) / G.ratio;
        ob = owner_at(Gc, owner, cw);
    }
    if (ob < 0) continue;
    const MBox& o = boxes[ob];
    const Fab& S = src ? o.snew : o.sold;
    const long long qs = S.off(cw[0], cw[1], cw[2]);
    const long long qd = b.sb.off(i, j, k);
    for (int c = 0; c < nc; ++c) b.sb.p[qd + c * b.sb.ns] = S.p[qs + c * S.ns];
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_fill_bc(const MBox* __restrict__ boxes, const LevelG* __restrict__ lev,
                                                 const Tile* __restrict__ tiles, int ntiles, int stage, int nc) {
    TILE_LOOP
    const MBox& b = boxes[tl.box];
    int i, j, k;
    grown_of(b, t, i, j, k);
    const LevelG& G = lev[b.level];
    const int iv[3] = {i, j, k};
    bool out[3];
    int nout = 0;
    for (int d = 0; d < 3; ++d) {
        out[d] = !G.per[d] && (iv[d] < G.dlo[d] || iv[d] > G.dhi[d]);
        nout += out[d];
    }
    if (nout != stage) continue;
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
    const Fab& S = b.sb;
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
                                                int ntiles, int stage, double dt) {
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
    for (int c = 0; c < nc; ++c) b.sold(i, j, k, c) = b.snew(i, j, k, c);
    TILE_END
}

template <int NS>
__global__ void __launch_bounds__(BT) bk_chem(const MBox* __restrict__ boxes, const Tile* __restrict__ tiles,
                                              int ntiles, double dt, int nc) {
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
    if (ph == PH_FLUX) L.flux_tiles_kind = flux_kind(L);
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
void b_fill(mfg_boxlist& L, const PhaseTiles& T, int src, cudaStream_t st) {
    if (!T.n) return;
    const int nc = NFLO + c_host_params().nspec;
    {
        ProfScope ps(K_FILL_COPY, st);
        bk_fill_copy<<<T.grid, BT, 0, st>>>(L.d_mbox, L.d_lev, L.d_owner, T.d, T.n, src, nc);
    }
    for (int s = 1; s <= 3; ++s) {
        ProfScope ps(K_FILL_BC, st);
        NS_DISPATCH(bk_fill_bc, (T.grid, BT, 0, st), (L.d_mbox, L.d_lev, T.d, T.n, s, nc));
    }
}

void b_cutcells(mfg_boxlist& L, cudaStream_t st) {
    const PhaseTiles& T = L.ph[PH_VALID];
    ProfScope ps(K_CUT, st);
    cudaMemsetAsync(L.d_count, 0, sizeof(unsigned), st);
    bk_cut_list<<<T.grid, BT, 0, st>>>(L.d_cut, T.d, T.n, L.d_cutlist, L.d_count);
    NS_DISPATCH(bk_cut, (L.cut_grid, BT, 0, st), (L.d_cut, L.d_cutlist, L.d_count));
}

void b_rhs(mfg_boxlist& L, int stage, double dt, cudaStream_t st) {
    const int ord = c_host_params().order_hyp;
    if (ord >= 4) {
        const PhaseTiles& T = L.ph[PH_GROWN];
        ProfScope ps(K_PRIM, st);
        NS_DISPATCH(bk_prim, (T.grid, BT, 0, st), (L.d_rhs, T.d, T.n));
    }
    {
        const PhaseTiles& T = L.ph[PH_FACE];
        ProfScope ps(K_FACE, st);
        NS_DISPATCH(bk_face, (T.grid, BT, 0, st), (L.d_rhs, T.d, T.n));
    }
    if (!(c_host_params().do_ns && ord <= 2)) {
        const PhaseTiles& T = L.ph[PH_FLUX];
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
        const PhaseTiles& T = L.ph[PH_UPDATE];
        ProfScope ps(K_UPDATE, st);
        bk_update<<<T.grid, BT, 0, st>>>(L.d_rhs, T.d, T.n, stage, dt);
    }
}

void step_batched(mfg_boxlist& L, double dt, cudaStream_t st) {
    const int nc = NFLO + c_host_params().nspec;
    const PhaseTiles& V = L.ph[PH_VALID];
    {
        ProfScope ps(K_COPY, st);
        bk_copy_old<<<V.grid, BT, 0, st>>>(L.d_mbox, V.d, V.n, nc);
    }
    for (int stage = 1; stage <= 3; ++stage) {
        b_fill(L, L.ph[PH_GROWN], stage == 1 ? 0 : 1, st);
        b_cutcells(L, st);
        b_rhs(L, stage, dt, st);
    }
    {
        ProfScope ps(K_COPY, st);
        bk_copy_old<<<V.grid, BT, 0, st>>>(L.d_mbox, V.d, V.n, nc);
    }
    {
        ProfScope ps(K_CHEM, st);
        NS_DISPATCH(bk_chem, (V.grid, BT, 0, st), (L.d_mbox, V.d, V.n, dt, nc));
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
                        case PH_VALID: b_cutcells(*L, st); break;
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
                        case PH_UPDATE: bk_update<<<P.grid, BT, 0, st>>>(L->d_rhs, P.d, P.n, 0, dt); break;
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
