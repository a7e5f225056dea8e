// Single-level ghost fill of every box's Sborder (FillPatchSingleLevel with
// the case's physical boundary functor): copy of valid data from the owning
// box (periodic images included), then the physical boundaries in the order
// faces -> edges -> corners.  A cell outside the domain in the set D of
// non-periodic directions takes its value from the cell one step inward
// along d*: the highest direction of D whose boundary is ext_dir (the user
// functor runs after the extrapolation rules and checks x, y, z in turn,
// Source/mflo_bcfill.H:236-320), otherwise the highest direction of D.
// The physical-boundary launches cover only the blocks ("slabs") of the
// grown boxes that lie outside the domain, listed once per box layout, not
// every grown cell of every box.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "mfg_fill_body.cuh"

namespace mfg {
namespace {

constexpr int TPB = 256;

struct FillBox {
    int lo[3], hi[3];
    Fab sb, src;
};

struct FillGeom {
    int dlo[3], dhi[3], per[3];
    int gran;       // owner-map granularity (cells)
    int mlen[3];    // owner-map extent
    double dx[3], plo[3];
};

// A block of a box's grown region outside the domain: its cells leave the
// domain through the same directions (the bc_kernel stage = their number).
struct BcSlab {
    int box;
    int lo[3], len[3];
};

__device__ __forceinline__ void grown_cell(const FillBox& b, int64_t t, int& i, int& j, int& k, int64_t& n) {
    const int l0 = b.hi[0] - b.lo[0] + 1 + 2 * MFG_NGROW, l1 = b.hi[1] - b.lo[1] + 1 + 2 * MFG_NGROW,
              l2 = b.hi[2] - b.lo[2] + 1 + 2 * MFG_NGROW;
    n = (int64_t)l0 * l1 * l2;
    split3(t < n ? t : 0, l0, l1, i, j, k);
    i += b.lo[0] - MFG_NGROW;
    j += b.lo[1] - MFG_NGROW;
    k += b.lo[2] - MFG_NGROW;
}

__global__ void copy_kernel(const FillBox* __restrict__ boxes, FillGeom G, const int* __restrict__ owner, int ncomp) {
    const FillBox& b = boxes[blockIdx.y];
    int i, j, k;
    int64_t n;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    grown_cell(b, t, i, j, k, n);
    if (t >= n) return;
    int w[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int len = G.dhi[d] - G.dlo[d] + 1;
        if (G.per[d]) {
            while (w[d] < G.dlo[d]) w[d] += len;
            while (w[d] > G.dhi[d]) w[d] -= len;
        } else if (w[d] < G.dlo[d] || w[d] > G.dhi[d]) {
            return;  // physical boundary cell
        }
    }
    const int m0 = (w[0] - G.dlo[0]) / G.gran, m1 = (w[1] - G.dlo[1]) / G.gran, m2 = (w[2] - G.dlo[2]) / G.gran;
    const int ob = owner[m0 + G.mlen[0] * (m1 + G.mlen[1] * m2)];
    if (ob < 0) return;  // not covered at this level
    const FillBox& o = boxes[ob];
    // Sborder is never a state FAB, and the states are not written here
    copy_comps(b.sb.p + b.sb.off(i, j, k), b.sb.ns, o.src.p + o.src.off(w[0], w[1], w[2]), o.src.ns, ncomp);
}

// One launch per stage over the slabs of that stage only (blockIdx.y = slab).
template <int NS>
__global__ void bc_kernel(const FillBox* __restrict__ boxes, const BcSlab* __restrict__ slabs, FillGeom G, int stage,
                          int ncomp) {
    const BcSlab& sl = slabs[blockIdx.y];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)sl.len[0] * sl.len[1] * sl.len[2]) return;
    const FillBox& b = boxes[sl.box];
    int i, j, k;
    split3(t, sl.len[0], sl.len[1], i, j, k);
    i += sl.lo[0];
    j += sl.lo[1];
    k += sl.lo[2];
    const int iv[3] = {i, j, k};
    bool out[3];
    int nout = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        out[d] = !G.per[d] && (iv[d] < G.dlo[d] || iv[d] > G.dhi[d]);
        nout += out[d];
    }
    if (nout != stage) return;
    const DevParams& P = c_P;
    int dext = -1, dlast = -1;
#pragma unroll
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
    const int64_t qd = S.off(i, j, k);
    if (dext >= 0) {
        sv[ds] = lo ? G.dlo[ds] : G.dhi[ds];
        const int64_t qs = S.off(sv[0], sv[1], sv[2]);
        double s_int[NFLO + MAXS], s_ext[NFLO + MAXS];
        for (int c = 0; c < ncomp; ++c) s_int[c] = S.p[qs + c * S.ns];
        external_state<NS>(lo ? P.ext_lo[ds] : P.ext_hi[ds], ds, s_int, s_ext, ncomp);
        for (int c = 0; c < ncomp; ++c) S.p[qd + c * S.ns] = s_ext[c];
    } else if (kind == MFG_BC_FOEXTRAP) {
        sv[ds] = lo ? G.dlo[ds] : G.dhi[ds];
        const int64_t qs = S.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < ncomp; ++c) S.p[qd + c * S.ns] = S.p[qs + c * S.ns];
    } else {  // wall: reflect_even, reflect_odd for momenta and velocities
        sv[ds] = lo ? (2 * G.dlo[ds] - iv[ds] - 1) : (2 * G.dhi[ds] - iv[ds] + 1);
        const int64_t qs = S.off(sv[0], sv[1], sv[2]);
        for (int c = 0; c < ncomp; ++c) {
            const double x = S.p[qs + c * S.ns];
            S.p[qd + c * S.ns] = odd_at_wall(c) ? -x : x;
        }
    }
}

// Owner map cache (host-built, device-resident); rebuilt when the box layout changes.
struct OwnerCache {
    std::vector<int> key;
    int* d_owner = nullptr;
    size_t cap = 0;
    int gran = 1, mlen[3] = {0, 0, 0};
    FillBox* d_boxes = nullptr;
    size_t bcap = 0;
    std::vector<char> table;
    BcSlab* d_slabs = nullptr;  // grouped by stage 1, 2, 3
    size_t scap = 0;
    int nslab[3] = {0, 0, 0}, soff[3] = {0, 0, 0};
    int64_t smax[3] = {0, 0, 0};  // largest slab of each stage (cells)
} g_fill;

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

cudaError_t ensure_owner(const mfg_box* boxes, int nbox, const mfg_geom& g) {
    std::vector<int> key;
    key.reserve(nbox * 6 + 6);
    for (int d = 0; d < 3; ++d) {
        key.push_back(g.domain_lo[d]);
        key.push_back(g.domain_hi[d]);
    }
    for (int d = 0; d < 3; ++d) key.push_back(g.is_periodic[d] ? 1 : 0);
    for (int b = 0; b < nbox; ++b)
        for (int d = 0; d < 3; ++d) {
            key.push_back(boxes[b].lo[d]);
            key.push_back(boxes[b].hi[d]);
        }
    if (key == g_fill.key && g_fill.d_owner) return cudaSuccess;
    int gr = 0;
    for (int d = 0; d < 3; ++d) gr = igcd(gr, g.domain_hi[d] - g.domain_lo[d] + 1);
    for (int b = 0; b < nbox; ++b)
        for (int d = 0; d < 3; ++d) {
            gr = igcd(gr, boxes[b].lo[d] - g.domain_lo[d]);
            gr = igcd(gr, boxes[b].hi[d] + 1 - g.domain_lo[d]);
        }
    if (gr <= 0) gr = 1;
    int ml[3];
    for (int d = 0; d < 3; ++d) ml[d] = (g.domain_hi[d] - g.domain_lo[d] + 1) / gr;
    std::vector<int> own((size_t)ml[0] * ml[1] * ml[2], -1);
    for (int b = 0; b < nbox; ++b) {
        int a[3], e[3];
        for (int d = 0; d < 3; ++d) {
            a[d] = (boxes[b].lo[d] - g.domain_lo[d]) / gr;
            e[d] = (boxes[b].hi[d] + 1 - g.domain_lo[d]) / gr;
        }
        for (int z = a[2]; z < e[2]; ++z)
            for (int y = a[1]; y < e[1]; ++y)
                for (int x = a[0]; x < e[0]; ++x)
                    if (x >= 0 && y >= 0 && z >= 0 && x < ml[0] && y < ml[1] && z < ml[2])
                        own[x + (size_t)ml[0] * (y + (size_t)ml[1] * z)] = b;
    }
    cudaError_t e;
    if (own.size() > g_fill.cap) {
        if (g_fill.d_owner) cudaFree(g_fill.d_owner);
        g_fill.d_owner = nullptr;
        if ((e = cudaMalloc(&g_fill.d_owner, own.size() * sizeof(int))) != cudaSuccess) return e;
        g_fill.cap = own.size();
    }
    if ((e = cudaMemcpy(g_fill.d_owner, own.data(), own.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    // Slabs: per direction the grown extent splits into below / inside /
    // above the domain (one range when periodic); every combination with at
    // least one outside range is a slab of the stage = number of those.
    std::vector<BcSlab> sl[3];
    for (int b = 0; b < nbox; ++b) {
        int rlo[3][3], rhi[3][3], rout[3][3], nr[3];
        for (int d = 0; d < 3; ++d) {
            const int glo = boxes[b].lo[d] - MFG_NGROW, ghi = boxes[b].hi[d] + MFG_NGROW;
            const int dlo = g.domain_lo[d], dhi = g.domain_hi[d];
            nr[d] = 0;
            auto add = [&](int a, int z, int out) {
                if (a > z) return;
                rlo[d][nr[d]] = a;
                rhi[d][nr[d]] = z;
                rout[d][nr[d]] = out;
                ++nr[d];
            };
            if (g.is_periodic[d]) {
                add(glo, ghi, 0);
            } else {
                add(glo, std::min(ghi, dlo - 1), 1);
                add(std::max(glo, dlo), std::min(ghi, dhi), 0);
                add(std::max(glo, dhi + 1), ghi, 1);
            }
        }
        for (int c = 0; c < nr[2]; ++c)
            for (int bb = 0; bb < nr[1]; ++bb)
                for (int a = 0; a < nr[0]; ++a) {
                    const int r[3] = {a, bb, c};
                    int nout = 0;
                    BcSlab x;
                    x.box = b;
                    for (int d = 0; d < 3; ++d) {
                        nout += rout[d][r[d]];
                        x.lo[d] = rlo[d][r[d]];
                        x.len[d] = rhi[d][r[d]] - rlo[d][r[d]] + 1;
                    }
                    if (nout) sl[nout - 1].push_back(x);
                }
    }
    std::vector<BcSlab> all;
    for (int q = 0; q < 3; ++q) {
        g_fill.soff[q] = (int)all.size();
        g_fill.nslab[q] = (int)sl[q].size();
        g_fill.smax[q] = 0;
        for (const BcSlab& x : sl[q]) g_fill.smax[q] = std::max<int64_t>(g_fill.smax[q], (int64_t)x.len[0] * x.len[1] * x.len[2]);
        all.insert(all.end(), sl[q].begin(), sl[q].end());
    }
    if (all.size() > g_fill.scap) {
        if (g_fill.d_slabs) cudaFree(g_fill.d_slabs);
        g_fill.d_slabs = nullptr;
        if ((e = cudaMalloc(&g_fill.d_slabs, all.size() * sizeof(BcSlab))) != cudaSuccess) return e;
        g_fill.scap = all.size();
    }
    if (!all.empty() &&
        (e = cudaMemcpy(g_fill.d_slabs, all.data(), all.size() * sizeof(BcSlab), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    g_fill.gran = gr;
    for (int d = 0; d < 3; ++d) g_fill.mlen[d] = ml[d];
    g_fill.key = key;
    return cudaSuccess;
}

}  // namespace

void fill_release() {
    if (g_fill.d_owner) cudaFree(g_fill.d_owner);
    if (g_fill.d_boxes) cudaFree(g_fill.d_boxes);
    if (g_fill.d_slabs) cudaFree(g_fill.d_slabs);
    g_fill = OwnerCache();
}

cudaError_t launch_fill_patch(const mfg_box* boxes, int nbox, const mfg_geom& g, int s_src, double time,
                              cudaStream_t st) {
    (void)time;
    cudaError_t e = ensure_owner(boxes, nbox, g);
    if (e != cudaSuccess) return e;
    // Box tables for both source arrays; re-uploaded only when a descriptor changes.
    std::vector<FillBox> fb(2 * (size_t)nbox);
    int64_t maxn = 0;
    for (int b = 0; b < nbox; ++b) {
        for (int h = 0; h < 2; ++h) {
            FillBox& x = fb[(size_t)h * nbox + b];
            for (int d = 0; d < 3; ++d) {
                x.lo[d] = boxes[b].lo[d];
                x.hi[d] = boxes[b].hi[d];
            }
            x.sb = make_fab(boxes[b].sborder);
            x.src = make_fab(h ? boxes[b].s_new : boxes[b].s_old);
        }
        int64_t n = 1;
        for (int d = 0; d < 3; ++d) n *= (boxes[b].hi[d] - boxes[b].lo[d] + 1 + 2 * MFG_NGROW);
        maxn = n > maxn ? n : maxn;
    }
    const size_t bytes = fb.size() * sizeof(FillBox);
    if (bytes != g_fill.table.size() || std::memcmp(fb.data(), g_fill.table.data(), bytes) != 0) {
        if (fb.size() > g_fill.bcap) {
            if (g_fill.d_boxes) cudaFree(g_fill.d_boxes);
            g_fill.d_boxes = nullptr;
            if ((e = cudaMalloc(&g_fill.d_boxes, bytes)) != cudaSuccess) return e;
            g_fill.bcap = fb.size();
        }
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        if ((e = cudaMemcpy(g_fill.d_boxes, fb.data(), bytes, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
        g_fill.table.resize(bytes);
        std::memcpy(g_fill.table.data(), fb.data(), bytes);
    }
    const FillBox* tab = g_fill.d_boxes + (s_src ? nbox : 0);
    FillGeom G;
    for (int d = 0; d < 3; ++d) {
        G.dlo[d] = g.domain_lo[d];
        G.dhi[d] = g.domain_hi[d];
        G.per[d] = g.is_periodic[d];
        G.mlen[d] = g_fill.mlen[d];
        G.dx[d] = g.dx[d];
        G.plo[d] = g.prob_lo[d];
    }
    G.gran = g_fill.gran;
    const int nc = NFLO + c_host_params().nspec;
    dim3 grid((unsigned)((maxn + TPB - 1) / TPB), nbox);
    {
        ProfScope ps(K_FILL_COPY, st);
        copy_kernel<<<grid, TPB, 0, st>>>(tab, G, g_fill.d_owner, nc);
    }
    const int ns = c_host_params().nspec;
    for (int s = 1; s <= 3; ++s) {
        // faces, then edges, then corners; at most 65535 slabs per launch
        for (int s0 = 0; s0 < g_fill.nslab[s - 1]; s0 += 65535) {
            const int cnt = std::min(65535, g_fill.nslab[s - 1] - s0);
            const BcSlab* sl = g_fill.d_slabs + g_fill.soff[s - 1] + s0;
            dim3 gb((unsigned)((g_fill.smax[s - 1] + TPB - 1) / TPB), (unsigned)cnt);
            ProfScope ps(K_FILL_BC, st);
            if (ns <= 1) bc_kernel<1><<<gb, TPB, 0, st>>>(tab, sl, G, s, nc);
            else if (ns <= 2) bc_kernel<2><<<gb, TPB, 0, st>>>(tab, sl, G, s, nc);
            else if (ns <= 4) bc_kernel<4><<<gb, TPB, 0, st>>>(tab, sl, G, s, nc);
            else if (ns <= 8) bc_kernel<8><<<gb, TPB, 0, st>>>(tab, sl, G, s, nc);
            else bc_kernel<16><<<gb, TPB, 0, st>>>(tab, sl, G, s, nc);
        }
    }
    return cudaGetLastError();
}

}  // namespace mfg
