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
// so no lane idles on pure fluid or solid cells.  With the cache, a level's
// boxes run in one launch per phase (launch_cutcells_level), box after box so
// that each box's Sborder stays in L2 while its cut cells gather from it.
//
// Cut-cell cache: the list and the weights depend on the volume fraction of
// the grown box only, while the reference recomputes them for every stage of
// every step.  The volume fraction is a state component, so the RK3 algebra
// can move it by an ulp (x 1/3 in stage 3), but the geometry does not change.
// The first call for a box (keyed by its Sborder view and extent) keeps a
// copy of the grown volume fraction and the box's cut cells, sorted by their
// number of fluid neighbours (so the lanes of a warp loop about equally
// often), with each fluid neighbour's offset and weights laid out so that a
// warp's loads of one neighbour entry are contiguous.  Every later call first
// compares the volume fraction with the copy on the device (exact, bit
// patterns): the cut-cell kernel uses the stored entries when nothing
// changed; otherwise it rebuilds the list and recomputes on the fly, so a
// changed geometry is never served stale weights and no host round trip is
// needed.  All paths give bitwise equal results.  Entries whose volume
// fraction changed are dropped by cutcache_sweep (called where the host
// synchronizes anyway) and rebuilt by the next call.
#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

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

// Appends the linear index of every cut cell (0 < vfrac < 1) of the box to
// list; with a non-null flag, only when *flag is set.
__global__ void cut_list_kernel(CutBox c, int* __restrict__ list, unsigned* __restrict__ count,
                                const unsigned* __restrict__ flag) {
    if (flag && !*flag) return;
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

// Grown-box volume fraction: copy (mode 0) or compare with the copy (mode 1,
// sets *dirty on any difference of bit patterns).
__global__ void cut_vf_kernel(Fab S, int lo0, int lo1, int lo2, int l0, int l1, int l2, double* __restrict__ vf,
                              unsigned* __restrict__ dirty, int mode) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool diff = false;
    if (t < (int64_t)l0 * l1 * l2) {
        int i, j, k;
        split3(t, l0, l1, i, j, k);
        const double v = S(lo0 + i, lo1 + j, lo2 + k, VFRAC);
        if (mode == 0)
            vf[t] = v;
        else
            diff = __double_as_longlong(v) != __double_as_longlong(vf[t]);
    }
    if (mode == 1 && __any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(dirty, 1u);
}

__global__ void cut_count_kernel(CutBox c, const int* __restrict__ list, unsigned n, int* __restrict__ kc) {
    const unsigned w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < n) kc[w] = cut_count_one(c, list[w]);
}

__global__ void cut_entries_kernel(CutBox c, CutCacheView cc, unsigned n, int* off, double* wn, double* wd,
                                   double* scal) {
    const unsigned w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < n) cut_entries_one(c, (int)w, cc, off, wn, wd, scal);
}

// Stored entries when the volume fraction is unchanged (*dirty == 0), else
// the on-the-fly form over the freshly built list.  The grid stride is a
// multiple of 32, so a warp always holds one group of 32 list positions.
template <int NS>
__global__ void __launch_bounds__(TPB) cutcell_cached_kernel(CutBox c, CutCacheView cc, unsigned ncut,
                                                             const unsigned* __restrict__ dirty,
                                                             const int* __restrict__ list,
                                                             const unsigned* __restrict__ count) {
    if (*dirty) {
        const unsigned n = *count;
        for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x)
            cutcell_one<NS>(c, list[w]);
        return;
    }
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < ncut; w += gridDim.x * blockDim.x)
        cutcell_cached<NS>(c, (int)w, cc);
}

// ---- all boxes of a level in one launch per phase -------------------------
// One box of the level table: its cut-cell geometry, stored entries, grown
// volume-fraction copy and change flag.
struct LevelCutBox {
    CutBox c;
    CutCacheView v;
    unsigned ncut;
    unsigned* dirty;
    double* vf;
    int glo[3], glen[3];  // grown box
};

// Clears every box's change flag and rebuilt-list count.
__global__ void cut_level_reset_kernel(const LevelCutBox* __restrict__ tab, int nbox, unsigned* __restrict__ cnt) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbox) {
        *tab[b].dirty = 0;
        cnt[b] = 0;
    }
}

// Grown volume fraction against the stored copy (blockIdx.y = box).
__global__ void cut_level_vf_kernel(const LevelCutBox* __restrict__ tab) {
    const LevelCutBox& L = tab[blockIdx.y];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)L.glen[0] * L.glen[1] * L.glen[2];
    bool diff = false;
    if (t < n) {
        int i, j, k;
        split3(t, L.glen[0], L.glen[1], i, j, k);
        const double v = L.c.S(L.glo[0] + i, L.glo[1] + j, L.glo[2] + k, VFRAC);
        diff = __double_as_longlong(v) != __double_as_longlong(L.vf[t]);
    }
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(L.dirty, 1u);
}

// For a box whose volume fraction changed: its cut cells listed afresh
// (grid-stride over the box; one atomic per warp).
__global__ void cut_level_list_kernel(const LevelCutBox* __restrict__ tab, unsigned* __restrict__ cnt,
                                      int* __restrict__ lists, int64_t cap) {
    const LevelCutBox& L = tab[blockIdx.y];
    if (!*L.dirty) return;
    const CutBox& c = L.c;
    int* list = lists + (int64_t)blockIdx.y * cap;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < c.n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = base + threadIdx.x;
        bool cut = false;
        if (t < c.n) {
            int i, j, k;
            cell_of(c, t, i, j, k);
            const double vf = c.S(i, j, k, VFRAC);
            cut = vf > 0.0 && vf < 1.0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, cut);
        if (!m) continue;
        const int lane = threadIdx.x & 31;
        unsigned at = 0;
        if (lane == __ffs(m) - 1) at = atomicAdd(cnt + blockIdx.y, (unsigned)__popc(m));
        at = __shfl_sync(0xffffffffu, at, __ffs(m) - 1);
        if (cut) list[at + __popc(m & ((1u << lane) - 1u))] = (int)t;
    }
}

// Stored entries of every unchanged box: one warp per group of 32 list
// positions, box after box (a box's Sborder stays in L2 while its groups
// run), each box's groups in its own sorted order.
template <int NS>
__global__ void __launch_bounds__(TPB) cutcell_level_kernel(const LevelCutBox* __restrict__ tab,
                                                            const int2* __restrict__ groups, unsigned ngroups) {
    const unsigned gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= ngroups) return;
    const int2 bg = groups[gw];
    const LevelCutBox& L = tab[bg.x];
    if (*L.dirty) return;
    const unsigned w = 32u * (unsigned)bg.y + (threadIdx.x & 31);
    if (w < L.ncut) cutcell_cached<NS>(L.c, (int)w, L.v);
}

// Level tables (drivers alternate levels, so a few are kept), each rebuilt
// when an entry is built or freed (g_cache_gen) or a box descriptor
// changes; the rebuilt-list scratch is shared.
struct CutLevelTable {
    unsigned long long gen = ~0ull, used = 0;
    std::vector<char> key;
    LevelCutBox* d_tab = nullptr;
    int2* d_groups = nullptr;
    size_t tab_cap = 0, grp_cap = 0;
    unsigned ngroups = 0;
    int64_t cap = 0;  // list capacity per box (cells of the largest box)
    int64_t maxgrown = 0;
};
constexpr int kLevelTables = 4;
struct CutLevelCache {
    CutLevelTable t[kLevelTables];
    unsigned long long clock = 0;
    unsigned* d_cnt = nullptr;
    int* d_lists = nullptr;
    size_t cnt_cap = 0, list_cap = 0;
} g_level;

void level_release() {
    for (CutLevelTable& x : g_level.t) {
        cudaFree(x.d_tab);
        cudaFree(x.d_groups);
    }
    cudaFree(g_level.d_cnt);
    cudaFree(g_level.d_lists);
    g_level = CutLevelCache();
}

double g_wdir_dx[3] = {-1.0, -1.0, -1.0};

struct CutEntry {
    int lo[3], hi[3];
    int64_t js, ks, ns;
    double dx[3];
    double* vf = nullptr;
    int* list = nullptr;          // cut cells, sorted by decreasing fluid-neighbour count
    int* kc = nullptr;            // fluid-neighbour count by list position
    int64_t* base = nullptr;      // first entry of each group of 32 list positions
    int* off = nullptr;           // entries: neighbour offset, weights
    double* wn = nullptr;
    double* wd = nullptr;
    double* scal = nullptr;       // 2 per list position
    unsigned ncut = 0;
    int slot = -1;  // index of this entry's flag in g_cache.dirty

    CutCacheView view() const { return {list, kc, base, off, wn, wd, scal}; }
};

// Bumped whenever an entry is built or freed: the level tables below are
// keyed by it.
unsigned long long g_cache_gen = 0;

struct CutCache {
    std::unordered_map<const double*, CutEntry> map;
    unsigned* dirty = nullptr;  // one flag per slot
    unsigned* count = nullptr;  // build scratch
    int nslots = 0, cap = 0;
    std::vector<int> free_slots;
    size_t bytes = 0;
    bool enabled = true;
} g_cache;

void free_entry(CutEntry& e) {
    ++g_cache_gen;
    cudaFree(e.vf);
    cudaFree(e.list);
    cudaFree(e.kc);
    cudaFree(e.base);
    cudaFree(e.off);
    cudaFree(e.wn);
    cudaFree(e.wd);
    cudaFree(e.scal);
    if (e.slot >= 0) g_cache.free_slots.push_back(e.slot);
    e = CutEntry();
}

bool same_key(const CutEntry& e, const mfg_box& b, const Fab& S, const mfg_geom& g) {
    for (int d = 0; d < 3; ++d)
        if (e.lo[d] != b.lo[d] || e.hi[d] != b.hi[d] || e.dx[d] != g.dx[d]) return false;
    return e.js == S.js && e.ks == S.ks && e.ns == S.ns;
}

int new_slot(cudaStream_t st) {
    if (!g_cache.free_slots.empty()) {
        const int s = g_cache.free_slots.back();
        g_cache.free_slots.pop_back();
        return s;
    }
    if (g_cache.nslots == g_cache.cap) {
        const int cap = std::max(256, 2 * g_cache.cap);
        unsigned* d = nullptr;
        if (cudaMalloc(&d, cap * sizeof(unsigned)) != cudaSuccess) return -1;
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        if (g_cache.dirty) {
            cudaMemcpy(d, g_cache.dirty, g_cache.cap * sizeof(unsigned), cudaMemcpyDeviceToDevice);
            cudaFree(g_cache.dirty);
        }
        g_cache.dirty = d;
        g_cache.cap = cap;
    }
    return g_cache.nslots++;
}

// Builds the cache entry of a box from its current Sborder (synchronizes
// twice: for the cut-cell list and for the fluid-neighbour counts, which the
// host sorts).
bool build_entry(const mfg_box& b, const CutBox& c, const mfg_geom& g, CutEntry& e, cudaStream_t st) {
    const int l0 = c.len[0] + 6, l1 = c.len[1] + 6, l2 = c.len[2] + 6;
    const size_t ng = (size_t)l0 * l1 * l2;
    for (int d = 0; d < 3; ++d) {
        e.lo[d] = b.lo[d];
        e.hi[d] = b.hi[d];
        e.dx[d] = g.dx[d];
    }
    e.js = c.S.js;
    e.ks = c.S.ks;
    e.ns = c.S.ns;
    if (!g_cache.count && cudaMalloc(&g_cache.count, sizeof(unsigned)) != cudaSuccess) return false;
    if (cudaMalloc(&e.vf, ng * sizeof(double)) != cudaSuccess) return false;
    if (cudaMalloc(&e.list, std::max<int64_t>(c.n, 1) * sizeof(int)) != cudaSuccess) return false;
    if (cudaMalloc(&e.kc, std::max<int64_t>(c.n, 1) * sizeof(int)) != cudaSuccess) return false;
    cut_vf_kernel<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(c.S, b.lo[0] - 3, b.lo[1] - 3, b.lo[2] - 3, l0, l1,
                                                                 l2, e.vf, nullptr, 0);
    cudaMemsetAsync(g_cache.count, 0, sizeof(unsigned), st);
    cut_list_kernel<<<(unsigned)((c.n + TPB - 1) / TPB), TPB, 0, st>>>(c, e.list, g_cache.count, nullptr);
    if (cudaMemcpyAsync(&e.ncut, g_cache.count, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return false;
    const unsigned n = e.ncut;
    std::vector<int> hl(n), hk(n);
    if (n) {
        cut_count_kernel<<<(n + TPB - 1) / TPB, TPB, 0, st>>>(c, e.list, n, e.kc);
        if (cudaMemcpyAsync(hl.data(), e.list, n * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(hk.data(), e.kc, n * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return false;
    }
    // decreasing count; equal counts keep the cell order (the compaction's
    // order varies between runs, so sort equal counts by cell index)
    std::vector<int> ord(n);
    for (unsigned w = 0; w < n; ++w) ord[w] = (int)w;
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return hk[x] != hk[y] ? hk[x] > hk[y] : hl[x] < hl[y]; });
    std::vector<int> sl(n), sk(n);
    for (unsigned w = 0; w < n; ++w) {
        sl[w] = hl[ord[w]];
        sk[w] = hk[ord[w]];
    }
    const unsigned ngrp = (n + 31) / 32;
    std::vector<int64_t> hb(ngrp + 1, 0);
    for (unsigned gi = 0; gi < ngrp; ++gi) hb[gi + 1] = hb[gi] + 32 * (int64_t)sk[32 * gi];
    const size_t nent = std::max<int64_t>(hb[ngrp], 1);
    const size_t need = nent * (sizeof(int) + 2 * sizeof(double)) + (ngrp + 1) * sizeof(int64_t) +
                        std::max<unsigned>(n, 1) * 2 * sizeof(double);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || need > fr / 4) return false;  // leave room for the caller
    if (cudaMalloc(&e.base, (ngrp + 1) * sizeof(int64_t)) != cudaSuccess) return false;
    if (cudaMalloc(&e.off, nent * sizeof(int)) != cudaSuccess) return false;
    if (cudaMalloc(&e.wn, nent * sizeof(double)) != cudaSuccess) return false;
    if (cudaMalloc(&e.wd, nent * sizeof(double)) != cudaSuccess) return false;
    if (cudaMalloc(&e.scal, std::max<unsigned>(n, 1) * 2 * sizeof(double)) != cudaSuccess) return false;
    if ((e.slot = new_slot(st)) < 0) return false;
    if (n) {
        if (cudaMemcpyAsync(e.list, sl.data(), n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(e.kc, sk.data(), n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(e.base, hb.data(), (ngrp + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
            return false;
        cut_entries_kernel<<<(n + TPB - 1) / TPB, TPB, 0, st>>>(c, e.view(), n, e.off, e.wn, e.wd, e.scal);
        // the host vectors above are read by the copies: wait for them
        if (cudaStreamSynchronize(st) != cudaSuccess) return false;
    }
    g_cache.bytes += ng * sizeof(double) + 2 * c.n * sizeof(int) + need;
    ++g_cache_gen;
    return cudaGetLastError() == cudaSuccess;
}

CutEntry* find_entry(const mfg_box& b, const CutBox& c, const mfg_geom& g, cudaStream_t st) {
    if (!g_cache.enabled) return nullptr;
    auto it = g_cache.map.find(c.S.p);
    if (it != g_cache.map.end()) {
        if (same_key(it->second, b, c.S, g)) return &it->second;
        free_entry(it->second);
        g_cache.map.erase(it);
    }
    CutEntry e;
    if (!build_entry(b, c, g, e, st)) {
        cudaGetLastError();  // an allocation refused here is not an error of the step
        free_entry(e);
        return nullptr;
    }
    return &(g_cache.map[c.S.p] = e);
}

}  // namespace

// Drops the entries whose volume fraction changed in the last call; the host
// has synchronized the stream before.
void cutcache_sweep() {
    if (g_cache.map.empty() || !g_cache.dirty) return;
    std::vector<unsigned> h(g_cache.nslots);
    if (cudaMemcpy(h.data(), g_cache.dirty, h.size() * sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return;
    for (auto it = g_cache.map.begin(); it != g_cache.map.end();) {
        if (it->second.slot >= 0 && h[it->second.slot]) {
            free_entry(it->second);
            it = g_cache.map.erase(it);
        } else {
            ++it;
        }
    }
}

void cutcache_release() {
    level_release();
    for (auto& kv : g_cache.map) free_entry(kv.second);
    g_cache.map.clear();
    cudaFree(g_cache.dirty);
    cudaFree(g_cache.count);
    const bool en = g_cache.enabled;
    g_cache = CutCache();
    g_cache.enabled = en;
}

void cutcache_enable(bool on) {
    if (!on) cutcache_release();
    g_cache.enabled = on;
}

namespace {

CutBox make_cutbox(const mfg_box& b, const mfg_geom& g, double* tcht_scratch) {
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
    return c;
}

// The Dirichlet weight table depends on the cell aspect ratios only (dx /
// dxmin), the same on every level; a new table drops the stored weights.
cudaError_t ensure_wdir(const mfg_geom& g, double dxmin, cudaStream_t st) {
    const double dnk[3] = {g.dx[0] / dxmin, g.dx[1] / dxmin, g.dx[2] / dxmin};
    if (dnk[0] == g_wdir_dx[0] && dnk[1] == g_wdir_dx[1] && dnk[2] == g_wdir_dx[2]) return cudaSuccess;
    // Dirichlet weights: 1/((l dx_nd)^2 + (m dy_nd)^2 + (n dz_nd)^2 + 1e-40), centre unused
    double w[SW * SW * SW];
    for (int n = -SG; n <= SG; ++n)
        for (int m = -SG; m <= SG; ++m)
            for (int l = -SG; l <= SG; ++l) {
                const double a = l * dnk[0], bb = m * dnk[1], e = n * dnk[2];
                const double d2 = (a * a + bb * bb) + e * e;
                w[(l + SG) + SW * ((m + SG) + SW * (n + SG))] = (l == 0 && m == 0 && n == 0) ? 0.0 : 1.0 / (d2 + kTiny2);
            }
    cudaError_t e = cudaMemcpyToSymbolAsync(c_wdir, w, sizeof(w), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    cudaStreamSynchronize(st);
    for (int d = 0; d < 3; ++d) g_wdir_dx[d] = dnk[d];
    cutcache_release();  // stored weights used the previous table
    return cudaSuccess;
}

template <class T>
bool grow_buf(T*& p, size_t& have, size_t want) {
    if (want <= have) return true;
    cudaFree(p);
    p = nullptr;
    have = 0;
    if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess) return false;
    have = want;
    return true;
}

// The table of this box layout, built (synchronizing) when missing; null when
// it would have to be built during stream capture or memory is short.
CutLevelTable* level_prepare(const std::vector<LevelCutBox>& tab) {
    const size_t bytes = tab.size() * sizeof(LevelCutBox);
    ++g_level.clock;
    for (CutLevelTable& x : g_level.t)
        if (x.gen == g_cache_gen && x.key.size() == bytes && std::memcmp(x.key.data(), tab.data(), bytes) == 0) {
            x.used = g_level.clock;
            return &x;
        }
    // the table and scratch about to be replaced may be read by kernels of an
    // earlier call, on any stream
    if (cudaDeviceSynchronize() != cudaSuccess) return nullptr;
    CutLevelTable* T = &g_level.t[0];
    for (CutLevelTable& x : g_level.t)
        if (x.used < T->used) T = &x;
    const int nbox = (int)tab.size();
    std::vector<int2> groups;
    int64_t cap = 1, maxgrown = 1;
    for (int b = 0; b < nbox; ++b) {
        const unsigned ng = (tab[b].ncut + 31) / 32;
        for (unsigned q = 0; q < ng; ++q) groups.push_back(make_int2(b, (int)q));
        cap = std::max<int64_t>(cap, tab[b].c.n);
        maxgrown = std::max<int64_t>(maxgrown, (int64_t)tab[b].glen[0] * tab[b].glen[1] * tab[b].glen[2]);
    }
    T->gen = ~0ull;  // invalid until filled
    if (!grow_buf(T->d_tab, T->tab_cap, tab.size())) return nullptr;
    if (!grow_buf(T->d_groups, T->grp_cap, std::max<size_t>(groups.size(), 1))) return nullptr;
    if (!grow_buf(g_level.d_cnt, g_level.cnt_cap, tab.size())) return nullptr;
    if (!grow_buf(g_level.d_lists, g_level.list_cap, (size_t)cap * nbox)) return nullptr;
    if (cudaMemcpy(T->d_tab, tab.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    if (!groups.empty() &&
        cudaMemcpy(T->d_groups, groups.data(), groups.size() * sizeof(int2), cudaMemcpyHostToDevice) != cudaSuccess)
        return nullptr;
    T->ngroups = (unsigned)groups.size();
    T->cap = cap;
    T->maxgrown = maxgrown;
    T->key.assign(reinterpret_cast<const char*>(tab.data()), reinterpret_cast<const char*>(tab.data()) + bytes);
    T->gen = g_cache_gen;
    T->used = g_level.clock;
    return T;
}

}  // namespace

// All boxes of a level in four launches (change flags cleared, volume
// fractions checked, lists of changed boxes rebuilt, stored entries applied)
// plus one on-the-fly launch per box that does work only where the box's
// volume fraction changed (the cache-off kernel itself, so those boxes give
// that path's results by construction).  Returns 1 when done, -1 on a CUDA
// error, and 0, having launched nothing, where the per-box path must run:
// cache off, conjugate heat transfer (its neighbour-temperature scratch is
// per box), a box without an entry, or a table to build during capture.
int launch_cutcells_level(const mfg_box* boxes, int nbox, const mfg_geom& g, cudaStream_t st) {
    if (nbox < 2 || !g_cache.enabled || c_host_params().conj_ht) return 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return 0;
    const double dxmin = fmin(g.dx[0], fmin(g.dx[1], g.dx[2]));
    if (ensure_wdir(g, dxmin, st) != cudaSuccess) return -1;
    std::vector<LevelCutBox> tab(nbox);
    std::vector<int> slots(nbox);
    for (int b = 0; b < nbox; ++b) {
        LevelCutBox& L = tab[b];
        memset(&L, 0, sizeof(L));
        L.c = make_cutbox(boxes[b], g, nullptr);
        CutEntry* ce = find_entry(boxes[b], L.c, g, st);
        if (!ce) return 0;
        slots[b] = ce->slot;
        L.v = ce->view();
        L.ncut = ce->ncut;
        L.vf = ce->vf;
        for (int d = 0; d < 3; ++d) {
            L.glo[d] = boxes[b].lo[d] - 3;
            L.glen[d] = L.c.len[d] + 6;
        }
    }
    // find_entry may have grown the flag array: flag pointers last
    for (int b = 0; b < nbox; ++b) tab[b].dirty = g_cache.dirty + slots[b];
    CutLevelTable* T = level_prepare(tab);
    if (!T) {
        cudaGetLastError();  // an allocation refused here is not an error of the step
        return 0;
    }
    const int ns = c_host_params().nspec;
    ProfScope ps(K_CUT, st, 4 + nbox);
    cut_level_reset_kernel<<<(nbox + 127) / 128, 128, 0, st>>>(T->d_tab, nbox, g_level.d_cnt);
    cut_level_vf_kernel<<<dim3((unsigned)((T->maxgrown + 255) / 256), (unsigned)nbox), 256, 0, st>>>(T->d_tab);
    cut_level_list_kernel<<<dim3(8, (unsigned)nbox), TPB, 0, st>>>(T->d_tab, g_level.d_cnt, g_level.d_lists, T->cap);
    const unsigned nb = std::max(1u, (unsigned)(((uint64_t)T->ngroups * 32 + TPB - 1) / TPB));
#define MFG_LEVEL_LAUNCH(K)                                                                                 \
    do {                                                                                                    \
        cutcell_level_kernel<K><<<nb, TPB, 0, st>>>(T->d_tab, T->d_groups, T->ngroups);                   \
        for (int b = 0; b < nbox; ++b)                                                                      \
            cutcell_kernel<K><<<152, TPB, 0, st>>>(tab[b].c, g_level.d_lists + (int64_t)b * T->cap,         \
                                                   g_level.d_cnt + b);                                      \
    } while (0)
    if (ns <= 1) MFG_LEVEL_LAUNCH(1);
    else if (ns <= 2) MFG_LEVEL_LAUNCH(2);
    else if (ns <= 4) MFG_LEVEL_LAUNCH(4);
    else if (ns <= 8) MFG_LEVEL_LAUNCH(8);
    else MFG_LEVEL_LAUNCH(16);
#undef MFG_LEVEL_LAUNCH
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

cudaError_t launch_cutcells_box(const mfg_box& b, const mfg_geom& g, double* tcht_scratch, int* list,
                                unsigned* count, cudaStream_t st) {
    CutBox c = make_cutbox(b, g, tcht_scratch);
    cudaError_t we = ensure_wdir(g, c.dxmin, st);
    if (we != cudaSuccess) return we;
    const unsigned nb = (unsigned)((c.n + TPB - 1) / TPB);
    const int ns = c_host_params().nspec;
    CutEntry* ce = find_entry(b, c, g, st);
    ProfScope ps(K_CUT, st, (ce ? 3 : 2) + (c_host_params().conj_ht ? 1 : 0));
    if (c_host_params().conj_ht) cht_avg_kernel<<<nb, TPB, 0, st>>>(c);
    cudaMemsetAsync(count, 0, sizeof(unsigned), st);
    if (ce) {
        unsigned* dirty = g_cache.dirty + ce->slot;
        const int l0 = c.len[0] + 6, l1 = c.len[1] + 6, l2 = c.len[2] + 6;
        const int64_t ngc = (int64_t)l0 * l1 * l2;
        cudaMemsetAsync(dirty, 0, sizeof(unsigned), st);
        cut_vf_kernel<<<(unsigned)((ngc + 255) / 256), 256, 0, st>>>(c.S, b.lo[0] - 3, b.lo[1] - 3, b.lo[2] - 3, l0,
                                                                      l1, l2, ce->vf, dirty, 1);
        cut_list_kernel<<<nb, TPB, 0, st>>>(c, list, count, dirty);
        const unsigned ng = (unsigned)std::min<int64_t>(std::max<int64_t>(nb, 1), 152 * 8);
#define MFG_CUT_ARGS c, ce->view(), ce->ncut, dirty, list, count
        if (ns <= 1) cutcell_cached_kernel<1><<<ng, TPB, 0, st>>>(MFG_CUT_ARGS);
        else if (ns <= 2) cutcell_cached_kernel<2><<<ng, TPB, 0, st>>>(MFG_CUT_ARGS);
        else if (ns <= 4) cutcell_cached_kernel<4><<<ng, TPB, 0, st>>>(MFG_CUT_ARGS);
        else if (ns <= 8) cutcell_cached_kernel<8><<<ng, TPB, 0, st>>>(MFG_CUT_ARGS);
        else cutcell_cached_kernel<16><<<ng, TPB, 0, st>>>(MFG_CUT_ARGS);
#undef MFG_CUT_ARGS
        return cudaGetLastError();
    }
    cut_list_kernel<<<nb, TPB, 0, st>>>(c, list, count, nullptr);
    // a fixed grid walks the list (its length stays on the device)
    const unsigned ng = (unsigned)std::min<int64_t>(nb, 152 * 8);
    if (ns <= 1) cutcell_kernel<1><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 2) cutcell_kernel<2><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 4) cutcell_kernel<4><<<ng, TPB, 0, st>>>(c, list, count);
    else if (ns <= 8) cutcell_kernel<8><<<ng, TPB, 0, st>>>(c, list, count);
    else cutcell_kernel<16><<<ng, TPB, 0, st>>>(c, list, count);
    return cudaGetLastError();
}

}  // namespace mfg
