// C ABI entry points (include/mflo_gpu.h): parameter upload, validation,
// library-owned scratch, per-box launches and the single-level step driver.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "mfg_internal.h"

namespace mfg {

cudaError_t launch_cutcells_box(const mfg_box& b, const mfg_geom& g, double* tcht_scratch, int* list,
                                unsigned* count, cudaStream_t st);
cudaError_t launch_chem_substep(const mfg_box& b, double dt, cudaStream_t st);
cudaError_t launch_resnorm_box(const mfg_box& b, double dt, double* partial, double* acc, cudaStream_t st);
void fill_release();

namespace {

DevParams g_hp;
// chemistry integrator settings (mfg_set_chem_integrator), kept across mfg_init
struct ChemSettings {
    int kind = 0, maxsub = 1000;
    double rtol = 1e-8, atol = 1e-12;
} g_chem;
bool g_ready = false;
bool g_fast_weno = true;

// Library-owned scratch: one growable device buffer.
struct Pool {
    char* p = nullptr;
    size_t cap = 0;
} g_pool;

cudaError_t pool_reserve(size_t bytes, cudaStream_t st) {
    if (bytes <= g_pool.cap) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (g_pool.p) cudaFree(g_pool.p);
    g_pool.p = nullptr;
    g_pool.cap = 0;
    size_t want = bytes + bytes / 8;
    if ((e = cudaMalloc(&g_pool.p, want)) != cudaSuccess) return e;
    g_pool.cap = want;
    return cudaSuccess;
}

// Copy stream and event of the host-buffer level step, created on first use
// for the device current then (re-created if the current device changed).
struct CopyStream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    int dev = -1;
} g_copy;

void copy_stream_release() {
    if (g_copy.s) cudaStreamDestroy(g_copy.s);
    if (g_copy.ev) cudaEventDestroy(g_copy.ev);
    g_copy = CopyStream();
}

cudaError_t copy_stream(cudaStream_t* s, cudaEvent_t* ev) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!g_copy.s || g_copy.dev != dev) {
        copy_stream_release();
        if ((e = cudaStreamCreateWithFlags(&g_copy.s, cudaStreamNonBlocking)) != cudaSuccess) return e;
        if ((e = cudaEventCreateWithFlags(&g_copy.ev, cudaEventDisableTiming)) != cudaSuccess) return e;
        g_copy.dev = dev;
    }
    *s = g_copy.s;
    *ev = g_copy.ev;
    return cudaSuccess;
}

// Doubles from a view's first element to its last (the memory one copy of
// the whole view moves).
size_t view_span_doubles(const mfg_array4& a) {
    return (size_t)((int64_t)(a.ncomp - 1) * a.nstride + (int64_t)(a.end[2] - a.begin[2] - 1) * a.kstride +
                    (int64_t)(a.end[1] - a.begin[1] - 1) * a.jstride + (a.end[0] - a.begin[0]));
}

bool same_layout(const mfg_array4& h, const mfg_array4& d) {
    if (!h.p || h.jstride != d.jstride || h.kstride != d.kstride || h.nstride != d.nstride || h.ncomp != d.ncomp)
        return false;
    for (int e = 0; e < 3; ++e)
        if (h.begin[e] != d.begin[e] || h.end[e] != d.end[e]) return false;
    return true;
}

int ncomp_total() { return NFLO + g_hp.nspec; }
int ncomp_adv() { return NCONS + g_hp.nspec; }

bool covers(const mfg_array4& a, const int lo[3], const int hi[3], int ncomp) {
    if (!a.p) return false;
    for (int d = 0; d < 3; ++d)
        if (a.begin[d] > lo[d] || a.end[d] < hi[d] + 1) return false;
    return a.ncomp >= ncomp;
}

int check_boxes(const mfg_box* boxes, int nbox, bool need_sb, bool need_dsdt, bool need_old, bool need_new) {
    if (!g_ready) return MFG_ERR_STATE;
    if (nbox < 0 || (nbox > 0 && !boxes)) return MFG_ERR_ARG;
    const int N = ncomp_total();
    for (int b = 0; b < nbox; ++b) {
        const mfg_box& x = boxes[b];
        for (int d = 0; d < 3; ++d)
            if (x.hi[d] < x.lo[d]) return MFG_ERR_ARG;
        int glo[3], ghi[3];
        for (int d = 0; d < 3; ++d) {
            glo[d] = x.lo[d] - MFG_NGROW;
            ghi[d] = x.hi[d] + MFG_NGROW;
        }
        if (need_sb && !covers(x.sborder, glo, ghi, N)) return MFG_ERR_ARG;
        if (need_dsdt && !covers(x.dsdt, x.lo, x.hi, N)) return MFG_ERR_ARG;
        if (need_old && !covers(x.s_old, x.lo, x.hi, N)) return MFG_ERR_ARG;
        if (need_new && !covers(x.s_new, x.lo, x.hi, N)) return MFG_ERR_ARG;
        for (int d = 0; d < 3; ++d) {
            if (!x.flux[d].p) continue;
            int fhi[3] = {x.hi[0], x.hi[1], x.hi[2]};
            fhi[d] += 1;
            if (!covers(x.flux[d], x.lo, fhi, N)) return MFG_ERR_ARG;
        }
    }
    return MFG_OK;
}

char g_last_error[256] = "";

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return MFG_OK;
    note_cuda_error(e, "fill patch");
    return MFG_ERR_CUDA;
}

size_t rhs_scratch_doubles(const int n[3]) {
    size_t s = aux_doubles(n);
    for (int d = 0; d < 3; ++d) s += face_doubles(n, d, NFS) + face_doubles(n, d, ncomp_adv());
    return s + face_list_doubles(n);
}

// Lay out one box's RHS scratch at base.
RhsBox make_rhs_box(const mfg_box& b, const mfg_geom& g, double* base) {
    RhsBox B;
    memset(&B, 0, sizeof(B));
    int n[3];
    for (int d = 0; d < 3; ++d) {
        B.lo[d] = b.lo[d];
        B.hi[d] = b.hi[d];
        B.dx[d] = g.dx[d];
        B.idx[d] = 1.0 / g.dx[d];
        n[d] = b.hi[d] - b.lo[d] + 1;
    }
    B.sb = make_fab(b.sborder);
    B.dsdt = make_fab(b.dsdt);
    B.sold = make_fab(b.s_old);
    B.snew = make_fab(b.s_new);
    for (int d = 0; d < 3; ++d) B.uflux[d] = make_fab(b.flux[d]);
    double* p = base;
    {
        int lo[3] = {b.lo[0] - 3, b.lo[1] - 3, b.lo[2] - 3}, len[3] = {n[0] + 6, n[1] + 6, n[2] + 6};
        B.aux = dense_fab(p, lo, len);
        p += aux_doubles(n);
    }
    for (int d = 0; d < 3; ++d) {
        int len[3] = {n[0] + (d == 0), n[1] + (d == 1), n[2] + (d == 2)};
        B.fs[d] = dense_fab(p, b.lo, len);
        p += face_doubles(n, d, NFS);
        B.flx[d] = dense_fab(p, b.lo, len);
        p += face_doubles(n, d, ncomp_adv());
    }
    B.fcount = reinterpret_cast<unsigned*>(p);
    B.flist = reinterpret_cast<int*>(p) + 4;
    return B;
}

int run_rhs(const mfg_box* boxes, int nbox, const mfg_geom* geom, int stage, double dt, cudaStream_t st) {
    size_t need = 0;
    for (int b = 0; b < nbox; ++b) {
        int n[3];
        for (int d = 0; d < 3; ++d) n[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
        need = std::max(need, rhs_scratch_doubles(n));
    }
    cudaError_t e = pool_reserve(need * sizeof(double), st);
    if (e != cudaSuccess) return MFG_ERR_CUDA;
    for (int b = 0; b < nbox; ++b) {
        RhsBox B = make_rhs_box(boxes[b], *geom, reinterpret_cast<double*>(g_pool.p));
        if ((e = launch_rhs_box(B, stage, dt, g_fast_weno, st)) != cudaSuccess) return MFG_ERR_CUDA;
    }
    return MFG_OK;
}

}  // namespace

const DevParams& c_host_params() { return g_hp; }

void note_cuda_error(cudaError_t e, const char* where) {
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%d)", where, cudaGetErrorString(e), (int)e);
}

// Shared with the allocation-free entry point (mfg_noalloc.cu).
int validate_boxes(const mfg_box* boxes, int nbox, bool need_sb, bool need_dsdt, bool need_old, bool need_new) {
    return check_boxes(boxes, nbox, need_sb, need_dsdt, need_old, need_new);
}
size_t rhs_box_scratch_doubles(const int n[3]) { return rhs_scratch_doubles(n); }
RhsBox layout_rhs_box(const mfg_box& b, const mfg_geom& g, double* base) { return make_rhs_box(b, g, base); }
bool weno_fast_mode() { return g_fast_weno; }

}  // namespace mfg

using namespace mfg;

extern "C" {

const char* mfg_version(void) { return "mesoflow-gb300 0.1 (sm_103a, FP64)"; }

const char* mfg_last_error(void) { return g_last_error; }

int mfg_init(const mfg_params* p) {
    if (!p) return MFG_ERR_ARG;
    if (p->nspec < 1 || p->nspec > MFG_MAX_SPECIES) return MFG_ERR_ARG;
    if (p->ngas < 0 || p->ngas > p->nspec) return MFG_ERR_ARG;
    if (p->thermo_kind < MFG_THERMO_MOLAR || p->thermo_kind > MFG_THERMO_BG_GAS) return MFG_ERR_ARG;
    if (p->thermo_kind != MFG_THERMO_MASS_SINGLE && p->ngas < 1) return MFG_ERR_ARG;
    if (!(p->order_hyp == 1 || p->order_hyp == 2 || p->order_hyp == 4 || p->order_hyp == 5)) return MFG_ERR_SCHEME;
    if (p->nreact < 0 || p->nreact > MFG_MAX_REACTIONS) return MFG_ERR_ARG;
    for (int d = 0; d < 3; ++d) {
        const int k[2] = {p->bc_lo[d], p->bc_hi[d]};
        for (int s = 0; s < 2; ++s)
            if (!(k[s] == MFG_BC_INT_DIR || k[s] == MFG_BC_FOEXTRAP || k[s] == MFG_BC_EXT_DIR || k[s] == MFG_BC_WALL))
                return MFG_ERR_ARG;
    }
    DevParams h;
    memset(&h, 0, sizeof(h));
    h.nspec = p->nspec;
    h.ngas = p->ngas;
    h.thermo_kind = p->thermo_kind;
    h.energy_form = p->energy_form;
    h.R_univ = p->R_univ;
    h.gas_R = p->gas_R;
    h.gamma_single = p->gamma_single;
    h.bg_molwt = p->bg_molwt;
    const double R = (p->thermo_kind == MFG_THERMO_BG_GAS) ? kRU : p->R_univ;
    for (int s = 0; s < MFG_MAX_SPECIES; ++s) {
        h.molwt[s] = p->molwt[s];
        h.advect_flag[s] = p->advect_flag[s];
        h.diff_mode[s] = p->diff_mode[s];
        h.diff_gas[s] = p->diff_gas[s];
        h.diff_solid[s] = p->diff_solid[s];
    }
    for (int s = 0; s <= MFG_MAX_SPECIES; ++s) h.gamma[s] = p->gamma[s];
    for (int s = 0; s <= p->ngas && s <= MFG_MAX_SPECIES; ++s) {
        if (s == p->ngas && p->thermo_kind != MFG_THERMO_BG_GAS) break;
        h.cv[s] = R / (p->gamma[s] - 1.0);
        h.igm1[s] = 1.0 / (p->gamma[s] - 1.0);
        if (s < p->ngas && p->molwt[s] != 0.0) h.cvmass[s] = R / (p->gamma[s] - 1.0) / p->molwt[s];
    }
    auto hmean = [](double d1, double d2) { return 2.0 * d1 * d2 / (d1 + d2 + 1e-30); };
    h.visc_hm = hmean(p->visc_gas, p->visc_gas);
    h.cond_hm = hmean(p->cond_gas, p->cond_gas);
    for (int s = 0; s < MFG_MAX_SPECIES; ++s) h.diff_hm[s] = hmean(p->diff_gas[s], p->diff_gas[s]);
    if (p->thermo_kind == MFG_THERMO_MASS_SINGLE) {
        h.g_gm1 = p->gamma_single / (p->gamma_single - 1.0);
        h.astar_fac = (2.0 * (p->gamma_single - 1.0)) / (p->gamma_single + 1.0);
        h.gm1_single = p->gamma_single - 1.0;
        h.inv_gas_R = 1.0 / p->gas_R;
    }
    h.visc_mode = p->visc_mode;
    h.cond_mode = p->cond_mode;
    h.visc_gas = p->visc_gas;
    h.visc_solid = p->visc_solid;
    h.cond_gas = p->cond_gas;
    h.cond_solid = p->cond_solid;
    h.order_hyp = p->order_hyp;
    h.do_ns = p->do_ns;
    h.species_in_solid = p->species_in_solid;
    h.conj_ht = p->conj_ht;
    h.dissfactor = p->dissfactor;
    h.solid_temp = p->solid_temp;
    h.cfl = p->cfl;
    h.chem_on = p->chem_on;
    h.nreact = p->nreact;
    for (int r = 0; r < MFG_MAX_REACTIONS; ++r) {
        h.A[r] = p->A[r];
        h.Ea[r] = p->Ea[r];
        for (int s = 0; s < MFG_MAX_SPECIES; ++s) {
            h.nu[r][s] = p->nu[r][s];
            h.order[r][s] = p->order[r][s];
            if (s < p->nspec && p->order[r][s] > 0.0) h.ord_mask[r] |= 1u << s;
            if (s < p->nspec && std::fabs(p->nu[r][s]) > 0.0) h.nu_mask[r] |= 1u << s;
        }
    }
    for (int d = 0; d < 3; ++d) {
        h.bc_lo[d] = p->bc_lo[d];
        h.bc_hi[d] = p->bc_hi[d];
        h.ext_lo[d] = p->ext_lo[d];
        h.ext_hi[d] = p->ext_hi[d];
    }
    h.chem_kind = g_chem.kind;
    h.chem_maxsub = g_chem.maxsub;
    h.chem_rtol = g_chem.rtol;
    h.chem_atol = g_chem.atol;
    if (upload_params(h) != cudaSuccess) return MFG_ERR_CUDA;
    g_hp = h;
    g_ready = true;
    return MFG_OK;
}

int mfg_set_chem_integrator(int kind, double rtol, double atol, int max_substeps) {
    if (kind < 0 || kind > 1 || !(rtol > 0.0) || !(atol > 0.0) || max_substeps < 1) return MFG_ERR_ARG;
    g_chem.kind = kind;
    g_chem.rtol = rtol;
    g_chem.atol = atol;
    g_chem.maxsub = max_substeps;
    if (!g_ready) return MFG_OK;
    g_hp.chem_kind = kind;
    g_hp.chem_rtol = rtol;
    g_hp.chem_atol = atol;
    g_hp.chem_maxsub = max_substeps;
    return upload_params(g_hp) == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

int mfg_finalize(void) {
    if (g_pool.p) cudaFree(g_pool.p);
    g_pool = Pool();
    fill_release();
    cutcache_release();
    noalloc_forget();
    copy_stream_release();
    g_ready = false;
    return MFG_OK;
}

int mfg_status(uint32_t* flags, int clear) {
    if (!flags) return MFG_ERR_ARG;
    if (cudaDeviceSynchronize() != cudaSuccess) return MFG_ERR_CUDA;
    unsigned v = 0;
    if (read_status(&v, clear != 0) != cudaSuccess) return MFG_ERR_CUDA;
    *flags = v;
    return MFG_OK;
}

int mfg_set_weno_mode(int fast) {
    g_fast_weno = fast != 0;
    return MFG_OK;
}

int mfg_fill_patch(const mfg_box* boxes, int nbox, const mfg_geom* geom, int s_src, double time, void* stream) {
    int rc = check_boxes(boxes, nbox, true, false, s_src == 0, s_src != 0);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    if (nbox == 0) return MFG_OK;
    return cuda_rc(launch_fill_patch(boxes, nbox, *geom, s_src, time, (cudaStream_t)stream));
}

int mfg_cutcells(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, void* stream) {
    (void)time;
    int rc = check_boxes(boxes, nbox, true, false, false, false);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int lv = launch_cutcells_level(boxes, nbox, *geom, st);
    if (lv < 0) return MFG_ERR_CUDA;
    if (lv > 0) return MFG_OK;
    size_t need = 0;
    for (int b = 0; b < nbox; ++b) {
        size_t n = 1;
        for (int d = 0; d < 3; ++d) n *= (size_t)(boxes[b].hi[d] - boxes[b].lo[d] + 1);
        need = std::max(need, n);
    }
    // scratch: [count | cut-cell list | CHT temperatures]
    const size_t list_bytes = ((need * sizeof(int) + 255) / 256) * 256;
    if (pool_reserve(256 + list_bytes + need * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
    unsigned* count = reinterpret_cast<unsigned*>(g_pool.p);
    int* list = reinterpret_cast<int*>(g_pool.p + 256);
    double* tcht = reinterpret_cast<double*>(g_pool.p + 256 + list_bytes);
    for (int b = 0; b < nbox; ++b)
        if (launch_cutcells_box(boxes[b], *geom, tcht, list, count, st) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_compute_dsdt_flow(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double dt,
                          void* stream) {
    (void)time;
    int rc = check_boxes(boxes, nbox, true, true, false, false);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    return run_rhs(boxes, nbox, geom, 0, dt, (cudaStream_t)stream);
}

int mfg_rk3_stage(const mfg_box* boxes, int nbox, const mfg_geom* geom, int stage, double time, double dt,
                  void* stream) {
    (void)time;
    if (stage < 1 || stage > 3) return MFG_ERR_ARG;
    int rc = check_boxes(boxes, nbox, true, false, stage > 1, true);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    return run_rhs(boxes, nbox, geom, stage, dt, (cudaStream_t)stream);
}

int mfg_chem_source(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, void* stream) {
    (void)time;
    (void)geom;
    int rc = check_boxes(boxes, nbox, false, true, false, true);
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (launch_chem_source(boxes[b], (cudaStream_t)stream) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_chem_substep(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double dt, void* stream) {
    (void)time;
    (void)geom;
    int rc = check_boxes(boxes, nbox, false, false, true, true);
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (launch_chem_substep(boxes[b], dt, (cudaStream_t)stream) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_update_primitive_vars(const mfg_box* boxes, int nbox, const mfg_geom* geom, void* stream) {
    (void)geom;
    int rc = check_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned before = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess || read_status(&before, false) != cudaSuccess) return MFG_ERR_CUDA;
    for (int b = 0; b < nbox; ++b)
        if (launch_update_prims(boxes[b], nullptr, st) != cudaSuccess) return MFG_ERR_CUDA;
    unsigned after = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess || read_status(&after, false) != cudaSuccess) return MFG_ERR_CUDA;
    return (after & MFG_STATUS_NEG_PRESSURE) ? MFG_ERR_NEG_PRESSURE : MFG_OK;
}

int mfg_chem_advance_rk2(const mfg_box* boxes, int nbox, double time, double dt, void* stream) {
    (void)time;
    int rc = check_boxes(boxes, nbox, false, false, true, true);
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (launch_split_chem(boxes[b], 0, dt, 0, (cudaStream_t)stream) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_store_inertgas_conc(const mfg_box* boxes, int nbox, void* stream) {
    int rc = check_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (launch_split_chem(boxes[b], 1, 0.0, 0, (cudaStream_t)stream) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_update_vars_after_chemsolve(const mfg_box* boxes, int nbox, int using_bg_inertgas, void* stream) {
    int rc = check_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    for (int b = 0; b < nbox; ++b)
        if (launch_split_chem(boxes[b], 2, 0.0, using_bg_inertgas, st) != cudaSuccess) return MFG_ERR_CUDA;
    unsigned after = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess || read_status(&after, false) != cudaSuccess) return MFG_ERR_CUDA;
    return (after & MFG_STATUS_NEG_PRESSURE) ? MFG_ERR_NEG_PRESSURE : MFG_OK;
}

int mfg_clip_species(const mfg_box* boxes, int nbox, void* stream) {
    int rc = check_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (launch_clip_species(boxes[b], (cudaStream_t)stream) != cudaSuccess) return MFG_ERR_CUDA;
    return MFG_OK;
}

int mfg_residual_norms(const mfg_box* boxes, int nbox, double dt, double* out, void* stream) {
    int rc = check_boxes(boxes, nbox, false, false, true, true);
    if (rc) return rc;
    if (!out || !(dt != 0.0)) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = ncomp_total();
    const size_t partial = (size_t)N * 1024;
    if (pool_reserve((partial + N) * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
    double* part = reinterpret_cast<double*>(g_pool.p);
    double* acc = part + partial;
    if (cudaMemsetAsync(acc, 0, N * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
    for (int b = 0; b < nbox; ++b)
        if (launch_resnorm_box(boxes[b], dt, part, acc, st) != cudaSuccess) return MFG_ERR_CUDA;
    std::vector<double> h(N);
    if (cudaMemcpyAsync(h.data(), acc, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MFG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MFG_ERR_CUDA;
    for (int n = 0; n < N; ++n) out[n] = std::sqrt(h[n]);
    return MFG_OK;
}

int mfg_est_timestep(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double* dt_out,
                     void* stream) {
    (void)time;
    int rc = check_boxes(boxes, nbox, false, false, false, true);
    if (rc) return rc;
    if (!geom || !dt_out) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (pool_reserve(2 * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
    double* acc = reinterpret_cast<double*>(g_pool.p);
    if (cudaMemsetAsync(acc, 0, 2 * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
    for (int b = 0; b < nbox; ++b)
        if (launch_timestep(boxes[b], acc, st) != cudaSuccess) return MFG_ERR_CUDA;
    double h[2];
    if (cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MFG_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MFG_ERR_CUDA;
    double dt_est = 1.7976931348623157e308;
    if (h[0] > 0)
        for (int d = 0; d < 3; ++d) dt_est = std::min(dt_est, geom->dx[d] / h[0]);
    if (h[1] > 0)
        for (int d = 0; d < 3; ++d) dt_est = std::min(dt_est, 0.5 * geom->dx[d] * geom->dx[d] / h[1] / 3);
    *dt_out = dt_est * g_hp.cfl;
    return MFG_OK;
}

// One coarse step of a single level: the swap, three RK3 stages (fill patch,
// cut cells, fused RHS + stage algebra), the Strang chemistry sub-step, the
// primitive refresh, species clipping and residual norms
// (Source/mflo_evolve.cpp:251-318, 470-493, 33-58).  The bookends of box b
// run right after its stage-3 update (the box's state is still in L2, and no
// other box's stage 3 reads it: every box reads its own filled Sborder), in
// box order, so the residual-norm sums run in the same order as a separate
// pass.  With h_state, each box's phi_new is copied in from the host first and
// copied back on the copy stream as soon as its bookends are done.
static int advance_level(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double dt,
                         int only_flow, int clip, double* resnorms, const mfg_array4* h_state, cudaStream_t st) {
    int rc;
    const int N = ncomp_total();
    size_t need = 0;
    for (int b = 0; b < nbox; ++b) {
        int n[3];
        for (int d = 0; d < 3; ++d) n[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
        need = std::max(need, rhs_scratch_doubles(n));
    }
    const size_t npart = (size_t)N * 1024;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    // every return after copies were queued on the copy stream first makes
    // the caller's stream wait for them (the host views stay in use until then)
    struct Join {
        cudaStream_t cs = nullptr, st = nullptr;
        cudaEvent_t ev = nullptr;
        ~Join() {
            if (cs && cudaEventRecord(ev, cs) == cudaSuccess) cudaStreamWaitEvent(st, ev, 0);
        }
    } join;
    if (h_state) {
        if (copy_stream(&cs, &ev) != cudaSuccess) return MFG_ERR_CUDA;
        join.cs = cs;
        join.st = st;
        join.ev = ev;
        for (int b = 0; b < nbox; ++b)
            if (cudaMemcpyAsync(boxes[b].s_new.p, h_state[b].p, view_span_doubles(boxes[b].s_new) * sizeof(double),
                                cudaMemcpyHostToDevice, st) != cudaSuccess)
                return MFG_ERR_CUDA;
    }
    Fab none;
    memset(&none, 0, sizeof(none));
    for (int b = 0; b < nbox; ++b)  // phi_old <- phi_new (std::swap of the reference)
        if (launch_axpy_valid(boxes[b], make_fab(boxes[b].s_old), none, 0.0, true, make_fab(boxes[b].s_new), N, st) !=
            cudaSuccess)
            return MFG_ERR_CUDA;
    double* acc = nullptr;
    for (int stage = 1; stage <= 3; ++stage) {
        if ((rc = mfg_fill_patch(boxes, nbox, geom, stage == 1 ? 0 : 1, stage == 1 ? time : time + dt, st)))
            return rc;
        if ((rc = mfg_cutcells(boxes, nbox, geom, time, st))) return rc;
        // the pool after the cut-cell pass (whose per-box form uses it too):
        // RHS scratch first, then the residual-norm partials and sums, which
        // must survive the later boxes' RHS launches of stage 3
        if (pool_reserve((need + npart + N) * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
        double* scratch = reinterpret_cast<double*>(g_pool.p);
        double* part = (resnorms && stage == 3) ? scratch + need : nullptr;
        acc = part ? part + npart : nullptr;
        if (acc && cudaMemsetAsync(acc, 0, N * sizeof(double), st) != cudaSuccess) return MFG_ERR_CUDA;
        for (int b = 0; b < nbox; ++b) {
            RhsBox B = make_rhs_box(boxes[b], *geom, scratch);
            if (launch_rhs_box(B, stage, dt, g_fast_weno, st) != cudaSuccess) return MFG_ERR_CUDA;
            if (stage < 3) continue;
            // the bookends in one pass: phi_old <- phi_new and the chemistry
            // sub-step (unless only_flow), primitive refresh, clipping, norms
            if (launch_post_step(boxes[b], dt, !only_flow, clip != 0, part, acc, st) != cudaSuccess)
                return MFG_ERR_CUDA;
            if (h_state) {
                if (cudaEventRecord(ev, st) != cudaSuccess || cudaStreamWaitEvent(cs, ev, 0) != cudaSuccess ||
                    cudaMemcpyAsync(h_state[b].p, boxes[b].s_new.p,
                                    view_span_doubles(boxes[b].s_new) * sizeof(double), cudaMemcpyDeviceToHost,
                                    cs) != cudaSuccess)
                    return MFG_ERR_CUDA;
            }
        }
    }
    if (h_state) {
        join.cs = nullptr;  // joined here, with its errors reported
        if (cudaEventRecord(ev, cs) != cudaSuccess || cudaStreamWaitEvent(st, ev, 0) != cudaSuccess)
            return MFG_ERR_CUDA;
    }
    std::vector<double> hn(resnorms ? N : 0);
    if (resnorms && cudaMemcpyAsync(hn.data(), acc, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MFG_ERR_CUDA;
    unsigned v = 0;
    if (cudaStreamSynchronize(st) != cudaSuccess || read_status(&v, false) != cudaSuccess) return MFG_ERR_CUDA;
    cutcache_sweep();
    if (resnorms)
        for (int n = 0; n < N; ++n) resnorms[n] = std::sqrt(hn[n]);
    if (v & MFG_STATUS_NEG_PRESSURE) return MFG_ERR_NEG_PRESSURE;
    if (v & MFG_STATUS_NAN) return MFG_ERR_NAN;
    return MFG_OK;
}

int mfg_advance_level(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double dt, int only_flow,
                      int clip, double* resnorms, void* stream) {
    int rc = check_boxes(boxes, nbox, true, false, true, true);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    return advance_level(boxes, nbox, geom, time, dt, only_flow, clip, resnorms, nullptr, (cudaStream_t)stream);
}

int mfg_advance_level_host(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time, double dt,
                           int only_flow, int clip, const mfg_array4* h_state, double* resnorms, void* stream) {
    int rc = check_boxes(boxes, nbox, true, false, true, true);
    if (rc) return rc;
    if (!geom || !h_state) return MFG_ERR_ARG;
    for (int b = 0; b < nbox; ++b)
        if (!same_layout(h_state[b], boxes[b].s_new)) return MFG_ERR_ARG;
    return advance_level(boxes, nbox, geom, time, dt, only_flow, clip, resnorms, h_state, (cudaStream_t)stream);
}

int mfg_set_cutcell_cache(int enable) {
    if (cudaDeviceSynchronize() != cudaSuccess) return MFG_ERR_CUDA;
    cutcache_enable(enable != 0);
    return MFG_OK;
}

}  // extern "C"
