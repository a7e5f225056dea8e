// Internal host/device interfaces shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include "mfg_common.cuh"

namespace mfg {

// Per-cell scalars of prim_kernel (scratch over grow(bx, 3)).
enum AuxComp { AUX_VX = 0, AUX_VY, AUX_VZ, AUX_PF, AUX_REIG, AUX_AOWN, AUX_GAM, NAUX };

// Per-face scalars of face_kernel (scratch over growHi(bx, d, 1)).
enum FsComp {
    FS_FLAGS = 0,  // bit0: hyperbolic + viscous flux active, bit1: first-order IB fallback
    FS_LAMBDA,     // LLF eigenvalue (orders 4, 5) or AUSM a_half (orders 1, 2)
    FS_MH,         // AUSM M_half
    FS_MODM,       // AUSM |M_half| with the entropy fix
    FS_PH,         // AUSM p_half
    FS_PL,         // AUSM left pressure
    FS_PR,         // AUSM right pressure
    FS_VIS,        // 3: viscous momentum terms tau_{d,a}
    FS_VISE = FS_VIS + 3,   // 3: viscous work terms tau_{d,a} * facevel_a
    FS_THERM = FS_VISE + 3, // heat-conduction term k dT/dn
    NFS
};

// Kernel kinds of the launch counter / event profiler (mfg_prof.cu).
enum KernelKind {
    K_PRIM = 0, K_FACE, K_FLUX, K_UPDATE, K_FILL_COPY, K_FILL_BC, K_CUT, K_CHEM, K_PRIMS, K_CLIP,
    K_RESNORM, K_TIMESTEP, K_COPY,
    // adjoint (mfg_adjoint.cu)
    K_ADJ_FACE, K_ADJ_CELL, K_ADJ_CUT, K_ADJ_FILL, K_ADJ_LOCAL, K_SNAPSHOT, K_ADJ_FLUX, K_AMR_SYNC, K_AMR_PATCH, K_AMR_INTERP,
    // fused step bookends (mfg_step.cu)
    K_POST, K_COUNT
};

// Counts one launch; when profiling is on, brackets it with CUDA events on its stream.
// True while mfg_profile is on (per-launch CUDA events are recorded).
bool profile_enabled();

// Counts the kernels launched inside it (nlaunch) and, while profiling is
// on, times them as one entry of their kind.
class ProfScope {
  public:
    ProfScope(int kind, cudaStream_t st, int nlaunch = 1);
    ~ProfScope();

  private:
    int kind_;
    cudaStream_t st_;
    void* a_;
};

// Everything the RHS kernels of one box need, passed by value.
struct RhsBox {
    int lo[3], hi[3];
    double dx[3];
    double idx[3];  // 1/dx
    Fab sb, dsdt, sold, snew;
    Fab uflux[3];
    Fab aux;
    Fab fs[3];
    Fab flx[3];
    int* flist;        // active faces of the three directions, one after the other (orders 1, 2
                       // with Navier-Stokes terms)
    unsigned* fcount;  // 3: active faces per direction
};

const DevParams& c_host_params();

// Box validation, scratch size and scratch layout of the RHS (mfg_api.cu).
int validate_boxes(const mfg_box* boxes, int nbox, bool need_sb, bool need_dsdt, bool need_old, bool need_new);
size_t rhs_box_scratch_doubles(const int n[3]);
struct RhsBox;
RhsBox layout_rhs_box(const mfg_box& b, const mfg_geom& g, double* base);
bool weno_fast_mode();

cudaError_t upload_params(const DevParams& h);
cudaError_t read_status(unsigned* v, bool clear);

// Records the description of a failed CUDA call for mfg_last_error (mfg_api.cu).
void note_cuda_error(cudaError_t e, const char* where);
cudaError_t launch_rhs_box(const RhsBox& B, int stage, double dt, bool fast, cudaStream_t st);

// Scratch sizes (doubles) for a box of the given valid extent.
inline size_t aux_doubles(const int n[3]) {
    return (size_t)(n[0] + 6) * (n[1] + 6) * (n[2] + 6) * NAUX;
}
inline size_t face_doubles(const int n[3], int d, int ncomp) {
    return (size_t)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2)) * ncomp;
}
// Four counters and the active-face lists of the three directions, as doubles.
inline size_t face_list_doubles(const int n[3]) {
    size_t m = 0;
    for (int d = 0; d < 3; ++d) m += face_doubles(n, d, 1);
    return (m + 4 + 1) / 2;
}

// Other kernels (mfg_ib.cu, mfg_fill.cu, mfg_step.cu)
cudaError_t launch_chem_source(const mfg_box& b, cudaStream_t st);
cudaError_t launch_axpy_valid(const mfg_box& b, const Fab& dst, const Fab& src, double a, bool copy_first,
                              const Fab& base, int ncomp, cudaStream_t st);
cudaError_t launch_update_prims(const mfg_box& b, double* minp_slot, cudaStream_t st);
cudaError_t launch_split_chem(const mfg_box& b, int kind, double dt, int bg, cudaStream_t st);
cudaError_t launch_clip_species(const mfg_box& b, cudaStream_t st);
cudaError_t launch_post_step(const mfg_box& b, double dt, bool chem, bool clip, double* partial, double* acc,
                             cudaStream_t st);
cudaError_t launch_timestep(const mfg_box& b, double* acc2, cudaStream_t st);

cudaError_t launch_fill_patch(const mfg_box* boxes, int nbox, const mfg_geom& g, int s_src, double time,
                              cudaStream_t st);

// Cut-cell cache (mfg_ib.cu): drop entries whose volume fraction changed
// (after a host synchronization), free everything, switch on/off.
void cutcache_sweep();
// All boxes of a level in one launch per phase: 1 done, 0 the per-box path
// must run (nothing launched), -1 CUDA error (mfg_ib.cu).
int launch_cutcells_level(const mfg_box* boxes, int nbox, const mfg_geom& g, cudaStream_t st);
void cutcache_release();
void cutcache_enable(bool on);
// Allocation-free entry point (mfg_noalloc.cu): forget the per-device addresses
// of its static scratch array.
void noalloc_forget();

}  // namespace mfg
