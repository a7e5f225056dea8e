// Allocation-free variant of the flow right-hand side (mfg_compute_dsdt_flow).
//
// Who needs it: callers that must not allocate device memory while they run.
// The main one is an AMReX application: by default AMReX reserves most of the
// GPU's memory for its own arena at start-up (amrex.the_arena_init_size), so a
// library that calls cudaMalloc on the side can fail or fragment what is left,
// and every cudaFree synchronizes the whole device.  Others are codes with a
// fixed device-memory budget decided up front, and callers that run the RHS
// from a context where CUDA allocation calls are not permitted.  This entry
// point therefore takes its scratch (per-cell primitives, per-face scheme
// scalars, per-face fluxes) from one statically sized device array compiled
// into the library instead of from the library's growable scratch pool.
//
// Limits and sharing:
//  * The array holds MFG_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB).  Every GPU
//    that loads this library holds it until the process exits.  A box whose
//    scratch would not fit is rejected with MFG_ERR_SIZE before anything is
//    launched.
//  * All calls share the one array and it keeps the previous call's contents.
//    The RHS kernels write every scratch entry before reading it, so nothing
//    has to be cleared between calls.  Calls whose work overlaps on the GPU
//    (different streams, or different host threads without ordering) race on
//    the array; serialize them.
//  * The device address of the array is looked up once per device, on the
//    first call made with that device current (host threads may make that
//    first call concurrently).  Make that first call before any stream
//    capture begins.  mfg_finalize forgets the addresses: after a
//    cudaDeviceReset, call mfg_finalize before this entry point runs again.
#include <atomic>
#include <mutex>

#include "mfg_internal.h"

namespace mfg {
namespace {

static __device__ __align__(256) double g_noalloc_scratch[MFG_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::atomic<double*> g_scratch_ptr[kMaxDevices];
std::mutex g_scratch_mu;

// Device address of the static array for the current device (host code may not
// use the symbol itself: on the host it names a stand-in, not device memory).
int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MFG_ERR_CUDA;
    double* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        p = g_scratch_ptr[dev].load(std::memory_order_relaxed);
        if (!p) {
            void* q = nullptr;
            if (cudaGetSymbolAddress(&q, g_noalloc_scratch) != cudaSuccess || !q) return MFG_ERR_CUDA;
            p = static_cast<double*>(q);
            g_scratch_ptr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return MFG_OK;
}

}  // namespace

// Forgets the looked-up addresses (mfg_finalize), so that the next call looks
// them up again in the current context.
void noalloc_forget() {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    for (auto& p : g_scratch_ptr) p.store(nullptr, std::memory_order_release);
}

}  // namespace mfg

using namespace mfg;

extern "C" int mfg_compute_dsdt_flow_noalloc(const mfg_box* boxes, int nbox, const mfg_geom* geom, double time,
                                             double dt, void* stream) {
    (void)time;
    int rc = validate_boxes(boxes, nbox, true, true, false, false);
    if (rc) return rc;
    if (!geom) return MFG_ERR_ARG;
    for (int b = 0; b < nbox; ++b) {
        int n[3];
        for (int d = 0; d < 3; ++d) n[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1;
        if (rhs_box_scratch_doubles(n) > (size_t)MFG_NOALLOC_SCRATCH_DOUBLES) return MFG_ERR_SIZE;
    }
    double* scratch = nullptr;
    if ((rc = scratch_for_current_device(&scratch))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    for (int b = 0; b < nbox; ++b) {
        RhsBox B = layout_rhs_box(boxes[b], *geom, scratch);
        if (launch_rhs_box(B, 0, dt, weno_fast_mode(), st) != cudaSuccess) return MFG_ERR_CUDA;
    }
    return MFG_OK;
}
