// Launch counter and per-kernel CUDA-event timing (enabled on request), the
// library's counterpart of the reference's BL_PROFILE regions.
#include <vector>

#include "mfg_internal.h"

namespace mfg {
namespace {

const char* kNames[K_COUNT] = {"prim", "face", "flux", "update", "fill_copy", "fill_bc",
                               "cutcell", "chem", "prims", "clip", "resnorm", "timestep", "copy",
                               "adj_face", "adj_cell", "adj_cut", "adj_fill", "adj_local", "snapshot",
                               "adj_flux", "amr_sync", "amr_patch", "amr_interp"};

struct Pending {
    int kind;
    cudaEvent_t a, b;
};

bool g_on = false;
unsigned long long g_launches = 0;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_free;
double g_ms[K_COUNT];
long long g_cnt[K_COUNT];

cudaEvent_t ev() {
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void drain() {
    for (auto& p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        g_ms[p.kind] += ms;
        g_cnt[p.kind] += 1;
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
}

}  // namespace

bool profile_enabled() { return g_on; }

ProfScope::ProfScope(int kind, cudaStream_t st, int nlaunch) : kind_(kind), st_(st), a_(nullptr) {
    g_launches += (unsigned long long)nlaunch;
    if (g_on) {
        a_ = ev();
        cudaEventRecord((cudaEvent_t)a_, st_);
    }
}

ProfScope::~ProfScope() {
    if (g_on && a_) {
        cudaEvent_t b = ev();
        cudaEventRecord(b, st_);
        g_pending.push_back({kind_, (cudaEvent_t)a_, b});
        if (g_pending.size() > 4096) drain();
    }
}

}  // namespace mfg

using namespace mfg;

extern "C" {

int mfg_profile(int enable) {
    drain();
    g_on = enable != 0;
    for (int k = 0; k < K_COUNT; ++k) {
        g_ms[k] = 0.0;
        g_cnt[k] = 0;
    }
    return MFG_OK;
}

int mfg_profile_read(double* ms, long long* count, int nkinds) {
    drain();
    for (int k = 0; k < K_COUNT && k < nkinds; ++k) {
        if (ms) ms[k] = g_ms[k];
        if (count) count[k] = g_cnt[k];
    }
    return K_COUNT;
}

const char* mfg_profile_name(int kind) { return (kind >= 0 && kind < K_COUNT) ? kNames[kind] : ""; }

unsigned long long mfg_launch_count(void) { return g_launches; }

}  // extern "C"

// ---- FP64 issue-rate probe (the roof of every hot kernel here) ------------
namespace mfg {
namespace {
__global__ void dfma_probe_kernel(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = threadIdx.x * 1e-3 + q;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += x[q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace
}  // namespace mfg

extern "C" int mfg_measure_fp64_peak(double* tflops, void* stream) {
    if (!tflops) return MFG_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MFG_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return MFG_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, st);
        dfma_probe_kernel<<<blocks, threads, 0, st>>>(buf, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    const double flop = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flop / (best * 1e-3) / 1e12;
    return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}
