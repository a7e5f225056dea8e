// Launch counter and per-kernel CUDA-event timing (enabled on request), the
// library's counterpart of the reference's BL_PROFILE regions.
#include <vector>

#include "mfg_internal.h"

namespace mfg {
namespace {

const char* kNames[K_COUNT] = {"prim", "face", "flux", "update", "fill_copy", "fill_bc",
                               "cutcell", "chem", "prims", "clip", "resnorm", "timestep", "copy",
                               "adj_face", "adj_cell", "adj_cut", "adj_fill", "adj_local", "snapshot",
                               "adj_flux", "amr_sync", "amr_patch", "amr_interp", "post"};

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

// Checks plus_zero (x + 0.0 on the integer pipe, used by the stage update)
// against the FP64 add, bit for bit, on boundary values (zeros, subnormals,
// the normal range's ends, infinities) and on pseudo-random bit patterns
// (xorshift64); NaN operands are skipped.  Counts mismatches in *bad.
__device__ unsigned long long exact_ops_value(unsigned long long i) {
    const unsigned long long special[] = {
        0x0000000000000000ULL, 0x0000000000000001ULL, 0x000FFFFFFFFFFFFFULL, 0x0010000000000000ULL,
        0x0020000000000000ULL, 0x0030000000000000ULL, 0x0031234567890ABCULL, 0x3FD0000000000000ULL,
        0x3FF0000000000000ULL, 0x7FD0000000000000ULL, 0x7FDFFFFFFFFFFFFFULL, 0x7FE0000000000000ULL,
        0x7FEFFFFFFFFFFFFFULL, 0x7FF0000000000000ULL, 0x0008000000000000ULL, 0x001FFFFFFFFFFFFFULL};
    const unsigned ns = sizeof(special) / sizeof(special[0]);
    if (i < 2 * ns) return special[i % ns] | ((i >= ns) ? 0x8000000000000000ULL : 0ULL);
    unsigned long long x = i * 0x9E3779B97F4A7C15ULL + 0x2545F4914F6CDD1DULL;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}
__device__ bool is_nan_bits(unsigned long long b) { return ((b >> 52) & 0x7ff) == 0x7ff && (b << 12) != 0; }
__global__ void exact_ops_kernel(unsigned long long n, unsigned* bad) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long bx = exact_ops_value(i);
    if (is_nan_bits(bx)) return;
    const double x = __longlong_as_double(bx);
    const unsigned m = __double_as_longlong(plus_zero(x)) != __double_as_longlong(__dadd_rn(x, 0.0)) ? 1u : 0u;
    if (m) atomicAdd(bad, m);
}
}  // namespace
}  // namespace mfg

extern "C" int mfg_selftest_exact_ops(unsigned long long n, unsigned* mismatches) {
    if (!mismatches || n == 0 || n > (1ULL << 32)) return MFG_ERR_ARG;
    unsigned* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned)) != cudaSuccess) return MFG_ERR_CUDA;
    cudaMemset(d, 0, sizeof(unsigned));
    mfg::exact_ops_kernel<<<(unsigned)((n + 255) / 256), 256>>>(n, d);
    const cudaError_t e = cudaMemcpy(mismatches, d, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return (e == cudaSuccess && cudaGetLastError() == cudaSuccess) ? MFG_OK : MFG_ERR_CUDA;
}

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
