// Step bookends and chemistry: reaction source, SSP-RK3 chemistry sub-step,
// primitive refresh, species clipping, residual norms and the CFL estimate.
#include "mfg_step_body.cuh"

namespace mfg {
namespace {

constexpr int TPB = 256;

template <int NS>
__global__ void chem_source_kernel(Valid v, Fab S, Fab D) {
    chem_source_body<NS>(v, S, D, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int NS>
__global__ void chem_substep_kernel(Valid v, Fab So, Fab Sn, double dt, int ncomp) {
    chem_substep_body<NS>(v, So, Sn, dt, ncomp, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int NS>
__global__ void prims_kernel(Valid v, Fab S) {
    prims_body<NS>(v, S, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int NS>
__global__ void chem_rk2_kernel(Valid v, Fab So, Fab Sn, double dt, int ncomp) {
    chem_rk2_body<NS>(v, So, Sn, dt, ncomp, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int NS>
__global__ void inertgas_kernel(Valid v, Fab S) {
    inertgas_body<NS>(v, S, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int NS>
__global__ void vars_after_chem_kernel(Valid v, Fab S, int bg) {
    vars_after_chem_body<NS>(v, S, bg, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void clip_kernel(Valid v, Fab S, int nspec) {
    clip_body(v, S, nspec, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Block partial sums of ((s_new - s_old)/dt [* vfrac_old])^2 per component;
// warp-shuffle reduction inside the block, partials in block order.
__global__ void resnorm_kernel(Valid v, Fab Sn, Fab So, double a, double b, double* partial, int nblk) {
    const int n = blockIdx.y;
    double acc = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        // LinComb then Multiply, rounded as the reference (no contraction)
        double d = add(mul(a, Sn(i, j, k, n)), mul(b, So(i, j, k, n)));
        if (n < VFRAC) d = mul(d, So(i, j, k, VFRAC));
        acc += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[TPB / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double x = (threadIdx.x < TPB / 32) ? ws[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (threadIdx.x == 0) partial[(int64_t)n * nblk + blockIdx.x] = x;
    }
}

// The bookends of a box after the RK3 stages in one pass (post_cell: phi_old
// <- phi_new and the chemistry sub-step when chem, primitive refresh, species
// clipping when clip) and, when partial != nullptr, the block partial sums of
// the residual norms ((s_new - s_old)/dt, flow components scaled by the old
// volume fraction).  Each thread keeps one running sum per component in
// registers (with the chemistry sub-step, only the components the bookends
// change can be non-zero); the block then sums them by warp shuffles and one
// warp adds the warps' sums in a fixed order, so the partials are
// deterministic.
constexpr int PTPB = 128;

template <int NS, int CHEM, bool NORMS>
__global__ void __launch_bounds__(PTPB) post_step_kernel(Valid v, Fab So, Fab Sn, double dt, int clip, double a,
                                                         double b, double* partial, int nblk) {
    constexpr int NM = NFLO + NS;
    const int N = NFLO + c_P.nspec;
    double acc[NM];
#pragma unroll
    for (int n = 0; n < NM; ++n) acc[n] = 0.0;
    bool nonfinite = false;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        post_cell<NS, CHEM, NORMS>(So, Sn, i, j, k, dt, clip != 0, a, b, acc, nonfinite);
    }
    if (!NORMS) return;
    const int any_nonfinite = __syncthreads_or(nonfinite ? 1 : 0);
    __shared__ double ws[PTPB / 32][NM];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int n = 0; n < NM; ++n) {
        if (CHEM != 0 && !(n >= DENS && n <= TEMP) && n < NFLO) continue;  // zero in every cell
        double x = acc[n];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) ws[warp][n] = x;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        const int n = threadIdx.x;
        double x;
        if (CHEM != 0 && !(n >= DENS && n <= TEMP) && n < NFLO) {
            x = any_nonfinite ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
        } else {
            x = 0.0;
            for (int w = 0; w < PTPB / 32; ++w) x += ws[w][n];
        }
        partial[(int64_t)n * nblk + blockIdx.x] = x;
    }
}

// Fixed-order final sum of the block partials, accumulated into acc[n].
__global__ void resnorm_final_kernel(const double* partial, int nblk, double* acc) {
    const int n = blockIdx.x;
    double x = 0.0;
    for (int b = threadIdx.x; b < nblk; b += 32) x += partial[(int64_t)n * nblk + b];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (threadIdx.x == 0) acc[n] += x;
}


// max wavespeed and max species diffusivity (Source/mflo_timestep.cpp:83-133)
template <int NS>
__global__ void timestep_kernel(Valid v, Fab S, double* acc2) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ws = 0.0, md = 0.0;
    if (t < v.n) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        timestep_cell<NS>(S, i, j, k, ws, md);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ws = fmax(ws, __shfl_down_sync(0xffffffffu, ws, o));
        md = fmax(md, __shfl_down_sync(0xffffffffu, md, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(acc2, ws);
        atomic_max_nonneg(acc2 + 1, md);
    }
}

// dst = (copy_first ? base : dst) + a*src over the valid box, all components.
__global__ void axpy_kernel(Valid v, Fab dst, Fab src, double a, int copy_first, Fab base, int ncomp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (t >= v.n || n >= ncomp) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    double x = copy_first ? base(i, j, k, n) : dst(i, j, k, n);
    if (src.p) x = add(x, mul(a, src(i, j, k, n)));
    dst(i, j, k, n) = x;
}

inline unsigned nblocks(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

template <template <int> class K>
struct Dispatch;

}  // namespace

cudaError_t launch_chem_source(const mfg_box& b, cudaStream_t st) {
    Valid v = valid_of(b);
    Fab S = make_fab(b.s_new), D = make_fab(b.dsdt);
    const int ns = c_host_params().nspec;
    ProfScope ps(K_CHEM, st);
    if (ns <= 1) chem_source_kernel<1><<<nblocks(v.n), TPB, 0, st>>>(v, S, D);
    else if (ns <= 2) chem_source_kernel<2><<<nblocks(v.n), TPB, 0, st>>>(v, S, D);
    else if (ns <= 4) chem_source_kernel<4><<<nblocks(v.n), TPB, 0, st>>>(v, S, D);
    else if (ns <= 8) chem_source_kernel<8><<<nblocks(v.n), TPB, 0, st>>>(v, S, D);
    else chem_source_kernel<16><<<nblocks(v.n), TPB, 0, st>>>(v, S, D);
    return cudaGetLastError();
}

cudaError_t launch_chem_substep(const mfg_box& b, double dt, cudaStream_t st) {
    Valid v = valid_of(b);
    Fab So = make_fab(b.s_old), Sn = make_fab(b.s_new);
    const int ns = c_host_params().nspec, nc = NFLO + ns;
    ProfScope ps(K_CHEM, st);
    if (ns <= 1) chem_substep_kernel<1><<<nblocks(v.n), TPB, 0, st>>>(v, So, Sn, dt, nc);
    else if (ns <= 2) chem_substep_kernel<2><<<nblocks(v.n), TPB, 0, st>>>(v, So, Sn, dt, nc);
    else if (ns <= 4) chem_substep_kernel<4><<<nblocks(v.n), TPB, 0, st>>>(v, So, Sn, dt, nc);
    else if (ns <= 8) chem_substep_kernel<8><<<nblocks(v.n), TPB, 0, st>>>(v, So, Sn, dt, nc);
    else chem_substep_kernel<16><<<nblocks(v.n), TPB, 0, st>>>(v, So, Sn, dt, nc);
    return cudaGetLastError();
}

cudaError_t launch_update_prims(const mfg_box& b, double*, cudaStream_t st) {
    Valid v = valid_of(b);
    Fab S = make_fab(b.s_new);
    const int ns = c_host_params().nspec;
    ProfScope ps(K_PRIMS, st);
    if (ns <= 1) prims_kernel<1><<<nblocks(v.n), TPB, 0, st>>>(v, S);
    else if (ns <= 2) prims_kernel<2><<<nblocks(v.n), TPB, 0, st>>>(v, S);
    else if (ns <= 4) prims_kernel<4><<<nblocks(v.n), TPB, 0, st>>>(v, S);
    else if (ns <= 8) prims_kernel<8><<<nblocks(v.n), TPB, 0, st>>>(v, S);
    else prims_kernel<16><<<nblocks(v.n), TPB, 0, st>>>(v, S);
    return cudaGetLastError();
}

// Split-chemistry pieces (Source/mflo_splitchem.cpp): kind 0 Advance_chemistry,
// 1 store_inertgas_conc, 2 update_vars_after_chemsolve (bg = using_bg_inertgas).
cudaError_t launch_split_chem(const mfg_box& b, int kind, double dt, int bg, cudaStream_t st) {
    Valid v = valid_of(b);
    Fab So = make_fab(b.s_old), Sn = make_fab(b.s_new);
    const int ns = c_host_params().nspec, nc = NFLO + ns;
    const unsigned g = nblocks(v.n);
    ProfScope ps(K_CHEM, st);
#define MFG_SPLIT(NSB)                                                                  \
    if (kind == 0) chem_rk2_kernel<NSB><<<g, TPB, 0, st>>>(v, So, Sn, dt, nc);         \
    else if (kind == 1) inertgas_kernel<NSB><<<g, TPB, 0, st>>>(v, Sn);                \
    else vars_after_chem_kernel<NSB><<<g, TPB, 0, st>>>(v, Sn, bg);
    if (ns <= 1) { MFG_SPLIT(1) }
    else if (ns <= 2) { MFG_SPLIT(2) }
    else if (ns <= 4) { MFG_SPLIT(4) }
    else if (ns <= 8) { MFG_SPLIT(8) }
    else { MFG_SPLIT(16) }
#undef MFG_SPLIT
    return cudaGetLastError();
}

cudaError_t launch_clip_species(const mfg_box& b, cudaStream_t st) {
    Valid v = valid_of(b);
    ProfScope ps(K_CLIP, st);
    clip_kernel<<<nblocks(v.n), TPB, 0, st>>>(v, make_fab(b.s_new), c_host_params().nspec);
    return cudaGetLastError();
}

// partial: scratch of (ncomp * 1024) doubles; acc: ncomp doubles (device).
cudaError_t launch_resnorm_box(const mfg_box& b, double dt, double* partial, double* acc, cudaStream_t st) {
    Valid v = valid_of(b);
    const int nc = NFLO + c_host_params().nspec;
    // 16 cells per thread: blocks of one cell per thread were dominated by their fixed cost
    int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(1024, (v.n + 16 * TPB - 1) / (16 * TPB)));
    dim3 g(nblk, nc);
    ProfScope ps(K_RESNORM, st, 2);
    resnorm_kernel<<<g, TPB, 0, st>>>(v, make_fab(b.s_new), make_fab(b.s_old), 1.0 / dt, -1.0 / dt, partial, nblk);
    resnorm_final_kernel<<<nc, 32, 0, st>>>(partial, nblk, acc);
    return cudaGetLastError();
}

// partial: scratch of (ncomp * 1024) doubles, acc: ncomp doubles (device), or
// both null (no residual norms).
cudaError_t launch_post_step(const mfg_box& b, double dt, bool chem, bool clip, double* partial, double* acc,
                             cudaStream_t st) {
    Valid v = valid_of(b);
    const int ns = c_host_params().nspec, nc = NFLO + ns;
    // one cell per thread up to one wave of blocks (4 of 128 threads resident
    // per SM at the kernel's ~115 registers), then a grid-stride loop: every
    // thread ends with warp sums of its norm terms, so fewer threads with
    // more cells each spend less of the FP64 pipe on them (3.37 -> 3.10 ms per
    // 256^3 step against 1024 blocks); at most 1024 (the partials' scratch)
    static int wave = 0;
    if (!wave) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        wave = std::max(1, std::min(1024, 4 * sms));
    }
    const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(wave, (v.n + PTPB - 1) / PTPB));
    const double a = 1.0 / dt, bb = -1.0 / dt;
    const size_t smem = 0;
    const DevParams& P = c_host_params();
    // the sub-step of a zero source (no reactions, explicit integrator) is s + 0
    const int kind = !chem ? 0 : (P.chem_kind == 0 && (!P.chem_on || P.nreact == 0)) ? 1 : 2;
    ProfScope ps(K_POST, st, partial ? 2 : 1);
#define MFG_POST_K(NSB, K)                                                                               \
    if (partial)                                                                                         \
        post_step_kernel<NSB, K, true><<<nblk, PTPB, smem, st>>>(v, make_fab(b.s_old), make_fab(b.s_new), dt, \
                                                                 clip, a, bb, partial, nblk);            \
    else                                                                                                 \
        post_step_kernel<NSB, K, false><<<nblk, PTPB, smem, st>>>(v, make_fab(b.s_old), make_fab(b.s_new), dt, \
                                                                  clip, a, bb, partial, nblk)
#define MFG_POST(NSB)                     \
    if (kind == 0) MFG_POST_K(NSB, 0);    \
    else if (kind == 1) MFG_POST_K(NSB, 1); \
    else MFG_POST_K(NSB, 2);
    if (ns <= 1) { MFG_POST(1) }
    else if (ns <= 2) { MFG_POST(2) }
    else if (ns <= 4) { MFG_POST(4) }
    else if (ns <= 8) { MFG_POST(8) }
    else { MFG_POST(16) }
#undef MFG_POST
#undef MFG_POST_K
    if (partial) resnorm_final_kernel<<<nc, 32, 0, st>>>(partial, nblk, acc);
    return cudaGetLastError();
}

cudaError_t launch_timestep(const mfg_box& b, double* acc2, cudaStream_t st) {
    Valid v = valid_of(b);
    Fab S = make_fab(b.s_new);
    const int ns = c_host_params().nspec;
    ProfScope ps(K_TIMESTEP, st);
    if (ns <= 1) timestep_kernel<1><<<nblocks(v.n), TPB, 0, st>>>(v, S, acc2);
    else if (ns <= 2) timestep_kernel<2><<<nblocks(v.n), TPB, 0, st>>>(v, S, acc2);
    else if (ns <= 4) timestep_kernel<4><<<nblocks(v.n), TPB, 0, st>>>(v, S, acc2);
    else if (ns <= 8) timestep_kernel<8><<<nblocks(v.n), TPB, 0, st>>>(v, S, acc2);
    else timestep_kernel<16><<<nblocks(v.n), TPB, 0, st>>>(v, S, acc2);
    return cudaGetLastError();
}

// Whether f holds exactly the valid box, components one after the other,
// with no padding (then a copy of it is one contiguous block).
static bool dense_over(const Fab& f, const mfg_box& b) {
    const int64_t l0 = b.hi[0] - b.lo[0] + 1, l1 = b.hi[1] - b.lo[1] + 1, l2 = b.hi[2] - b.lo[2] + 1;
    return f.p && f.b0 == b.lo[0] && f.b1 == b.lo[1] && f.b2 == b.lo[2] && f.js == l0 && f.ks == l0 * l1 &&
           f.ns == l0 * l1 * l2;
}

cudaError_t launch_axpy_valid(const mfg_box& b, const Fab& dst, const Fab& src, double a, bool copy_first,
                              const Fab& base, int ncomp, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing(st, &cs);
    if (ce != cudaSuccess) return ce;
    const bool capturing = cs != cudaStreamCaptureStatusNone;
    if (copy_first && !src.p && !capturing && dense_over(dst, b) && dense_over(base, b)) {
        // a plain copy of two dense arrays (phi_old <- phi_new): one block
        // copy at the copy bandwidth instead of a kernel per (cell, component)
        // (graphs keep the kernel: their conditional bodies take kernels);
        // arrays that overlap without being the same one take the kernel, whose
        // per-cell copy is defined for them
        const size_t bytes = (size_t)ncomp * dst.ns * sizeof(double);
        if (dst.p == base.p) {
            ProfScope ps(K_COPY, st, 0);
            return cudaSuccess;
        }
        const char *d0 = reinterpret_cast<const char*>(dst.p), *b0 = reinterpret_cast<const char*>(base.p);
        if (d0 + bytes <= b0 || b0 + bytes <= d0) {
            ProfScope ps(K_COPY, st, 0);
            return cudaMemcpyAsync(dst.p, base.p, bytes, cudaMemcpyDeviceToDevice, st);
        }
    }
    Valid v = valid_of(b);
    dim3 g(nblocks(v.n), ncomp);
    ProfScope ps(K_COPY, st);
    axpy_kernel<<<g, TPB, 0, st>>>(v, dst, src, a, copy_first ? 1 : 0, base, ncomp);
    return cudaGetLastError();
}

}  // namespace mfg
