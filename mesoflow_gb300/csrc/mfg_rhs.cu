// Flow right-hand side and fused RK3 stage update for one AMReX box.
//
// Structure (per RK stage, per box):
//   prim_kernel   per cell of grow(bx,3): velocities, pressure, eigen-pressure
//                 energy, own sound speed and gamma, computed once per cell
//                 instead of once per face use (the reference re-derives them
//                 inside every face's geteulerflux / get_max_eigenvalue).
//   face_kernel   per face of growHi(bx,d,1): scheme scalars (LLF eigenvalue,
//                 AUSM+-up Mach/pressure terms), IB flags, viscous stress and
//                 heat-conduction terms.  Orders 1/2 with Navier-Stokes terms
//                 split it: face_split_kernel writes the faces on the solid
//                 side (conduction and diffusion only) and lists the others,
//                 face_list_kernel runs the flux branch over those lists, each
//                 for the three directions in one launch, so no lane of a warp
//                 idles on a solid-side face.
//   flux_kernel   per (face, component): the hyperbolic flux of one
//                 component (WENO5-JS / MUSCL+AUSM+-up / central), species
//                 diffusion, and the viscous terms, written once per face and
//                 read by both neighbouring cells.
//   flux5_sweep_kernel  WENO5 with Navier-Stokes terms in the one-division
//                 mode: per (column segment along d, component), the per-cell
//                 parts of the reconstruction computed once per cell and kept
//                 in registers while the thread walks the faces.
//   update_kernel per (cell, component): flux divergence, IB masking, NaN
//                 status, and the RK3 stage algebra.
// Semantics: compute_flux (Source/Src_3d/compute_flux_3d.H:88-430),
// update_residual (Source/Src_3d/div_3d.H:13-76), stage algebra
// (Source/mflo_evolve.cpp:276-311).
#include <algorithm>
#include <cstdio>

#include "mfg_rhs_body.cuh"

namespace mfg {

__constant__ DevParams c_P;
__device__ unsigned int g_status = 0;

namespace {

constexpr int TPB = 256;
bool g_face_split = true;  // mfg_set_face_compaction

template <int NS>
__global__ void __launch_bounds__(TPB) prim_kernel(RhsBox B) {
    prim_body<NS>(B, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
template <int NS>
__global__ void __launch_bounds__(TPB) face_kernel(RhsBox B, int d) {
    face_body<NS>(B, d, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
// Orders 1 and 2 with Navier-Stokes terms: the inactive faces (solid side,
// conduction and diffusion only) of all three directions are written here
// (blockIdx.y = direction) and the active ones listed per direction (one
// atomic per warp), so that face_list_kernel runs the flux branch of all
// three directions in one launch with every lane of a warp busy (blocks past
// a direction's count exit at once).  Same
// per-face arithmetic: bitwise the results of face_kernel.
__device__ __forceinline__ int64_t face_list_off(const RhsBox& B, int d) {
    int64_t o = 0;
    for (int e = 0; e < d; ++e) o += face_count(B, e);
    return o;
}
template <int NS>
__global__ void __launch_bounds__(TPB) face_split_kernel(RhsBox B) {
    const int d = blockIdx.y;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool act = false;
    int lo[3] = {B.lo[0], B.lo[1], B.lo[2]}, len[3];
    for (int e = 0; e < 3; ++e) len[e] = B.hi[e] - B.lo[e] + 1 + (e == d);
    if (t < (int64_t)len[0] * len[1] * len[2]) {
        const Idx3 f = delinear(t, lo, len);  // once for the test and the body
        act = face_active(B, d, f);
        if (!act) face_body_at<NS, true>(B, d, f);
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    unsigned base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(B.fcount + d, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (act) B.flist[face_list_off(B, d) + base + __popc(m & ((1u << lane) - 1u))] = (int)t;
}
// The direction is the block's (blockIdx.y), uniform as in face_kernel, so
// the compiler forms the same multiply-adds in both.
// 128-thread blocks at 4 per SM (120 registers, no spills): after the FP64
// operation cuts the body fits without spilling at 16 resident warps, which
// measured 0.8% faster than 5 blocks at 96 registers with 80 bytes spilled
// (and 6 blocks at 80 registers 1% slower).
constexpr int LIST_TPB = 128;
template <int NS>
__global__ void __launch_bounds__(LIST_TPB, 4) face_list_kernel(RhsBox B) {
    const int d = blockIdx.y;
    const unsigned w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < B.fcount[d]) face_body<NS>(B, d, B.flist[face_list_off(B, d) + w]);
}
template <bool FAST>
__global__ void __launch_bounds__(TPB) flux_kernel(RhsBox B, int d) {
    flux_body<FAST>(B, d, blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
constexpr int SWEEP_TPB = 128;
__global__ void __launch_bounds__(SWEEP_TPB, 2) flux5_sweep_kernel(RhsBox B, int d, int seg) {
    flux5_sweep_body(B, d, blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, seg);
}
__global__ void __launch_bounds__(SWEEP_TPB, 2) flux5_face_kernel(RhsBox B, int d) {
    flux5_face_body(B, d, blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}
// One box's column segments must fill the GPU: segments of 32, 16 or 8 faces
// (longer ones share more per-cell work), else the per-face form of the same
// arithmetic.
constexpr int64_t SWEEP_MIN_THREADS = 152 * 2 * SWEEP_TPB * 2;
__global__ void __launch_bounds__(TPB) update_kernel(RhsBox B, int stage, double dt) {
    update_body(B, stage, dt, blockIdx.y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}


inline unsigned blocks_for(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

template <int NS>
cudaError_t launch_box_ns(const RhsBox& B, int stage, double dt, bool fast, cudaStream_t st) {
    const int nsp = c_host_params().nspec;
    const int C = NCONS + nsp;
    const int N = NFLO + nsp;
    int64_t ng = 1, nv = 1;
    for (int e = 0; e < 3; ++e) {
        ng *= (B.hi[e] - B.lo[e] + 1 + 2 * MFG_NGROW);
        nv *= (B.hi[e] - B.lo[e] + 1);
    }
    const int ord = c_host_params().order_hyp;
    if (ord == 4 || ord == 5) {
        ProfScope ps(K_PRIM, st);
        prim_kernel<NS><<<blocks_for(ng), TPB, 0, st>>>(B);
    }
    const bool split = g_face_split && c_host_params().do_ns && ord <= 2;
    if (split) {
        int64_t nfmax = 0;
        for (int d = 0; d < 3; ++d) {
            int64_t nf = 1;
            for (int e = 0; e < 3; ++e) nf *= (B.hi[e] - B.lo[e] + 1 + (e == d));
            nfmax = std::max(nfmax, nf);
        }
        cudaMemsetAsync(B.fcount, 0, 3 * sizeof(unsigned), st);
        ProfScope ps(K_FACE, st, 2);
        face_split_kernel<NS><<<dim3(blocks_for(nfmax), 3), TPB, 0, st>>>(B);
        face_list_kernel<NS><<<dim3((unsigned)((nfmax + LIST_TPB - 1) / LIST_TPB), 3), LIST_TPB, 0, st>>>(B);
    }
    for (int d = 0; d < 3 && !split; ++d) {
        int64_t nf = 1;
        for (int e = 0; e < 3; ++e) nf *= (B.hi[e] - B.lo[e] + 1 + (e == d));
        {
            ProfScope ps(K_FACE, st);
            face_kernel<NS><<<blocks_for(nf), TPB, 0, st>>>(B, d);
        }
        if (c_host_params().do_ns && ord <= 2) continue;  // the face kernels wrote the fluxes
        ProfScope ps(K_FLUX, st);
        if (fast && ord == 5 && c_host_params().do_ns) {
            int seg = 32;
            while (seg > 8 && sweep_items(B, d, seg) * C < SWEEP_MIN_THREADS) seg /= 2;
            const int64_t ns = sweep_items(B, d, seg);
            if (ns * C >= SWEEP_MIN_THREADS) {
                dim3 g((unsigned)((ns + SWEEP_TPB - 1) / SWEEP_TPB), C);
                flux5_sweep_kernel<<<g, SWEEP_TPB, 0, st>>>(B, d, seg);
            } else {
                dim3 g((unsigned)((nf + SWEEP_TPB - 1) / SWEEP_TPB), C);
                flux5_face_kernel<<<g, SWEEP_TPB, 0, st>>>(B, d);
            }
            continue;
        }
        dim3 g(blocks_for(nf), C);
        if (fast)
            flux_kernel<true><<<g, TPB, 0, st>>>(B, d);
        else
            flux_kernel<false><<<g, TPB, 0, st>>>(B, d);
    }
    dim3 gu(blocks_for(nv), N);
    ProfScope ps(K_UPDATE, st);
    update_kernel<<<gu, TPB, 0, st>>>(B, stage, dt);
    return cudaGetLastError();
}

}  // namespace

cudaError_t upload_params(const DevParams& h) { return cudaMemcpyToSymbol(c_P, &h, sizeof(DevParams)); }

cudaError_t read_status(unsigned* v, bool clear) {
    cudaError_t e = cudaMemcpyFromSymbol(v, g_status, sizeof(unsigned));
    if (e == cudaSuccess && clear) {
        unsigned z = 0;
        e = cudaMemcpyToSymbol(g_status, &z, sizeof(unsigned));
    }
    return e;
}

cudaError_t launch_rhs_box(const RhsBox& B, int stage, double dt, bool fast, cudaStream_t st) {
    const int ns = c_host_params().nspec;
    if (ns <= 1) return launch_box_ns<1>(B, stage, dt, fast, st);
    if (ns <= 2) return launch_box_ns<2>(B, stage, dt, fast, st);
    if (ns <= 4) return launch_box_ns<4>(B, stage, dt, fast, st);
    if (ns <= 8) return launch_box_ns<8>(B, stage, dt, fast, st);
    return launch_box_ns<16>(B, stage, dt, fast, st);
}

}  // namespace mfg

extern "C" int mfg_set_face_compaction(int on) {
    if (cudaDeviceSynchronize() != cudaSuccess) return MFG_ERR_CUDA;
    mfg::g_face_split = on != 0;
    return MFG_OK;
}
