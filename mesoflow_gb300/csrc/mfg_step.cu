// Step bookends and chemistry: reaction source, SSP-RK3 chemistry sub-step,
// primitive refresh, species clipping, residual norms and the CFL estimate.
#include "mfg_internal.h"
#include "mfg_physics.cuh"

namespace mfg {
namespace {

constexpr int TPB = 256;

struct Valid {
    int lo[3], len[3];
    int64_t n;
};

inline Valid valid_of(const mfg_box& b) {
    Valid v;
    v.n = 1;
    for (int d = 0; d < 3; ++d) {
        v.lo[d] = b.lo[d];
        v.len[d] = b.hi[d] - b.lo[d] + 1;
        v.n *= v.len[d];
    }
    return v;
}

__device__ __forceinline__ void cell_of(const Valid& v, int64_t t, int& i, int& j, int& k) {
    int64_t a = t / v.len[0];
    i = v.lo[0] + (int)(t - a * v.len[0]);
    k = v.lo[2] + (int)(a / v.len[1]);
    j = v.lo[1] + (int)(a - (int64_t)(k - v.lo[2]) * v.len[1]);
}

// Reaction source wdot (chemistry.H compute_spec_source, table form of
// py_utils/rxnscheme_writer/example/chemistry.H:27-54).  Rate constant:
// A_r, or A_r exp(-Ea_r/(RU T)) when Ea_r != 0.  Integer reaction orders 1
// and 2 are exact products (pow(c,1) = c, pow(c,2) = c*c).
template <int NS>
__device__ __forceinline__ void spec_source(const double* spec, double temp, double* wdot) {
    const DevParams& P = c_P;
#pragma unroll
    for (int s = 0; s < NS; ++s) wdot[s] = 0.0;
    if (!P.chem_on) return;
    for (int r = 0; r < P.nreact; ++r) {
        double cm = 1.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const double o = P.order[r][s];
            if (s < P.nspec && o > 0.0) {
                const double c = spec[s];
                cm *= (o == 1.0) ? c : (o == 2.0) ? c * c : pow(c, o);
            }
        }
        double kr = P.A[r];
        if (P.Ea[r] != 0.0) kr = P.A[r] * exp(-P.Ea[r] / (kRU * temp));
        const double rate = kr * cm;
#pragma unroll
        for (int s = 0; s < NS; ++s)
            if (s < P.nspec && fabs(P.nu[r][s]) > 0.0) wdot[s] += P.nu[r][s] * rate;
    }
}

template <int NS>
__global__ void chem_source_kernel(Valid v, Fab S, Fab D) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    double spec[NS], w[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) spec[s] = (s < c_P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
    spec_source<NS>(spec, S(i, j, k, TEMP), w);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        if (s < c_P.nspec) D(i, j, k, NFLO + s) = add(D(i, j, k, NFLO + s), add(0.0, w[s]));
}

// SSP-RK3 sub-step of the reaction source for one cell, all three stages in
// registers (the chemistry right-hand side is local to the cell).  Stage
// states S_i = S_old + sum_j (dt*a_ij) F_j, result S_old + sum_i (dt*w_i) F_i
// (AMReX RKIntegrator with the SSPRK3 tableau: a21=1, a31=a32=1/4,
// w=1/6,1/6,2/3).  Components without a source keep S_old.
template <int NS>
__global__ void chem_substep_kernel(Valid v, Fab So, Fab Sn, double dt, int ncomp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const int ns = c_P.nspec;
    double s0[NS], s1[NS], f0[NS], f1[NS], f2[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) s0[s] = (s < ns) ? So(i, j, k, NFLO + s) : 0.0;
    const double temp = So(i, j, k, TEMP);
    spec_source<NS>(s0, temp, f0);
    const double c10 = dt * 1.0, c20 = dt * 0.25, c21 = dt * 0.25;
#pragma unroll
    for (int s = 0; s < NS; ++s) s1[s] = add(s0[s], mul(c10, add(0.0, add(0.0, f0[s]))));
    spec_source<NS>(s1, temp, f1);
#pragma unroll
    for (int s = 0; s < NS; ++s)
        s1[s] = add(add(s0[s], mul(c20, add(0.0, add(0.0, f0[s])))), mul(c21, add(0.0, add(0.0, f1[s]))));
    spec_source<NS>(s1, temp, f2);
    const double w0 = dt * (1.0 / 6.0), w1 = dt * (1.0 / 6.0), w2 = dt * (2.0 / 3.0);
    for (int n = 0; n < ncomp; ++n) {
        if (n >= NFLO) continue;
        Sn(i, j, k, n) = So(i, j, k, n);
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        if (s >= ns) continue;
        double r = s0[s];
        r = add(r, mul(w0, add(0.0, add(0.0, f0[s]))));
        r = add(r, mul(w1, add(0.0, add(0.0, f1[s]))));
        r = add(r, mul(w2, add(0.0, add(0.0, f2[s]))));
        Sn(i, j, k, NFLO + s) = r;
    }
}

// cons -> prim refresh (Source/mflo_evolve.cpp:114-171); negative pressure
// raises a status bit instead of aborting.
template <int NS>
__global__ void prims_kernel(Valid v, Fab S) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    const DevParams& P = c_P;
    const double vf = S(i, j, k, VFRAC);
    if (vf == 1.0) {
        const double rho = S(i, j, k, RHO);
        double spec[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) spec[s] = (s < P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
        const double vx = S(i, j, k, RHOU) / rho, vy = S(i, j, k, RHOV) / rho, vz = S(i, j, k, RHOW) / rho;
        const double rhoe = S(i, j, k, RHOE) - (0.5 * rho) * ((vx * vx + vy * vy) + vz * vz);
        const double p = thermo_p<NS>(rhoe, rho, spec);
        S(i, j, k, DENS) = rho;
        S(i, j, k, VELX) = vx;
        S(i, j, k, VELY) = vy;
        S(i, j, k, VELZ) = vz;
        S(i, j, k, PRES) = p;
        S(i, j, k, TEMP) = thermo_t<NS>(rho, p, spec);
    } else if (P.conj_ht && vf == 0.0) {
        S(i, j, k, TEMP) = P.solid_temp;
    }
    if (P.do_ns && S(i, j, k, PRES) < 0.0) raise_status(MFG_STATUS_NEG_PRESSURE);
}

__global__ void clip_kernel(Valid v, Fab S, int nspec) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.n) return;
    int i, j, k;
    cell_of(v, t, i, j, k);
    for (int s = 0; s < nspec; ++s)
        if (S(i, j, k, NFLO + s) < 0.0) S(i, j, k, NFLO + s) = 0.0;
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

// Fixed-order final sum of the block partials, accumulated into acc[n].
__global__ void resnorm_final_kernel(const double* partial, int nblk, double* acc) {
    const int n = blockIdx.x;
    double x = 0.0;
    for (int b = threadIdx.x; b < nblk; b += 32) x += partial[(int64_t)n * nblk + b];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (threadIdx.x == 0) acc[n] += x;
}

__device__ __forceinline__ void atomic_max_nonneg(double* a, double v) {
    // IEEE order of non-negative doubles equals the order of their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

// max wavespeed and max species diffusivity (Source/mflo_timestep.cpp:83-133)
template <int NS>
__global__ void timestep_kernel(Valid v, Fab S, double* acc2) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ws = 0.0, md = 0.0;
    if (t < v.n) {
        int i, j, k;
        cell_of(v, t, i, j, k);
        const DevParams& P = c_P;
        const double vf = S(i, j, k, VFRAC);
        if (vf > 0.0) {
            const double ux = S(i, j, k, VELX), uy = S(i, j, k, VELY), uz = S(i, j, k, VELZ);
            const double fsp = sqrt((ux * ux + uy * uy) + uz * uz);
            double spec[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) spec[s] = (s < P.nspec) ? S(i, j, k, NFLO + s) : 0.0;
            const double gam = thermo_gamma<NS>(S(i, j, k, DENS), spec);
            const double ss = sqrt((gam * S(i, j, k, PRES)) / S(i, j, k, DENS));
            ws = fsp + (double)P.do_ns * ss;
        }
        double m = blend(P.diff_mode[0], P.diff_gas[0], P.diff_solid[0], vf);
        for (int s = 0; s < P.nspec; ++s) {
            const double dd = blend(P.diff_mode[s], P.diff_gas[s], P.diff_solid[s], vf);
            if (dd > m) m = dd;
        }
        md = fabs(m);
        ws = fabs(ws);
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
    int nblk = (int)std::min<int64_t>(1024, (v.n + TPB - 1) / TPB);
    dim3 g(nblk, nc);
    ProfScope ps(K_RESNORM, st);
    resnorm_kernel<<<g, TPB, 0, st>>>(v, make_fab(b.s_new), make_fab(b.s_old), 1.0 / dt, -1.0 / dt, partial, nblk);
    resnorm_final_kernel<<<nc, 32, 0, st>>>(partial, nblk, acc);
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

cudaError_t launch_axpy_valid(const mfg_box& b, const Fab& dst, const Fab& src, double a, bool copy_first,
                              const Fab& base, int ncomp, cudaStream_t st) {
    Valid v = valid_of(b);
    dim3 g(nblocks(v.n), ncomp);
    ProfScope ps(K_COPY, st);
    axpy_kernel<<<g, TPB, 0, st>>>(v, dst, src, a, copy_first ? 1 : 0, base, ncomp);
    return cudaGetLastError();
}

}  // namespace mfg
