// Common device-side definitions of the GB300 mesoflow RHS library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "mflo_gpu.h"

namespace mfg {

// State layout (Source/globalDefines.H:5-32)
constexpr int RHO = 0, RHOU = 1, RHOV = 2, RHOW = 3, RHOE = 4;
constexpr int DENS = 5, VELX = 6, VELY = 7, VELZ = 8, PRES = 9, TEMP = 10, VFRAC = 11;
constexpr int NFLO = 12;
constexpr int NCONS = 5;
constexpr int MAXS = MFG_MAX_SPECIES;
constexpr int MAXR = MFG_MAX_REACTIONS;

// Constants with the exact values of Source/mflo_constants.H:4-27.
constexpr double kTwo3rd = 0.6666666666666666667;
constexpr double kHalf = 0.5;
constexpr double kThird = kTwo3rd * kHalf;
constexpr double kTwelveth = 0.08333333333;  // truncated in the reference
constexpr double kRU = 8.31446261815324;
constexpr double kTiny = 1e-20;
constexpr double kTiny2 = 1e-40;

// Parameters as the kernels read them (derived from mfg_params at mfg_init).
struct DevParams {
    int nspec, ngas, thermo_kind, energy_form;
    double R_univ, gas_R, gamma_single, bg_molwt;
    double molwt[MAXS];
    double gamma[MAXS + 1];
    double cv[MAXS + 1];       // R/(gamma_k - 1) per gas species (+ background gas)
    double igm1[MAXS + 1];     // 1/(gamma_k - 1)
    double cvmass[MAXS];       // R/(gamma_k - 1)/W_k (mass-cv energy form)
    double advect_flag[MAXS];
    int visc_mode, cond_mode;
    double visc_gas, visc_solid, cond_gas, cond_solid;
    int diff_mode[MAXS];
    double diff_gas[MAXS], diff_solid[MAXS];
    // face coefficients of constant transport: harmonic_mean(g, g), evaluated once
    double visc_hm, cond_hm, diff_hm[MAXS];
    // gamma/(gamma-1) and 2(gamma-1)/(gamma+1) of the mass-single family
    double g_gm1, astar_fac, gm1_single, inv_gas_R;
    int order_hyp, do_ns, species_in_solid, conj_ht;
    double dissfactor, solid_temp, cfl;
    int chem_on, nreact;
    double nu[MAXR][MAXS];
    double order[MAXR][MAXS];
    double A[MAXR], Ea[MAXR];
    // sparsity of the reaction table as bit masks over the species (bit s:
    // order[r][s] > 0, resp. nu[r][s] != 0), so the kernels test integers
    unsigned ord_mask[MAXR], nu_mask[MAXR];
    // chemistry sub-step integrator: 0 SSP-RK3 (the reference's default), 1 adaptive ROS2
    int chem_kind, chem_maxsub;
    double chem_rtol, chem_atol;
    int bc_lo[3], bc_hi[3];
    mfg_extbc ext_lo[3], ext_hi[3];
};

// Device view of one box: AMReX Array4 with begin offsets folded into the base.
struct Fab {
    double* p;
    int64_t js, ks, ns;
    int b0, b1, b2;
    __host__ __device__ __forceinline__ int64_t off(int i, int j, int k) const {
        return (int64_t)(i - b0) + (int64_t)(j - b1) * js + (int64_t)(k - b2) * ks;
    }
    __host__ __device__ __forceinline__ double& operator()(int i, int j, int k, int n) const {
        return p[off(i, j, k) + (int64_t)n * ns];
    }
};

inline Fab make_fab(const mfg_array4& a) {
    Fab f;
    memset(&f, 0, sizeof(f));  // padding included: tables of Fabs are compared bytewise
    f.p = a.p;
    f.js = a.jstride;
    f.ks = a.kstride;
    f.ns = a.nstride;
    f.b0 = a.begin[0];
    f.b1 = a.begin[1];
    f.b2 = a.begin[2];
    return f;
}

// Dense scratch FAB over an index box [lo, lo+len) with ncomp components.
__host__ __device__ __forceinline__ Fab dense_fab(double* p, const int lo[3], const int len[3]) {
    Fab f;
    f.p = p;
    f.js = len[0];
    f.ks = (int64_t)len[0] * len[1];
    f.ns = (int64_t)len[0] * len[1] * len[2];
    f.b0 = lo[0];
    f.b1 = lo[1];
    f.b2 = lo[2];
    return f;
}

// Sticky status word in device memory (mfg_status).
extern __device__ unsigned int g_status;

__device__ __forceinline__ void raise_status(unsigned bits) { atomicOr(&g_status, bits); }

// Rounding-faithful helpers: the intrinsics are never contracted into FMA,
// so expressions written with them round exactly as the reference's
// separate multiply and add.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// x + 0.0 without the FP64 pipe: -0 becomes +0, anything else is x (a NaN
// keeps its bits, where the add would quiet a signalling NaN; the states
// never hold one and a NaN rate raises MFG_STATUS_NAN).
__device__ __forceinline__ bool is_zero_bits(double x) { return (__double_as_longlong(x) << 1) == 0; }
__device__ __forceinline__ double plus_zero(double x) { return is_zero_bits(x) ? 0.0 : x; }
__device__ __forceinline__ bool is_finite_bits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// Volume-fraction tests on the integer pipe: for v >= 0 the IEEE order of
// doubles is the order of their bit patterns, so v < 1 and v == 1 need no
// FP64 compare (the FP64 pipe is the bottleneck of these kernels).
__device__ __forceinline__ bool below_one(double v) { return __double_as_longlong(v) < 0x3FF0000000000000LL; }
__device__ __forceinline__ bool is_one(double v) { return __double_as_longlong(v) == 0x3FF0000000000000LL; }

// Offsets (a0, a1, a2) of linear item t of an l0 x l1 x n2 box, a0 fastest.
// Every per-box item count fits in 32 bits, so 32-bit divisions serve (a
// 64-bit division is a long instruction sequence, comparable to the FP64
// work of the small per-(cell, component) kernels).
__device__ __forceinline__ void split3(int64_t t, int l0, int l1, int& a0, int& a1, int& a2) {
    const unsigned u = (unsigned)t, n0 = (unsigned)l0, n1 = (unsigned)l1;
    const unsigned q = u / n0;
    const unsigned q2 = q / n1;
    a0 = (int)(u - q * n0);
    a1 = (int)(q - q2 * n1);
    a2 = (int)q2;
}

// Comparisons and min/max on the integer pipe.  For doubles >= 0 the IEEE
// order is the order of the bit patterns read as signed 64-bit integers, so
// these select exactly what the FP64 forms select (NaN aside).
__device__ __forceinline__ bool abs_le(double x, double c) {  // |x| <= c, c > 0
    return (__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) <= __double_as_longlong(c);
}
__device__ __forceinline__ bool nonneg_le(double x, double c) {  // x <= c for x >= 0
    return __double_as_longlong(x) <= __double_as_longlong(c);
}
__device__ __forceinline__ bool nonneg_ge(double x, double c) {  // x >= c for x >= 0
    return __double_as_longlong(x) >= __double_as_longlong(c);
}
__device__ __forceinline__ bool is_positive(double x) { return __double_as_longlong(x) > 0; }  // x > 0
__device__ __forceinline__ double max_nonneg(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return __longlong_as_double(ia > ib ? ia : ib);
}
__device__ __forceinline__ double min_nonneg(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return __longlong_as_double(ia < ib ? ia : ib);
}
__device__ __forceinline__ double pos_part(double x) { return is_positive(x) ? x : 0.0; }  // max(x, 0)
__device__ __forceinline__ bool is_negative(double x) {  // x < 0 (false for -0 and NaN)
    const long long b = __double_as_longlong(x), m = b & 0x7FFFFFFFFFFFFFFFLL;
    return b < 0 && m != 0 && m <= 0x7FF0000000000000LL;
}
__device__ __forceinline__ bool is_nan(double x) {
    return (__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
}

// Reciprocal of a positive, finite, normal x: the hardware approximation
// (PTX rcp.approx.ftz.f64) refined by two Newton-Raphson steps
// r <- r + r (1 - x r), each of which squares the relative error, so the
// result is within one ulp of 1/x.  Four FMAs instead of a full IEEE
// division; used where the reference divides by a positive weight sum or a
// squared distance and the result only enters tolerance-checked sums.
__device__ __forceinline__ double rcp_pos(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Copies nc components of one cell, src and dst component strides ss and ds,
// four components' loads issued before their stores (the caller guarantees
// the two do not overlap and src is not written meanwhile), so a thread keeps
// four loads in flight instead of one.
__device__ __forceinline__ void copy_comps(double* dst, int64_t ds, const double* src, int64_t ss, int nc) {
    int c = 0;
    for (; c + 4 <= nc; c += 4) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = __ldg(src + (c + u) * ss);
#pragma unroll
        for (int u = 0; u < 4; ++u) dst[(c + u) * ds] = v[u];
    }
    for (; c < nc; ++c) dst[c * ds] = __ldg(src + c * ss);
}

// The same refinement for a finite, normal x of either sign (the hardware
// approximation and the Newton steps are odd in x).
__device__ __forceinline__ double rcp_nonzero(double x) { return rcp_pos(x); }

}  // namespace mfg
