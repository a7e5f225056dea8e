// Test driver of the AMReX-side adapter (mesoflow_gb300/adapter/mflo_gpu_amrex.H),
// compiled against the AMReX stand-in in oracle/ref_shim (test infrastructure).
//   adapter_view_check   Array4 -> mfg_array4: the same element for every
//                        (i, j, k, n) of views with padded strides and offset
//                        begins (host only).
//   adapter_dsdt         a level's boxes as amrex::Array4<Real> views over the
//                        caller's device arrays, through BoxSet into
//                        mfg_compute_dsdt_flow.
//   adapter_cutcells     the same into mfg_cutcells.
// Built with ADAPTER_NO_LIB, only adapter_view_check (no library to link).
#include <cstdint>
#include <vector>

#include <AMReX_Array4.H>

#include "mflo_gpu_amrex.H"

namespace {

amrex::Array4<amrex::Real> grown_view(double* p, const int lo[3], const int hi[3], int g, int ncomp) {
    amrex::Array4<amrex::Real> a;
    const int64_t n0 = hi[0] - lo[0] + 1 + 2 * g, n1 = hi[1] - lo[1] + 1 + 2 * g, n2 = hi[2] - lo[2] + 1 + 2 * g;
    a.p = p;
    a.jstride = n0;
    a.kstride = n0 * n1;
    a.nstride = n0 * n1 * n2;
    a.begin = {lo[0] - g, lo[1] - g, lo[2] - g};
    a.end = {hi[0] + g + 1, hi[1] + g + 1, hi[2] + g + 1};
    a.ncomp = ncomp;
    return a;
}

}  // namespace

extern "C" {

int adapter_view_check(void) {
    int bad = 0;
    const int lo[3] = {-5, 7, 3}, hi[3] = {4, 12, 9};
    for (int pad = 0; pad < 3; ++pad) {
        const int n0 = hi[0] - lo[0] + 1 + pad, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1, nc = 4;
        std::vector<double> buf((size_t)n0 * n1 * n2 * nc + 7);
        amrex::Array4<amrex::Real> a;
        a.p = buf.data() + 3;
        a.jstride = n0;
        a.kstride = (int64_t)n0 * n1;
        a.nstride = (int64_t)n0 * n1 * n2 + pad;
        a.begin = {lo[0], lo[1], lo[2]};
        a.end = {hi[0] + 1, hi[1] + 1, hi[2] + 1};
        a.ncomp = nc;
        const mfg_array4 v = mflo_gpu::view(a);
        for (int n = 0; n < nc; ++n)
            for (int k = lo[2]; k <= hi[2]; ++k)
                for (int j = lo[1]; j <= hi[1]; ++j)
                    for (int i = lo[0]; i <= hi[0]; ++i) {
                        const double* m = v.p + (i - v.begin[0]) + (j - v.begin[1]) * v.jstride +
                                          (k - v.begin[2]) * v.kstride + n * v.nstride;
                        if (m != &a(i, j, k, n)) ++bad;
                    }
        for (int d = 0; d < 3; ++d)
            if (v.end[d] != hi[d] + 1) ++bad;
        if (v.ncomp != nc) ++bad;
    }
    return bad;
}

#ifndef ADAPTER_NO_LIB
// lohi: 6 ints per box (lo, hi); sb, dsdt, s_old, s_new: per-box device
// pointers laid out as dense component-major FABs (sborder grown by 3).
static mflo_gpu::BoxSet level_set(int nbox, const int* lohi, double* const* sb, double* const* dsdt,
                                  double* const* s_old, double* const* s_new, int ncomp) {
    mflo_gpu::BoxSet set;
    for (int b = 0; b < nbox; ++b) {
        const int* lo = lohi + 6 * b;
        const int* hi = lohi + 6 * b + 3;
        set.add(lo, hi, grown_view(sb[b], lo, hi, 3, ncomp), grown_view(dsdt[b], lo, hi, 0, ncomp),
                grown_view(s_old[b], lo, hi, 0, ncomp), grown_view(s_new[b], lo, hi, 0, ncomp));
    }
    return set;
}

int adapter_dsdt(int nbox, const int* lohi, double* const* sb, double* const* dsdt, double* const* s_old,
                 double* const* s_new, int ncomp, const double* dx, const double* plo, const int* dlo,
                 const int* dhi, const int* per, double time, double dt, void* stream) {
    const auto set = level_set(nbox, lohi, sb, dsdt, s_old, s_new, ncomp);
    const mfg_geom g = mflo_gpu::geometry({{dx[0], dx[1], dx[2]}}, {{plo[0], plo[1], plo[2]}}, dlo, dhi, per);
    return set.compute_dsdt_flow(g, time, dt, stream);
}

int adapter_cutcells(int nbox, const int* lohi, double* const* sb, double* const* dsdt, double* const* s_old,
                     double* const* s_new, int ncomp, const double* dx, const double* plo, const int* dlo,
                     const int* dhi, const int* per, double time, void* stream) {
    const auto set = level_set(nbox, lohi, sb, dsdt, s_old, s_new, ncomp);
    const mfg_geom g = mflo_gpu::geometry({{dx[0], dx[1], dx[2]}}, {{plo[0], plo[1], plo[2]}}, dlo, dhi, per);
    return set.cutcells(g, time, stream);
}

double adapter_register_scale(int side, int d, const double* dx, double tstep, double fluxfactor) {
    return mflo_gpu::register_scale(side, d, {{dx[0], dx[1], dx[2]}}, tstep, fluxfactor);
}
#endif

}  // extern "C"
