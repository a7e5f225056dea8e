// AMReX-side adapter of the GB300 library: what a mesoflow build adds to call
// include/mflo_gpu.h from its MFIter loops.  Header-only C++ on AMReX's public
// types (amrex::Array4<Real>, GpuArray, IntVect), so it compiles unchanged
// against AMReX itself and against any stand-in with the same interface.
//
// It replaces the box bodies of
//   mflo::compute_dsdt_flow    Source/mflo_evolve.cpp:579-651 (and the flux
//                              register updates :655-681, through fluxfactor)
//   mflo::update_cutcell_data  Source/mflo_evolve.cpp:509-519
// with one library call per level: the loop collects one mfg_box per MFIter
// iteration (BoxSet::add), then BoxSet::compute_dsdt_flow / cutcells run the
// whole level on the caller's stream.
//
// Flux registers: mfg_compute_dsdt_flow writes the face fluxes themselves
// (flux[d] of each box), unscaled, exactly as the reference's flux MultiFabs
// hold them; the reference applies fluxfactor (1/6, 1/6, 2/3 per RK3 stage) only
// in the register calls, as scale = -+ tstep * dA * fluxfactor
// (Source/mflo_evolve.cpp:655-681).  register_scale() gives that factor for
// FluxRegister::CrseInit (coarse side, sign -1) and FineAdd (fine side, +1).
#ifndef MFLO_GPU_AMREX_H_
#define MFLO_GPU_AMREX_H_

#include <vector>

#include <AMReX_Array4.H>
#include <AMReX_REAL.H>

#include "mflo_gpu.h"

namespace mflo_gpu {

// amrex::Array4<Real> -> mfg_array4, field for field: data pointer, j/k/n
// strides, begin and (exclusive) end, component count.
inline mfg_array4 view(const amrex::Array4<amrex::Real>& a) {
    mfg_array4 v{};
    v.p = reinterpret_cast<double*>(a.p);
    v.jstride = a.jstride;
    v.kstride = a.kstride;
    v.nstride = a.nstride;
    v.begin[0] = a.begin.x;
    v.begin[1] = a.begin.y;
    v.begin[2] = a.begin.z;
    v.end[0] = a.end.x;
    v.end[1] = a.end.y;
    v.end[2] = a.end.z;
    v.ncomp = a.ncomp;
    return v;
}

// geom[lev] as the library's level geometry (CellSizeArray, ProbLoArray,
// Domain, isPeriodic).
inline mfg_geom geometry(const amrex::GpuArray<amrex::Real, 3>& dx, const amrex::GpuArray<amrex::Real, 3>& prob_lo,
                         const int domain_lo[3], const int domain_hi[3], const int periodic[3]) {
    mfg_geom g{};
    for (int d = 0; d < 3; ++d) {
        g.dx[d] = static_cast<double>(dx[d]);
        g.prob_lo[d] = static_cast<double>(prob_lo[d]);
        g.domain_lo[d] = domain_lo[d];
        g.domain_hi[d] = domain_hi[d];
        g.is_periodic[d] = periodic[d] ? 1 : 0;
    }
    return g;
}

// The factor the reference gives FluxRegister::CrseInit (side = -1) or
// FineAdd (side = +1) for direction d: side * tstep * dA * fluxfactor, dA the
// face area of the level (Source/mflo_evolve.cpp:662-678).
inline double register_scale(int side, int d, const amrex::GpuArray<amrex::Real, 3>& dx, double tstep,
                             double fluxfactor) {
    const double dA = (d == 0) ? static_cast<double>(dx[1]) * static_cast<double>(dx[2])
                    : (d == 1) ? static_cast<double>(dx[0]) * static_cast<double>(dx[2])
                               : static_cast<double>(dx[0]) * static_cast<double>(dx[1]);
    return (side < 0 ? -tstep : tstep) * dA * fluxfactor;
}

// The boxes of one level, collected in an MFIter loop.
class BoxSet {
public:
    // valid box lo/hi (Box::smallEnd/bigEnd); sborder grown by >= 3 cells;
    // any view may be empty (p == nullptr) where the call does not use it;
    // flux: three nodal views (for the flux registers) or nullptr.
    void add(const int lo[3], const int hi[3], const amrex::Array4<amrex::Real>& sborder,
             const amrex::Array4<amrex::Real>& dsdt, const amrex::Array4<amrex::Real>& s_old,
             const amrex::Array4<amrex::Real>& s_new, const amrex::Array4<amrex::Real>* flux = nullptr,
             int level = 0) {
        mfg_box b{};
        for (int d = 0; d < 3; ++d) {
            b.lo[d] = lo[d];
            b.hi[d] = hi[d];
        }
        b.sborder = view(sborder);
        b.dsdt = view(dsdt);
        b.s_old = view(s_old);
        b.s_new = view(s_new);
        if (flux)
            for (int d = 0; d < 3; ++d) b.flux[d] = view(flux[d]);
        b.level = level;
        boxes_.push_back(b);
    }
    void clear() { boxes_.clear(); }
    int size() const { return static_cast<int>(boxes_.size()); }
    const mfg_box* data() const { return boxes_.data(); }

    // mflo::compute_dsdt_flow's box loop for the whole level (dsdt and, where
    // given, the face fluxes); stream is the caller's cudaStream_t.
    int compute_dsdt_flow(const mfg_geom& g, double time, double tstep, void* stream) const {
        return mfg_compute_dsdt_flow(boxes_.data(), size(), &g, time, tstep, stream);
    }
    // mflo::update_cutcell_data's box loop for the whole level (in place on sborder).
    int cutcells(const mfg_geom& g, double time, void* stream) const {
        return mfg_cutcells(boxes_.data(), size(), &g, time, stream);
    }
    // compute_dsdt_flow fused with the RK3 stage algebra (Source/mflo_evolve.cpp:283,
    // 296-298, 309-311): s_new of each box becomes the stage result.
    int rk3_stage(const mfg_geom& g, int stage, double time, double dt, void* stream) const {
        return mfg_rk3_stage(boxes_.data(), size(), &g, stage, time, dt, stream);
    }

private:
    std::vector<mfg_box> boxes_;
};

// The reference's abort messages for the library's status codes
// (div_3d.H:74, Source/mflo_evolve.cpp:166, compute_flux_3d.H:273).
inline const char* abort_message(int rc) {
    switch (rc) {
        case MFG_ERR_NAN: return "NaN detected in dsdt\n";
        case MFG_ERR_NEG_PRESSURE: return "Pressure has gone negative";
        case MFG_ERR_SCHEME: return "unknown hyperbolics scheme";
        default: return "mflo_gpu: library call failed";
    }
}

}  // namespace mflo_gpu

#endif
