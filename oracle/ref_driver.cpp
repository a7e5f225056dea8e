// REFERENCE DRIVER — test infrastructure only.  Compiled (by oracle/ref.mk)
// together with the reference's own, unmodified per-cell numerics
// (Source/Src_3d/compute_flux_3d.H, flux_schemes.H, consprim_funcs.H,
// div_3d.H, ib_utils.H) and one case's plugin sources (species.H/.cpp,
// thermo.H, transport.H, userfuncs.H/.cpp, chemistry.H), against the AMReX
// stand-in in oracle/ref_shim/.  One shared library per case, since the
// plugins fix NUM_SPECIES at compile time.
//
// The loops below are the box bodies of the reference's drivers, over the
// same mfg_box descriptors the oracle and the GPU library take:
//   ref_compute_dsdt   mflo::compute_dsdt_flow's MFIter body
//                      (Source/mflo_evolve.cpp:579-651): transport and
//                      species-diffusion coefficients over grow(bx, ng), the
//                      fluid source over bx, compute_flux over growHi(bx, d, 1)
//                      for d = x, y, z into zeroed flux FABs (:566-573), then
//                      update_residual over bx and every component.
//   ref_cutcells       mflo::update_cutcell_data (:495-519): update_cutcells
//                      over the valid box, k, j, i ascending (AMReX's CPU
//                      ParallelFor order).
//   ref_chem_source    mflo::compute_dsdt_chemistry (:684-720) on s_new:
//                      dsdt = 0 + compute_spec_source.
// Built with MFG_COUNT_FLOPS (libref_count_<case>.so), Real is a counting
// double and ref_flop_counts reports the FP64 operations of those loops.
// Nothing here is linked into the product library.
#include <cstring>
#include <vector>

#include <globalDefines.H>
#include <mflo_constants.H>
#include <species.H>
#include <thermo.H>
#include <userfuncs.H>
#include <transport.H>
#include <chemistry.H>
#include <compute_flux_3d.H>
#include <div_3d.H>
#include <ib_utils.H>

#include "mflo_gpu.h"

namespace {

amrex::Array4<amrex::Real> view(const mfg_array4& a) {
    amrex::Array4<amrex::Real> v;
    v.p = reinterpret_cast<amrex::Real*>(a.p);
    v.jstride = a.jstride;
    v.kstride = a.kstride;
    v.nstride = a.nstride;
    v.begin = {a.begin[0], a.begin[1], a.begin[2]};
    v.end = {a.end[0], a.end[1], a.end[2]};
    v.ncomp = a.ncomp;
    return v;
}

// A host FAB over [lo, hi] (inclusive) with nc components, zero-filled.
struct Fab {
    std::vector<amrex::Real> v;
    amrex::Array4<amrex::Real> a;
    Fab(const int lo[3], const int hi[3], int nc) {
        int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
        v.assign((size_t)n0 * n1 * n2 * nc, 0.0);
        a.p = v.data();
        a.jstride = n0;
        a.kstride = (int64_t)n0 * n1;
        a.nstride = (int64_t)n0 * n1 * n2;
        a.begin = {lo[0], lo[1], lo[2]};
        a.end = {hi[0] + 1, hi[1] + 1, hi[2] + 1};
        a.ncomp = nc;
    }
};

amrex::GpuArray<amrex::Real, 3> arr3(const double* x) { return {{x[0], x[1], x[2]}}; }

template <class F>
void for_box(const int lo[3], const int hi[3], F f) {
    for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) f(i, j, k);
}

}  // namespace

extern "C" {

int ref_num_species(void) { return NUM_SPECIES; }

// species.cpp's init(): molecular weights, advection flags (and, where the
// plugin has them, reaction tables and species gammas).
int ref_init(void) {
    mflo_species::init();
    return 0;
}

double ref_molwt(int sp) { return static_cast<double>(mflo_species::molwts[sp]); }
double ref_advect_flag(int sp) { return static_cast<double>(mflo_species::advect_flags[sp]); }

int ref_compute_dsdt(const mfg_geom* G, const mfg_box* boxes, int nbox, double time, int order, double dissfactor,
                     int nsflag, int spec_in_solid, int conj_ht) {
    const auto dx = arr3(G->dx);
    const auto prob_lo = arr3(G->prob_lo);
    const int ncomp = TOTAL_NVARS;
    const int ng = MFG_NGROW;
    int status = MFG_OK;
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        int glo[3], ghi[3];
        for (int d = 0; d < 3; d++) {
            glo[d] = b.lo[d] - ng;
            ghi[d] = b.hi[d] + ng;
        }
        auto sb = view(b.sborder);
        auto dsdt = view(b.dsdt);
        Fab transport(glo, ghi, 2), specdiff(glo, ghi, NUM_SPECIES), source(b.lo, b.hi, ncomp);
        std::vector<Fab> flux;
        for (int d = 0; d < 3; d++) {
            int hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
            hi[d] += 1;
            flux.emplace_back(b.lo, hi, ncomp);
        }
        auto tr = transport.a, sd = specdiff.a, src = source.a;
        for_box(glo, ghi, [&](int i, int j, int k) {
            mflo_user_funcs::compute_fluid_transport(i, j, k, sb, tr, prob_lo, dx, time);
        });
        for_box(glo, ghi, [&](int i, int j, int k) {
            mflo_chem_transport::compute_spec_dcoeff(i, j, k, sb, sd, prob_lo, dx, time);
        });
        for_box(b.lo, b.hi, [&](int i, int j, int k) {
            mflo_user_funcs::compute_fluid_source(i, j, k, sb, src, prob_lo, dx, time);
        });
        try {
            for (int d = 0; d < 3; d++) {
                int hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
                hi[d] += 1;
                auto fx = flux[d].a;
                for_box(b.lo, hi, [&](int i, int j, int k) {
                    compute_flux(i, j, k, d, sb, tr, sd, fx, dx, order, dissfactor, nsflag != 0, spec_in_solid);
                });
            }
        } catch (const amrex::amrex_shim_abort&) {
            return MFG_ERR_SCHEME;
        }
        for (int n = 0; n < ncomp; n++)
            for_box(b.lo, b.hi, [&](int i, int j, int k) {
                try {
                    update_residual(i, j, k, n, dsdt, src, sb, flux[0].a, flux[1].a, flux[2].a, dx, spec_in_solid,
                                    conj_ht);
                } catch (const amrex::amrex_shim_abort&) {
                    status = MFG_ERR_NAN;
                }
            });
        for (int d = 0; d < 3; d++) {
            if (!b.flux[d].p) continue;
            auto out = view(b.flux[d]);
            int hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
            hi[d] += 1;
            for (int n = 0; n < ncomp; n++)
                for_box(b.lo, hi, [&](int i, int j, int k) { out(i, j, k, n) = flux[d].a(i, j, k, n); });
        }
    }
    return status;
}

int ref_cutcells(const mfg_geom* G, const mfg_box* boxes, int nbox, double time, int spec_in_solid,
                 int use_bg_gas, int cht) {
    const auto dx = arr3(G->dx);
    const auto plo = arr3(G->prob_lo);
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        auto sb = view(b.sborder);
        for_box(b.lo, b.hi, [&](int i, int j, int k) {
            update_cutcells(i, j, k, sb, dx, plo, time, spec_in_solid, use_bg_gas, cht);
        });
    }
    return MFG_OK;
}

int ref_chem_source(const mfg_geom* G, const mfg_box* boxes, int nbox, double time) {
    const auto dx = arr3(G->dx);
    const auto prob_lo = arr3(G->prob_lo);
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        auto s = view(b.s_new);
        auto dsdt = view(b.dsdt);
        Fab source(b.lo, b.hi, TOTAL_NVARS);
        auto src = source.a;
        for_box(b.lo, b.hi, [&](int i, int j, int k) {
            mflo_chem_reactions::compute_spec_source(i, j, k, s, src, prob_lo, dx, time);
        });
        for (int n = 0; n < TOTAL_NVARS; n++)
            for_box(b.lo, b.hi, [&](int i, int j, int k) { dsdt(i, j, k, n) = 0.0 + src(i, j, k, n); });
    }
    return MFG_OK;
}

#ifdef MFG_COUNT_FLOPS
// FP64 operations counted since the last reset (count_double.H): add, mul,
// div, sqrt, other.
void ref_flop_counts(uint64_t* out, int reset) {
    auto& c = mfg_count::counts();
    out[0] = c.add;
    out[1] = c.mul;
    out[2] = c.div;
    out[3] = c.sqrt;
    out[4] = c.other;
    if (reset) c = mfg_count::Counts();
}
#endif

}  // extern "C"
