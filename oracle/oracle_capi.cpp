// ORACLE — test infrastructure only (see mflo_oracle.hpp).  C API over the
// restatement, operating on host arrays described by the same mfg_box /
// mfg_array4 views as the product's C ABI, plus a single-level driver that
// restates mflo::Advance_coupled_strang and the step bookends.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mflo_oracle.hpp"

using namespace oracle;

namespace {

struct Level {
    const mfg_params* P;
    const mfg_geom* G;
    const mfg_box* boxes;
    int nbox;
};

inline int ncomp_of(const mfg_params* P) { return FLO_NVARS + P->nspec; }

inline bool in_box(const mfg_box& b, int i, int j, int k) {
    return i >= b.lo[0] && i <= b.hi[0] && j >= b.lo[1] && j <= b.hi[1] && k >= b.lo[2] && k <= b.hi[2];
}

// Flux FAB (nodal in d) holding the box's faces, zero-initialised (setVal, mflo_evolve.cpp:566-573).
struct FluxFab {
    std::vector<double> v;
    A4 a;
    void define(const mfg_box& b, int d, int nc) {
        int n0 = b.hi[0] - b.lo[0] + 1 + (d == 0), n1 = b.hi[1] - b.lo[1] + 1 + (d == 1),
            n2 = b.hi[2] - b.lo[2] + 1 + (d == 2);
        v.assign((size_t)n0 * n1 * n2 * nc, 0.0);
        a.p = v.data();
        a.js = n0;
        a.ks = (int64_t)n0 * n1;
        a.ns = (int64_t)n0 * n1 * n2;
        a.b0 = b.lo[0]; a.b1 = b.lo[1]; a.b2 = b.lo[2];
    }
};

int dsdt_box(const Ctx& c, const mfg_geom* G, const mfg_box& b) {
    const int nc = ncomp_of(c.P);
    A4 phi(b.sborder), dsdt(b.dsdt);
    FluxFab F[3];
    for (int d = 0; d < 3; d++) F[d].define(b, d, nc);
    for (int d = 0; d < 3; d++) {
        int hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
        hi[d] += 1;  // growHi(bx, d, 1)
        for (int k = b.lo[2]; k <= hi[2]; k++)
            for (int j = b.lo[1]; j <= hi[1]; j++)
                for (int i = b.lo[0]; i <= hi[0]; i++) {
                    int rc = compute_flux(c, i, j, k, d, phi, F[d].a, G->dx);
                    if (rc) return rc;
                }
    }
    int status = MFG_OK;
    for (int n = 0; n < nc; n++)
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    int rc = update_residual(c, i, j, k, n, dsdt, phi, F[0].a, F[1].a, F[2].a, G->dx);
                    if (rc) status = rc;
                }
    for (int d = 0; d < 3; d++) {
        if (!b.flux[d].p) continue;
        A4 out(b.flux[d]);
        int hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
        hi[d] += 1;
        for (int n = 0; n < nc; n++)
            for (int k = b.lo[2]; k <= hi[2]; k++)
                for (int j = b.lo[1]; j <= hi[1]; j++)
                    for (int i = b.lo[0]; i <= hi[0]; i++) out(i, j, k, n) = F[d].a(i, j, k, n);
    }
    return status;
}

// ---- single-level FillPatch restatement ----------------------------------
// Valid data (periodic images included) is copied first (AMReX
// FillPatchSingleLevel -> FillBoundary/ParallelCopy).  Cells outside the
// domain in a set D of non-periodic directions are then filled in order of
// |D| = 1, 2, 3 (faces, edges, corners of GpuBndryFuncFab), each from the
// cell one layer "inward" along a single direction d*: the highest direction
// of D whose bc is ext_dir (the user functor AmrCoreFill, mflo_bcfill.H,
// runs after filcc_cell and checks x, y, z in turn), else the highest
// direction of D (filcc_cell checks x, y, z in turn).  Unpinned: AMReX is not
// vendored in the reference.
void externalbc(const Ctx& c, const mfg_extbc& E, const double* s_int, double* s_ext, int idir, int sgn) {
    const mfg_params* P = c.P;
    const int ns = c.nspec, nc = FLO_NVARS + ns;
    for (int n = 0; n < nc; n++) s_ext[n] = 0.0;
    if (E.kind == MFG_EXT_FIXED_STATE) {
        // tests/Cartesian/ShockTube_N2/externbc.H:95-126
        for (int n = 0; n < nc; n++) s_ext[n] = E.state[n];
        if (E.keep_interior_pres) s_ext[PRES_INDX] = s_int[PRES_INDX];
        return;
    }
    double spec_ext[MAXS];
    double dens, pres, vel[3];
    if (E.kind == MFG_EXT_PRESSURE_INLET) {
        // models/porousParticle/externbc.H:27-43 (normal = idir)
        dens = E.dens;
        pres = E.pres;
        double velmag = std::sqrt(s_int[VELX_INDX] * s_int[VELX_INDX] + s_int[VELY_INDX] * s_int[VELY_INDX] +
                                  s_int[VELZ_INDX] * s_int[VELZ_INDX]);
        vel[0] = vel[1] = vel[2] = zeroval;
        vel[idir] = velmag;
        for (int sp = 0; sp < ns; sp++) spec_ext[sp] = E.spec[sp];
    } else if (E.kind == MFG_EXT_PRESSURE_OUTLET) {
        // models/porousParticle/externbc.H:44-58
        dens = s_int[DENS_INDX];
        pres = E.pres;
        vel[0] = s_int[VELX_INDX]; vel[1] = s_int[VELY_INDX]; vel[2] = s_int[VELZ_INDX];
        for (int sp = 0; sp < ns; sp++) spec_ext[sp] = s_int[FLO_NVARS + sp];
    } else {  // MFG_EXT_VELOCITY_INLET
        dens = E.dens;
        pres = E.pres;
        vel[0] = E.vel[0]; vel[1] = E.vel[1]; vel[2] = E.vel[2];
        for (int sp = 0; sp < ns; sp++) spec_ext[sp] = E.spec[sp];
    }
    (void)sgn;
    s_ext[DENS_INDX] = dens;
    s_ext[PRES_INDX] = pres;
    s_ext[VELX_INDX] = vel[0]; s_ext[VELY_INDX] = vel[1]; s_ext[VELZ_INDX] = vel[2];
    s_ext[TEMP_INDX] = get_t_from_rpc(c, s_ext[DENS_INDX], s_ext[PRES_INDX], spec_ext);
    s_ext[RHO_INDX] = s_ext[DENS_INDX];
    s_ext[RHOU_INDX] = s_ext[DENS_INDX] * s_ext[VELX_INDX];
    s_ext[RHOV_INDX] = s_ext[DENS_INDX] * s_ext[VELY_INDX];
    s_ext[RHOW_INDX] = s_ext[DENS_INDX] * s_ext[VELZ_INDX];
    s_ext[RHOE_INDX] = s_ext[DENS_INDX] * get_e_from_rpc(c, s_ext[DENS_INDX], s_ext[PRES_INDX], spec_ext);
    s_ext[RHOE_INDX] += half * s_ext[DENS_INDX] *
                        (s_ext[VELX_INDX] * s_ext[VELX_INDX] + s_ext[VELY_INDX] * s_ext[VELY_INDX] +
                         s_ext[VELZ_INDX] * s_ext[VELZ_INDX]);
    for (int sp = 0; sp < ns; sp++) s_ext[FLO_NVARS + sp] = spec_ext[sp];
    s_ext[VFRAC_INDX] = s_int[VFRAC_INDX];
}

inline bool odd_at_wall(int n) {  // Source/mflo.cpp:98-110
    return n == RHOU_INDX || n == RHOV_INDX || n == RHOW_INDX || n == VELX_INDX || n == VELY_INDX || n == VELZ_INDX;
}

int fill_patch(const Ctx& c, const Level& L, int s_src, double time) {
    (void)time;
    const mfg_geom* G = L.G;
    const mfg_params* P = c.P;
    const int nc = ncomp_of(P);
    const int* dlo = G->domain_lo;
    const int* dhi = G->domain_hi;
    int status = MFG_OK;
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 sb(b.sborder);
        int glo[3], ghi[3];
        for (int d = 0; d < 3; d++) { glo[d] = b.lo[d] - MFG_NGROW; ghi[d] = b.hi[d] + MFG_NGROW; }
        // 1) copy valid data (own box + other boxes + periodic images)
        std::vector<signed char> nout;  // per grown cell: number of outside directions, -1 = filled
        int n0 = ghi[0] - glo[0] + 1, n1 = ghi[1] - glo[1] + 1, n2 = ghi[2] - glo[2] + 1;
        nout.assign((size_t)n0 * n1 * n2, 0);
        for (int k = glo[2]; k <= ghi[2]; k++)
            for (int j = glo[1]; j <= ghi[1]; j++)
                for (int i = glo[0]; i <= ghi[0]; i++) {
                    int iv[3] = {i, j, k}, w[3];
                    int out = 0;
                    for (int d = 0; d < 3; d++) {
                        int len = dhi[d] - dlo[d] + 1;
                        w[d] = iv[d];
                        if (G->is_periodic[d]) {
                            while (w[d] < dlo[d]) w[d] += len;
                            while (w[d] > dhi[d]) w[d] -= len;
                        } else if (w[d] < dlo[d] || w[d] > dhi[d]) {
                            out++;
                        }
                    }
                    size_t idx = (size_t)(i - glo[0]) + (size_t)(j - glo[1]) * n0 + (size_t)(k - glo[2]) * n0 * n1;
                    if (out) { nout[idx] = (signed char)out; continue; }
                    int src = -1;
                    if (in_box(b, w[0], w[1], w[2])) src = ib;
                    for (int ob = 0; src < 0 && ob < L.nbox; ob++)
                        if (in_box(L.boxes[ob], w[0], w[1], w[2])) src = ob;
                    nout[idx] = -1;
                    if (src < 0) continue;  // not covered at this level (unchanged)
                    A4 s(s_src ? L.boxes[src].s_new : L.boxes[src].s_old);
                    for (int n = 0; n < nc; n++) sb(i, j, k, n) = s(w[0], w[1], w[2], n);
                }
        // 2) physical boundaries: faces, then edges, then corners
        for (int stage = 1; stage <= 3; stage++)
            for (int k = glo[2]; k <= ghi[2]; k++)
                for (int j = glo[1]; j <= ghi[1]; j++)
                    for (int i = glo[0]; i <= ghi[0]; i++) {
                        size_t idx = (size_t)(i - glo[0]) + (size_t)(j - glo[1]) * n0 + (size_t)(k - glo[2]) * n0 * n1;
                        if (nout[idx] != stage) continue;
                        int iv[3] = {i, j, k};
                        bool outd[3];
                        for (int d = 0; d < 3; d++) outd[d] = !G->is_periodic[d] && (iv[d] < dlo[d] || iv[d] > dhi[d]);
                        int dstar = -1;
                        for (int d = 0; d < 3; d++) {
                            if (!outd[d]) continue;
                            int kind = (iv[d] < dlo[d]) ? P->bc_lo[d] : P->bc_hi[d];
                            if (kind == MFG_BC_EXT_DIR) dstar = d;
                        }
                        bool ext = dstar >= 0;
                        if (!ext)
                            for (int d = 0; d < 3; d++)
                                if (outd[d]) dstar = d;
                        bool lo_side = iv[dstar] < dlo[dstar];
                        int kind = lo_side ? P->bc_lo[dstar] : P->bc_hi[dstar];
                        int bnd = lo_side ? dlo[dstar] : dhi[dstar];
                        int sv[3] = {i, j, k};
                        if (ext) {
                            sv[dstar] = bnd;
                            double s_int[FLO_NVARS + MAXS], s_ext[FLO_NVARS + MAXS];
                            for (int n = 0; n < nc; n++) s_int[n] = sb.at(sv, n);
                            externalbc(c, lo_side ? P->ext_lo[dstar] : P->ext_hi[dstar], s_int, s_ext, dstar, lo_side ? +1 : -1);
                            for (int n = 0; n < nc; n++) sb(i, j, k, n) = s_ext[n];
                        } else if (kind == MFG_BC_FOEXTRAP) {
                            sv[dstar] = bnd;
                            for (int n = 0; n < nc; n++) sb(i, j, k, n) = sb.at(sv, n);
                        } else if (kind == MFG_BC_WALL) {
                            sv[dstar] = lo_side ? (2 * dlo[dstar] - iv[dstar] - 1) : (2 * dhi[dstar] - iv[dstar] + 1);
                            for (int n = 0; n < nc; n++) sb(i, j, k, n) = odd_at_wall(n) ? -sb.at(sv, n) : sb.at(sv, n);
                        } else {
#pragma omp critical
                            status = MFG_ERR_ARG;
                        }
                    }
    }
    return status;
}

// Stage algebra on the valid box, all components (mflo_evolve.cpp:283, 296-298, 309-311).
void stage_algebra(const Ctx& c, const mfg_box& b, int stage, double dt) {
    const int nc = ncomp_of(c.P);
    A4 sb(b.sborder), ds(b.dsdt), so(b.s_old), sn(b.s_new);
    for (int n = 0; n < nc; n++)
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    if (stage == 1) {
                        sn(i, j, k, n) = one * sb(i, j, k, n) + dt * ds(i, j, k, n);  // LinComb
                    } else if (stage == 2) {
                        double v = sn(i, j, k, n);
                        v += dt * ds(i, j, k, n);      // Saxpy
                        v += 3.0 * so(i, j, k, n);      // Saxpy
                        v *= fourth;                    // mult
                        sn(i, j, k, n) = v;
                    } else {
                        double v = sn(i, j, k, n);
                        v += dt * ds(i, j, k, n);      // Saxpy
                        v = so(i, j, k, n) + two * v;  // Xpay: dst = src + a*dst
                        v *= third;                     // mult
                        sn(i, j, k, n) = v;
                    }
                }
}

void copy_valid(const mfg_box& b, const mfg_array4& dst, const mfg_array4& src, int nc) {
    A4 d(dst), s(src);
    for (int n = 0; n < nc; n++)
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) d(i, j, k, n) = s(i, j, k, n);
}

void chem_rhs_box(const Ctx& c, const mfg_box& b, const A4& S, const A4& F) {
    const int ns = c.nspec, nc = FLO_NVARS + ns;
    for (int k = b.lo[2]; k <= b.hi[2]; k++)
        for (int j = b.lo[1]; j <= b.hi[1]; j++)
            for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                double spec[MAXS], wdot[MAXS];
                for (int sp = 0; sp < ns; sp++) spec[sp] = S(i, j, k, FLO_NVARS + sp);
                compute_spec_source(c, spec, S(i, j, k, TEMP_INDX), wdot);
                for (int n = 0; n < FLO_NVARS; n++) F(i, j, k, n) = zeroval;
                for (int sp = 0; sp < ns; sp++) F(i, j, k, FLO_NVARS + sp) = zeroval + (zeroval + wdot[sp]);
                (void)nc;
            }
}

struct ValidFab {
    std::vector<double> v;
    mfg_array4 a;
    void define(const mfg_box& b, int nc) {
        int n0 = b.hi[0] - b.lo[0] + 1, n1 = b.hi[1] - b.lo[1] + 1, n2 = b.hi[2] - b.lo[2] + 1;
        v.assign((size_t)n0 * n1 * n2 * nc, 0.0);
        a.p = v.data();
        a.jstride = n0;
        a.kstride = (int64_t)n0 * n1;
        a.nstride = (int64_t)n0 * n1 * n2;
        for (int d = 0; d < 3; d++) { a.begin[d] = b.lo[d]; a.end[d] = b.hi[d] + 1; }
        a.ncomp = nc;
    }
};

// AMReX TimeIntegrator, RungeKutta rk.type=3 = SSP-RK3 (nodes 0,1,1/2;
// a21=1, a31=a32=1/4; weights 1/6,1/6,2/3), restated from AMReX's
// RKIntegrator::advance: stage state = S_old + sum_j (h*a_ij) F_j, new
// state = S_old + sum_i (h*w_i) F_i.  Unpinned (AMReX not vendored).
int chem_substep(const Ctx& c, const Level& L, double dt) {
    const int nc = ncomp_of(c.P);
    static const double tab[3][3] = {{0, 0, 0}, {1.0, 0, 0}, {0.25, 0.25, 0}};
    static const double w[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        ValidFab F[3], S;
        for (int s = 0; s < 3; s++) F[s].define(b, nc);
        S.define(b, nc);
        A4 so(b.s_old), sn(b.s_new), Sa(S.a);
        for (int st = 0; st < 3; st++) {
            copy_valid(b, S.a, b.s_old, nc);
            for (int jj = 0; jj < st; jj++) {
                double coef = dt * tab[st][jj];
                A4 f(F[jj].a);
                for (int n = 0; n < nc; n++)
                    for (int k = b.lo[2]; k <= b.hi[2]; k++)
                        for (int j = b.lo[1]; j <= b.hi[1]; j++)
                            for (int i = b.lo[0]; i <= b.hi[0]; i++) Sa(i, j, k, n) += coef * f(i, j, k, n);
            }
            chem_rhs_box(c, b, Sa, A4(F[st].a));
        }
        copy_valid(b, b.s_new, b.s_old, nc);
        for (int st = 0; st < 3; st++) {
            double coef = dt * w[st];
            A4 f(F[st].a);
            for (int n = 0; n < nc; n++)
                for (int k = b.lo[2]; k <= b.hi[2]; k++)
                    for (int j = b.lo[1]; j <= b.hi[1]; j++)
                        for (int i = b.lo[0]; i <= b.hi[0]; i++) sn(i, j, k, n) += coef * f(i, j, k, n);
        }
    }
    return MFG_OK;
}

int update_prims(const Ctx& c, const Level& L) {  // mflo_evolve.cpp:114-171
    const int ns = c.nspec;
    int status = MFG_OK;
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 s(b.s_new);
        double minp = 1e300;
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    if (s(i, j, k, VFRAC_INDX) == one) {
                        double u[MAXC], p[NCVARS];
                        for (int q = 0; q < NCVARS; q++) u[q] = s(i, j, k, q);
                        for (int q = 0; q < ns; q++) u[q + NCVARS] = s(i, j, k, q + FLO_NVARS);
                        cons_to_prim(c, u, p);
                        for (int q = 0; q < NCVARS; q++) s(i, j, k, q + DENS_INDX) = p[q];
                        s(i, j, k, TEMP_INDX) = get_t_from_rpc(c, s(i, j, k, DENS_INDX), s(i, j, k, PRES_INDX), u + NCVARS);
                    } else if (c.P->conj_ht && s(i, j, k, VFRAC_INDX) == zeroval) {
                        s(i, j, k, TEMP_INDX) = c.P->solid_temp;
                    }
                    minp = std::min(minp, s(i, j, k, PRES_INDX));
                }
        if (minp < 0 && c.P->do_ns) status = MFG_ERR_NEG_PRESSURE;
    }
    return status;
}

void clip_species(const Ctx& c, const Level& L) {  // mflo_evolve.cpp:521-540
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 s(b.s_new);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++)
                    for (int sp = 0; sp < c.nspec; sp++)
                        if (s(i, j, k, FLO_NVARS + sp) < 0.0) s(i, j, k, FLO_NVARS + sp) = 0.0;
    }
}

void residual_norms(const Ctx& c, const Level& L, double dt, double* out) {  // mflo_evolve.cpp:91-112
    const int nc = ncomp_of(c.P);
    std::vector<double> acc(nc, 0.0);
    double a = 1.0 / dt, bcoef = -1.0 / dt;
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 sn(b.s_new), so(b.s_old);
        for (int n = 0; n < nc; n++)
            for (int k = b.lo[2]; k <= b.hi[2]; k++)
                for (int j = b.lo[1]; j <= b.hi[1]; j++)
                    for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                        double d = a * sn(i, j, k, n) + bcoef * so(i, j, k, n);
                        if (n >= RHO_INDX && n < VFRAC_INDX) d *= so(i, j, k, VFRAC_INDX);
                        acc[n] += d * d;
                    }
    }
    for (int n = 0; n < nc; n++) out[n] = std::sqrt(acc[n]);
}

double est_timestep(const Ctx& c, const Level& L) {  // mflo_timestep.cpp:53-153
    const mfg_params* P = c.P;
    const double* dx = L.G->dx;
    double max_ws = 0.0, max_sd = 0.0;  // MultiFab::norm0 = max |x|
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 s(b.s_new);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    double ws = zeroval;
                    if (s(i, j, k, VFRAC_INDX) > zeroval) {
                        double fs = std::sqrt(s(i, j, k, VELX_INDX) * s(i, j, k, VELX_INDX) +
                                              s(i, j, k, VELY_INDX) * s(i, j, k, VELY_INDX) +
                                              s(i, j, k, VELZ_INDX) * s(i, j, k, VELZ_INDX));
                        double spec[MAXS];
                        for (int sp = 0; sp < c.nspec; sp++) spec[sp] = s(i, j, k, FLO_NVARS + sp);
                        double gama = get_gama_from_rpc(c, s(i, j, k, DENS_INDX), s(i, j, k, PRES_INDX), spec);
                        double ss = std::sqrt(gama * s(i, j, k, PRES_INDX) / s(i, j, k, DENS_INDX));
                        ws = fs + double(P->do_ns) * ss;
                    }
                    max_ws = std::max(max_ws, std::fabs(ws));
                    int iv[3] = {i, j, k};
                    double md = diff_at(c, s, iv, 0);
                    for (int sp = 0; sp < c.nspec; sp++) {
                        double dsp = diff_at(c, s, iv, sp);
                        if (dsp > md) md = dsp;
                    }
                    max_sd = std::max(max_sd, std::fabs(md));
                }
    }
    double dt_est = 1.7976931348623157e308;
    if (max_ws > 0)
        for (int i = 0; i < 3; i++) dt_est = std::min(dt_est, dx[i] / max_ws);
    if (max_sd > 0)
        for (int i = 0; i < 3; i++) dt_est = std::min(dt_est, half * dx[i] * dx[i] / max_sd / 3);
    dt_est *= P->cfl;
    return dt_est;
}

}  // namespace

extern "C" {

int oracle_compute_dsdt(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    int status = MFG_OK;
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < nbox; ib++) {
        int rc = dsdt_box(c, G, boxes[ib]);
        if (rc) {
#pragma omp critical
            status = rc;
        }
    }
    return status;
}

int oracle_cutcells(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 phi(b.sborder);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) update_cutcells(c, i, j, k, phi, G->dx);
    }
    return MFG_OK;
}

int oracle_stage_algebra(const mfg_params* P, const mfg_box* boxes, int nbox, int stage, double dt) {
    Ctx c{P, P->nspec};
    for (int ib = 0; ib < nbox; ib++) stage_algebra(c, boxes[ib], stage, dt);
    return MFG_OK;
}

int oracle_fill_patch(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox, int s_src,
                      double time) {
    Ctx c{P, P->nspec};
    Level L{P, G, boxes, nbox};
    return fill_patch(c, L, s_src, time);
}

int oracle_chem_source(const mfg_params* P, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 S(b.s_new), D(b.dsdt);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    double spec[MAXS], wdot[MAXS];
                    for (int sp = 0; sp < c.nspec; sp++) spec[sp] = S(i, j, k, FLO_NVARS + sp);
                    compute_spec_source(c, spec, S(i, j, k, TEMP_INDX), wdot);
                    for (int sp = 0; sp < c.nspec; sp++) D(i, j, k, FLO_NVARS + sp) += (zeroval + wdot[sp]);
                }
    }
    return MFG_OK;
}

int oracle_chem_substep(const mfg_params* P, const mfg_box* boxes, int nbox, double dt) {
    Ctx c{P, P->nspec};
    Level L{P, nullptr, boxes, nbox};
    return chem_substep(c, L, dt);
}

int oracle_update_primitive_vars(const mfg_params* P, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    Level L{P, nullptr, boxes, nbox};
    return update_prims(c, L);
}

int oracle_clip_species(const mfg_params* P, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    Level L{P, nullptr, boxes, nbox};
    clip_species(c, L);
    return MFG_OK;
}

int oracle_residual_norms(const mfg_params* P, const mfg_box* boxes, int nbox, double dt, double* out) {
    Ctx c{P, P->nspec};
    Level L{P, nullptr, boxes, nbox};
    residual_norms(c, L, dt, out);
    return MFG_OK;
}

int oracle_est_timestep(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox, double* dt_out) {
    Ctx c{P, P->nspec};
    Level L{P, G, boxes, nbox};
    *dt_out = est_timestep(c, L);
    return MFG_OK;
}

// One coarse step of a single-level run (Source/mflo_evolve.cpp:251-318 plus
// the bookends of EvolveAMR :33-58).  On entry box.s_new holds phi_new; on
// exit box.s_new holds the new state and box.s_old phi_old (the post-flow
// state when chemistry runs, as the reference's second swap :473).
// sborder and dsdt are workspace.  resnorms (ncomp) may be NULL.
int oracle_advance(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox, double time, double dt,
                   int only_flow, int clip, double* resnorms) {
    Ctx c{P, P->nspec};
    Level L{P, G, boxes, nbox};
    const int nc = ncomp_of(P);
    int rc;
    for (int ib = 0; ib < nbox; ib++) copy_valid(boxes[ib], boxes[ib].s_old, boxes[ib].s_new, nc);  // swap
    for (int stage = 1; stage <= 3; stage++) {
        rc = fill_patch(c, L, stage == 1 ? 0 : 1, stage == 1 ? time : time + dt);
        if (rc) return rc;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nbox; ib++) {
            const mfg_box& b = boxes[ib];
            A4 phi(b.sborder);
            for (int k = b.lo[2]; k <= b.hi[2]; k++)
                for (int j = b.lo[1]; j <= b.hi[1]; j++)
                    for (int i = b.lo[0]; i <= b.hi[0]; i++) update_cutcells(c, i, j, k, phi, G->dx);
        }
        int st = MFG_OK;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nbox; ib++) {
            int r = dsdt_box(c, G, boxes[ib]);
            if (r) {
#pragma omp critical
                st = r;
            }
        }
        if (st) return st;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nbox; ib++) stage_algebra(c, boxes[ib], stage, dt);
    }
    if (!only_flow) {
        for (int ib = 0; ib < nbox; ib++) copy_valid(boxes[ib], boxes[ib].s_old, boxes[ib].s_new, nc);  // swap
        rc = chem_substep(c, L, dt);
        if (rc) return rc;
    }
    rc = update_prims(c, L);
    if (rc) return rc;
    if (clip) clip_species(c, L);
    if (resnorms) residual_norms(c, L, dt, resnorms);
    return MFG_OK;
}

// FP64 operation counts are measured with a counting build; this is the
// plain-double library.
const char* oracle_build_info(void) {
#ifdef __FP_FAST_FMA
    return "oracle: fma-contracting build";
#else
    return "oracle: strict IEEE build";
#endif
}

}  // extern "C"

// Sizes and offsets of the C ABI structures, for the ctypes layout check.
#include <cstddef>
extern "C" int oracle_abi_layout(int64_t* out, int n) {
    const int64_t v[] = {
        (int64_t)sizeof(mfg_array4), (int64_t)sizeof(mfg_box), (int64_t)sizeof(mfg_geom),
        (int64_t)sizeof(mfg_extbc), (int64_t)sizeof(mfg_params),
        (int64_t)offsetof(mfg_box, flux), (int64_t)offsetof(mfg_box, level),
        (int64_t)offsetof(mfg_params, order_hyp), (int64_t)offsetof(mfg_params, nu),
        (int64_t)offsetof(mfg_params, bc_lo), (int64_t)offsetof(mfg_params, ext_hi),
        (int64_t)offsetof(mfg_extbc, state), (int64_t)offsetof(mfg_params, cfl),
    };
    int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < m && i < n; i++) out[i] = v[i];
    return m;
}

// Integrated surface reaction rate J = V_cell * sum_cells sum_r rate_r (the
// differentiation objective): rate_r = k_r(T) prod_j c_j^order_rj on s_new,
// k_r = A_r exp(-Ea_r/(RU T)), T the temperature component.
extern "C" int oracle_objective(const mfg_params* P, const mfg_geom* G, const mfg_box* boxes, int nbox, double* J) {
    double acc = 0.0;
    const double vol = G->dx[0] * G->dx[1] * G->dx[2];
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 s(b.s_new);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    double cell = 0.0;
                    for (int r = 0; r < P->nreact; r++) {
                        double cm = 1.0;
                        for (int sp = 0; sp < P->nspec; sp++)
                            if (P->order[r][sp] > 0.0) cm *= std::pow(s(i, j, k, FLO_NVARS + sp), P->order[r][sp]);
                        double kr = P->A[r];
                        if (P->Ea[r] != 0.0) kr = P->A[r] * std::exp(-P->Ea[r] / (RU * s(i, j, k, TEMP_INDX)));
                        cell += kr * cm;
                    }
                    acc += cell;
                }
    }
    *J = acc * vol;
    return MFG_OK;
}
