// ORACLE — test infrastructure only (see mflo_oracle.hpp).  C API over the
// restatement, operating on host arrays described by the same mfg_box /
// mfg_array4 views as the product's C ABI, plus a single-level driver that
// restates mflo::Advance_coupled_strang and the step bookends.
#include <cstdio>
#include <cstdlib>
#include <array>
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

// keep (optional): receives the three face-flux FABs (the multi-level step's
// flux registers read them).
int dsdt_box(const Ctx& c, const mfg_geom* G, const mfg_box& b, FluxFab* keep = nullptr) {
    const int nc = ncomp_of(c.P);
    A4 phi(b.sborder), dsdt(b.dsdt);
    FluxFab local[3];
    FluxFab* F = keep ? keep : local;
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
    if (E.kind == MFG_EXT_SPECIES_DIRICHLET) {
        // tests/Cartesian/SpeciesEqTests/externbc.H:20-52: flow from the
        // interior, vfrac one, species reflected about the boundary value
        // (models/blockCatalyst1d/externbc.H:18-55 keeps VFRAC and copies S2)
        for (int n = 0; n < FLO_NVARS; n++) s_ext[n] = s_int[n];
        if (!E.vfrac_interior) s_ext[VFRAC_INDX] = one;
        for (int sp = 0; sp < ns; sp++)
            s_ext[FLO_NVARS + sp] = ((E.spec_zero_grad_mask >> sp) & 1) ? s_int[FLO_NVARS + sp]
                                                                       : two * E.spec[sp] - s_int[FLO_NVARS + sp];
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

// Physical boundaries of the cells of [glo, ghi] that lie outside the domain
// of G in non-periodic directions: faces, then edges, then corners, each from
// the array itself (the rule of the comment above).
int physbc_region(const Ctx& c, const mfg_geom* G, const A4& sb, const int glo[3], const int ghi[3]) {
    const mfg_params* P = c.P;
    const int nc = ncomp_of(P);
    const int* dlo = G->domain_lo;
    const int* dhi = G->domain_hi;
    int status = MFG_OK;
    for (int stage = 1; stage <= 3; stage++)
        for (int k = glo[2]; k <= ghi[2]; k++)
            for (int j = glo[1]; j <= ghi[1]; j++)
                for (int i = glo[0]; i <= ghi[0]; i++) {
                    int iv[3] = {i, j, k};
                    bool outd[3];
                    int nout = 0;
                    for (int d = 0; d < 3; d++) {
                        outd[d] = !G->is_periodic[d] && (iv[d] < dlo[d] || iv[d] > dhi[d]);
                        nout += outd[d];
                    }
                    if (nout != stage) continue;
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
                        status = MFG_ERR_ARG;
                    }
                }
    return status;
}

// Periodic image of iv inside the domain of G; false if iv lies outside in a
// non-periodic direction.
inline bool wrap_into(const mfg_geom* G, const int iv[3], int w[3]) {
    bool inside = true;
    for (int d = 0; d < 3; d++) {
        const int len = G->domain_hi[d] - G->domain_lo[d] + 1;
        w[d] = iv[d];
        if (G->is_periodic[d]) {
            while (w[d] < G->domain_lo[d]) w[d] += len;
            while (w[d] > G->domain_hi[d]) w[d] -= len;
        } else if (w[d] < G->domain_lo[d] || w[d] > G->domain_hi[d]) {
            inside = false;
        }
    }
    return inside;
}

int owner_of(const mfg_box* boxes, int nbox, const int w[3], int first = -1) {
    if (first >= 0 && in_box(boxes[first], w[0], w[1], w[2])) return first;
    for (int ob = 0; ob < nbox; ob++)
        if (in_box(boxes[ob], w[0], w[1], w[2])) return ob;
    return -1;
}

int fill_patch(const Ctx& c, const Level& L, int s_src, double time) {
    (void)time;
    const int nc = ncomp_of(c.P);
    int status = MFG_OK;
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < L.nbox; ib++) {
        const mfg_box& b = L.boxes[ib];
        A4 sb(b.sborder);
        int glo[3], ghi[3];
        for (int d = 0; d < 3; d++) { glo[d] = b.lo[d] - MFG_NGROW; ghi[d] = b.hi[d] + MFG_NGROW; }
        // 1) copy valid data (own box + other boxes + periodic images); cells
        //    not covered at this level stay unchanged
        for (int k = glo[2]; k <= ghi[2]; k++)
            for (int j = glo[1]; j <= ghi[1]; j++)
                for (int i = glo[0]; i <= ghi[0]; i++) {
                    int iv[3] = {i, j, k}, w[3];
                    if (!wrap_into(L.G, iv, w)) continue;
                    const int src = owner_of(L.boxes, L.nbox, w, ib);
                    if (src < 0) continue;
                    A4 s(s_src ? L.boxes[src].s_new : L.boxes[src].s_old);
                    for (int n = 0; n < nc; n++) sb(i, j, k, n) = s(w[0], w[1], w[2], n);
                }
        // 2) physical boundaries: faces, then edges, then corners
        const int rc = physbc_region(c, L.G, sb, glo, ghi);
        if (rc) {
#pragma omp critical
            status = rc;
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

// ---- multi-level step ------------------------------------------------------
// mflo::timeStep / Advance_coupled_strang (Source/mflo_evolve.cpp:174-311)
// with the AMReX pieces they call, restated from AMReX's published semantics
// (AMReX is not vendored in the reference, so this part is unpinned):
//  * GetData (Source/mflo.cpp:310-330): data at `time` is phi_new or phi_old
//    when within 1e-3 dt of t_new / t_old, else the two in linear
//    combination (t1-time)/(t1-t0) old + (time-t0)/(t1-t0) new
//    (FillPatchSingleLevel with two time levels);
//  * FillPatchTwoLevels (Source/mflo_gridwork.cpp:135-173): ghost cells of a
//    fine box that lie inside the (periodically extended) domain and are not
//    covered by the fine level are interpolated with cell_cons_interp from a
//    coarse patch (the coarsened grown box, grown by one) filled from the
//    coarse level at `time` plus the coarse physical boundaries; then the fine
//    level's valid data is copied and the fine physical boundaries applied;
//  * cell_cons_interp = CellConservativeLinear without cross-component
//    limiting: per component MC-limited central slopes (one-sided 4-point
//    slopes at ext_dir domain faces), scaled by one factor per coarse cell and
//    component that keeps every fine value within the 27-neighbour coarse
//    bounds, fine = crse + sum_d off_d slope_d;
//  * FluxRegister: CrseInit(ADD) adds scale x coarse flux, FineAdd adds
//    scale x each of the ratio^2 fine faces (higher transverse direction
//    outer), Reflux visits the orientations x-lo, y-lo, z-lo, x-hi, y-hi,
//    z-hi and adds -reg/vol (lo) or +reg/vol (hi) to the coarse cell outside
//    the fine box (registers whose outside cell is covered by the fine level
//    or lies outside the domain change nothing that average_down keeps);
//  * average_down: covered coarse cell = (1/ratio^3) x the sum of its fine
//    cells (k, j, i order), every component.
inline int floor_div(int a, int r) { return a >= 0 ? a / r : -((-a + r - 1) / r); }

struct RegEnt {
    int fb, cb, d, side;
    int cc[3], cf[3], ff[3];
    std::vector<double> v;
};

struct Amr {
    const mfg_params* P;
    Ctx c;
    int nlev, nc;
    std::vector<const mfg_geom*> G;
    std::vector<int> ratio;                    // to the coarser level ([0] = 1)
    std::vector<std::vector<mfg_box>> lv;      // boxes per level
    std::vector<std::vector<std::array<FluxFab, 3>>> flux;
    std::vector<std::vector<RegEnt>> reg;      // [l]: registers of the l / l-1 interface
    std::vector<double> t_old, t_new, dt;
    bool only_flow;
};

// cell_cons_interp of component n at fine cell (i, j, k) from the coarse patch u.
double cc_interp(const Amr& A, int l, const A4& u, const int cplo[3], const int cphi[3], int i, int j, int k, int n) {
    const mfg_params* P = A.P;
    const mfg_geom* Gc = A.G[l - 1];
    const int r = A.ratio[l];
    const int ic[3] = {floor_div(i, r), floor_div(j, r), floor_div(k, r)};
    const int fv[3] = {i, j, k};
    auto U = [&](int d, int o) {
        int q[3] = {ic[0], ic[1], ic[2]};
        q[d] += o;
        return u(q[0], q[1], q[2], n);
    };
    const double u0 = u(ic[0], ic[1], ic[2], n);
    double sl[3];
    for (int d = 0; d < 3; d++) {
        double dc = 0.5 * (U(d, 1) - U(d, -1));
        if (!Gc->is_periodic[d] && ic[d] == Gc->domain_lo[d] && P->bc_lo[d] == MFG_BC_EXT_DIR) {
            if (ic[d] + 2 <= cphi[d])
                dc = -16. / 15. * U(d, -1) + 0.5 * u0 + 2. / 3. * U(d, 1) - 0.1 * U(d, 2);
            else
                dc = 0.25 * (U(d, 1) + 5. * u0 - 6. * U(d, -1));
        }
        if (!Gc->is_periodic[d] && ic[d] == Gc->domain_hi[d] && P->bc_hi[d] == MFG_BC_EXT_DIR) {
            if (ic[d] - 2 >= cplo[d])
                dc = 16. / 15. * U(d, 1) - 0.5 * u0 - 2. / 3. * U(d, -1) + 0.1 * U(d, -2);
            else
                dc = -0.25 * (U(d, -1) + 5. * u0 - 6. * U(d, 1));
        }
        const double df = 2.0 * (U(d, 1) - u0);
        const double db = 2.0 * (u0 - U(d, -1));
        double sx = (df * db >= 0.0) ? std::min(std::fabs(df), std::fabs(db)) : 0.0;
        sx = std::copysign(1.0, dc) * std::min(sx, std::fabs(dc));
        sl[d] = sx;
    }
    double alpha = 1.0;
    if (sl[0] != 0.0 || sl[1] != 0.0 || sl[2] != 0.0) {
        const double f = (double)(r - 1);
        const double g = (double)(2 * r);
        const double dumax = std::fabs(sl[0]) * f / g + std::fabs(sl[1]) * f / g + std::fabs(sl[2]) * f / g;
        double umax = u0, umin = u0;
        for (int kk = -1; kk <= 1; kk++)
            for (int jj = -1; jj <= 1; jj++)
                for (int ii = -1; ii <= 1; ii++) {
                    const double x = u(ic[0] + ii, ic[1] + jj, ic[2] + kk, n);
                    umin = std::min(umin, x);
                    umax = std::max(umax, x);
                }
        if (dumax * alpha > (umax - u0)) alpha = (umax - u0) / dumax;
        if (dumax * alpha > (u0 - umin)) alpha = (u0 - umin) / dumax;
    }
    double off[3];
    for (int d = 0; d < 3; d++) off[d] = (fv[d] - ic[d] * r + 0.5) / (double)r - 0.5;
    return u0 + off[0] * (sl[0] * alpha) + off[1] * (sl[1] * alpha) + off[2] * (sl[2] * alpha);
}

// Data of level l at time T: 0 old, 1 new, 2 a*old + b*new.
int get_data(const Amr& A, int l, double T, double& a, double& b) {
    const double teps = (A.t_new[l] - A.t_old[l]) * 1.e-3;
    if (T > A.t_new[l] - teps && T < A.t_new[l] + teps) return 1;
    if (T > A.t_old[l] - teps && T < A.t_old[l] + teps) return 0;
    const double t0 = A.t_old[l], t1 = A.t_new[l];
    a = (t1 - T) / (t1 - t0);
    b = (T - t0) / (t1 - t0);
    return 2;
}

int fill_level(Amr& A, int l, int s_src, double T) {
    const int nc = A.nc;
    std::vector<mfg_box>& bl = A.lv[l];
    const int nb = (int)bl.size();
    double ca = 0.0, cb = 0.0;
    const int ckind = l > 0 ? get_data(A, l - 1, T, ca, cb) : 0;
    int status = MFG_OK;
#pragma omp parallel for schedule(dynamic)
    for (int ib = 0; ib < nb; ib++) {
        const mfg_box& b = bl[ib];
        A4 sb(b.sborder);
        int glo[3], ghi[3];
        for (int d = 0; d < 3; d++) { glo[d] = b.lo[d] - MFG_NGROW; ghi[d] = b.hi[d] + MFG_NGROW; }
        std::vector<double> cpv;
        A4 cp;
        int clo[3] = {0, 0, 0}, chi[3] = {0, 0, 0};
        int rc = MFG_OK;
        if (l > 0) {  // coarse patch at time T
            const int r = A.ratio[l];
            const std::vector<mfg_box>& cl = A.lv[l - 1];
            size_t len[3];
            for (int d = 0; d < 3; d++) {
                clo[d] = floor_div(glo[d], r) - 1;
                chi[d] = floor_div(ghi[d], r) + 1;
                len[d] = (size_t)(chi[d] - clo[d] + 1);
            }
            cpv.assign(len[0] * len[1] * len[2] * nc, 0.0);
            cp.p = cpv.data();
            cp.js = (int64_t)len[0];
            cp.ks = (int64_t)(len[0] * len[1]);
            cp.ns = (int64_t)(len[0] * len[1] * len[2]);
            cp.b0 = clo[0]; cp.b1 = clo[1]; cp.b2 = clo[2];
            int hint = -1;
            for (int k = clo[2]; k <= chi[2]; k++)
                for (int j = clo[1]; j <= chi[1]; j++)
                    for (int i = clo[0]; i <= chi[0]; i++) {
                        int iv[3] = {i, j, k}, w[3];
                        if (!wrap_into(A.G[l - 1], iv, w)) continue;
                        const int src = owner_of(cl.data(), (int)cl.size(), w, hint);
                        if (src < 0) { rc = MFG_ERR_ARG; continue; }  // not properly nested
                        hint = src;
                        A4 so(cl[src].s_old), sn(cl[src].s_new);
                        for (int n = 0; n < nc; n++) {
                            const double x0 = so(w[0], w[1], w[2], n), x1 = sn(w[0], w[1], w[2], n);
                            cp(i, j, k, n) = ckind == 0 ? x0 : ckind == 1 ? x1 : ca * x0 + cb * x1;
                        }
                    }
            const int r2 = physbc_region(A.c, A.G[l - 1], cp, clo, chi);
            if (r2) rc = r2;
        }
        int hint = ib;
        for (int k = glo[2]; k <= ghi[2]; k++)
            for (int j = glo[1]; j <= ghi[1]; j++)
                for (int i = glo[0]; i <= ghi[0]; i++) {
                    int iv[3] = {i, j, k}, w[3];
                    if (!wrap_into(A.G[l], iv, w)) continue;
                    const int src = owner_of(bl.data(), nb, w, hint);
                    if (src >= 0) {
                        hint = src;
                        A4 s(s_src ? bl[src].s_new : bl[src].s_old);
                        for (int n = 0; n < nc; n++) sb(i, j, k, n) = s(w[0], w[1], w[2], n);
                    } else if (l > 0) {
                        for (int n = 0; n < nc; n++) sb(i, j, k, n) = cc_interp(A, l, cp, clo, chi, i, j, k, n);
                    }
                }
        const int r3 = physbc_region(A.c, A.G[l], sb, glo, ghi);
        if (r3) rc = r3;
        if (rc) {
#pragma omp critical
            status = rc;
        }
    }
    return status;
}

// Registers of the interface between level l (fine) and l-1.
int build_registers(Amr& A, int l) {
    const int r = A.ratio[l];
    const mfg_geom* Gc = A.G[l - 1];
    const std::vector<mfg_box>& fl = A.lv[l];
    const std::vector<mfg_box>& cl = A.lv[l - 1];
    A.reg[l].clear();
    for (int side = 0; side < 2; side++)
        for (int d = 0; d < 3; d++)
            for (int fb = 0; fb < (int)fl.size(); fb++) {
                const mfg_box& b = fl[fb];
                const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
                const int fface = side ? b.hi[d] + 1 : b.lo[d];
                const int cface = floor_div(fface, r);
                for (int q2 = floor_div(b.lo[t2], r); q2 <= floor_div(b.hi[t2] + 1, r) - 1; q2++)
                    for (int q1 = floor_div(b.lo[t1], r); q1 <= floor_div(b.hi[t1] + 1, r) - 1; q1++) {
                        int cc[3];
                        cc[d] = side ? cface : cface - 1;
                        cc[t1] = q1;
                        cc[t2] = q2;
                        int w[3];
                        if (!wrap_into(Gc, cc, w)) continue;
                        const int fw[3] = {w[0] * r, w[1] * r, w[2] * r};
                        if (owner_of(fl.data(), (int)fl.size(), fw) >= 0) continue;  // covered
                        const int cb = owner_of(cl.data(), (int)cl.size(), w);
                        if (cb < 0) return MFG_ERR_ARG;
                        RegEnt e;
                        e.fb = fb;
                        e.cb = cb;
                        e.d = d;
                        e.side = side;
                        for (int q = 0; q < 3; q++) { e.cc[q] = w[q]; e.cf[q] = w[q]; }
                        e.cf[d] = side ? w[d] : w[d] + 1;
                        e.ff[d] = fface;
                        e.ff[t1] = q1 * r;
                        e.ff[t2] = q2 * r;
                        e.v.assign(A.nc, 0.0);
                        A.reg[l].push_back(std::move(e));
                    }
            }
    return MFG_OK;
}

void reg_zero(Amr& A, int l) {
    for (RegEnt& e : A.reg[l]) std::fill(e.v.begin(), e.v.end(), 0.0);
}

void reg_crse(Amr& A, int l, const double scale[3]) {  // registers of l+1 from level l's fluxes
    for (RegEnt& e : A.reg[l + 1]) {
        const A4& F = A.flux[l][e.cb][e.d].a;
        for (int n = 0; n < A.nc; n++) e.v[n] = e.v[n] + F(e.cf[0], e.cf[1], e.cf[2], n) * scale[e.d];
    }
}

void reg_fine(Amr& A, int l, const double scale[3]) {  // registers of l from level l's fluxes
    const int r = A.ratio[l];
    for (RegEnt& e : A.reg[l]) {
        const A4& F = A.flux[l][e.fb][e.d].a;
        const int t1 = e.d == 0 ? 1 : 0, t2 = e.d == 2 ? 1 : 2;
        for (int n = 0; n < A.nc; n++)
            for (int o2 = 0; o2 < r; o2++)
                for (int o1 = 0; o1 < r; o1++) {
                    int q[3] = {e.ff[0], e.ff[1], e.ff[2]};
                    q[t1] += o1;
                    q[t2] += o2;
                    e.v[n] = e.v[n] + scale[e.d] * F(q[0], q[1], q[2], n);
                }
    }
}

void reflux(Amr& A, int l) {  // level l from the registers of l+1
    const double* dx = A.G[l]->dx;
    const double vol = dx[0] * dx[1] * dx[2];
    for (int o = 0; o < 6; o++)
        for (RegEnt& e : A.reg[l + 1]) {
            if (e.d + 3 * e.side != o) continue;
            A4 s(A.lv[l][e.cb].s_new);
            for (int n = 0; n < A.nc; n++) {
                double& x = s(e.cc[0], e.cc[1], e.cc[2], n);
                x += e.side ? (1.0 * e.v[n]) / vol : (-1.0 * e.v[n]) / vol;
            }
        }
}

int average_down(Amr& A, int l) {  // level l+1 onto level l
    const int r = A.ratio[l + 1];
    const double volfrac = 1.0 / (double)(r * r * r);
    const std::vector<mfg_box>& cl = A.lv[l];
    for (const mfg_box& b : A.lv[l + 1]) {
        A4 f(b.s_new);
        for (int k = floor_div(b.lo[2], r); k <= floor_div(b.hi[2] + 1, r) - 1; k++)
            for (int j = floor_div(b.lo[1], r); j <= floor_div(b.hi[1] + 1, r) - 1; j++)
                for (int i = floor_div(b.lo[0], r); i <= floor_div(b.hi[0] + 1, r) - 1; i++) {
                    const int w[3] = {i, j, k};
                    const int cb = owner_of(cl.data(), (int)cl.size(), w);
                    if (cb < 0) return MFG_ERR_ARG;
                    A4 s(cl[cb].s_new);
                    for (int n = 0; n < A.nc; n++) {
                        double c = 0.;
                        for (int kr = 0; kr < r; kr++)
                            for (int jr = 0; jr < r; jr++)
                                for (int ir = 0; ir < r; ir++) c += f(i * r + ir, j * r + jr, k * r + kr, n);
                        s(i, j, k, n) = volfrac * c;
                    }
                }
    }
    return MFG_OK;
}

int amr_advance(Amr& A, int l, double time, double dtl) {
    std::vector<mfg_box>& bl = A.lv[l];
    const int nb = (int)bl.size();
    for (int ib = 0; ib < nb; ib++) copy_valid(bl[ib], bl[ib].s_old, bl[ib].s_new, A.nc);  // swap
    A.t_old[l] = A.t_new[l];
    A.t_new[l] += dtl;
    if (l + 1 < A.nlev) reg_zero(A, l + 1);
    const double* dx = A.G[l]->dx;
    const double dA[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
    Level L{A.P, A.G[l], bl.data(), nb};
    for (int stage = 1; stage <= 3; stage++) {
        int rc = fill_level(A, l, stage == 1 ? 0 : 1, stage == 1 ? time : time + dtl);
        if (rc) return rc;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nb; ib++) {
            const mfg_box& b = bl[ib];
            A4 phi(b.sborder);
            for (int k = b.lo[2]; k <= b.hi[2]; k++)
                for (int j = b.lo[1]; j <= b.hi[1]; j++)
                    for (int i = b.lo[0]; i <= b.hi[0]; i++) update_cutcells(A.c, i, j, k, phi, dx);
        }
        int st = MFG_OK;
#pragma omp parallel for schedule(dynamic)
        for (int ib = 0; ib < nb; ib++) {
            int r = dsdt_box(A.c, A.G[l], bl[ib], A.flux[l][ib].data());
            if (r) {
#pragma omp critical
                st = r;
            }
        }
        if (st) return st;
        for (int ib = 0; ib < nb; ib++) stage_algebra(A.c, bl[ib], stage, dtl);
        const double ff = stage < 3 ? sixth : two3rd;
        if (l + 1 < A.nlev) {
            const double sc[3] = {-dtl * dA[0] * ff, -dtl * dA[1] * ff, -dtl * dA[2] * ff};
            reg_crse(A, l, sc);
        }
        if (l > 0) {
            const double sc[3] = {dtl * dA[0] * ff, dtl * dA[1] * ff, dtl * dA[2] * ff};
            reg_fine(A, l, sc);
        }
    }
    if (!A.only_flow) {
        for (int ib = 0; ib < nb; ib++) copy_valid(bl[ib], bl[ib].s_old, bl[ib].s_new, A.nc);  // swap
        int rc = chem_substep(A.c, L, dtl);
        if (rc) return rc;
    }
    return MFG_OK;
}

int amr_time_step(Amr& A, int l, double time) {
    int rc = amr_advance(A, l, time, A.dt[l]);
    if (rc) return rc;
    if (l + 1 < A.nlev) {
        for (int i = 1; i <= A.ratio[l + 1]; i++)
            if ((rc = amr_time_step(A, l + 1, time + (i - 1) * A.dt[l + 1]))) return rc;
        reflux(A, l);
        if ((rc = average_down(A, l))) return rc;
    }
    return MFG_OK;
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

// Implicit chemistry sub-step (the product's ROS2 option, which stands in for
// the reference's SUNDIALS CVODE path): per cell, over dt, the adaptive
// second-order Rosenbrock method with the analytic mass-action Jacobian,
// restated from Verwer et al. (1999) with the same step control as the
// product: RMS error norm of h (k1 + k2)/2 against atol + rtol max(|y|, |y+|),
// accept at <= 1, factor min(5, max(0.2, 0.9/sqrt(norm))).  Returns
// MFG_ERR_TIMEOUT if a cell needs more than maxsub attempts.
int oracle_chem_substep_ros2(const mfg_params* P, const mfg_box* boxes, int nbox, double dt, double rtol,
                             double atol, int maxsub) {
    Ctx c{P, P->nspec};
    const int ns = P->nspec, nc = ncomp_of(P);
    const double g = 1.0 + 1.0 / std::sqrt(2.0);
    int status = MFG_OK;
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 so(b.s_old), sn(b.s_new);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    for (int n = 0; n < FLO_NVARS && n < nc; n++) sn(i, j, k, n) = so(i, j, k, n);
                    const double temp = so(i, j, k, TEMP_INDX);
                    double y[MAXS], f0[MAXS], k1[MAXS], k2[MAXS], y1[MAXS], W[MAXS][MAXS];
                    int piv[MAXS];
                    for (int s = 0; s < ns; s++) y[s] = so(i, j, k, FLO_NVARS + s);
                    double t = 0.0, h = dt;
                    bool done = false;
                    for (int att = 0; att < maxsub && !done; att++) {
                        bool last = false;
                        if (t + h >= dt) { h = dt - t; last = true; }
                        // source and Jacobian
                        compute_spec_source(c, y, temp, f0);
                        for (int s = 0; s < ns; s++)
                            for (int q = 0; q < ns; q++) W[s][q] = 0.0;
                        if (P->chem_on)
                            for (int r = 0; r < P->nreact; r++) {
                                double kr = P->A[r];
                                if (P->Ea[r] != 0.0) kr = P->A[r] * std::exp(-P->Ea[r] / (RU * temp));
                                for (int q = 0; q < ns; q++) {
                                    if (!(P->order[r][q] > 0.0)) continue;
                                    double dr = kr;
                                    for (int p = 0; p < ns; p++) {
                                        const double o = P->order[r][p];
                                        if (!(o > 0.0)) continue;
                                        dr *= (p == q) ? o * std::pow(y[p], o - 1.0) : std::pow(y[p], o);
                                    }
                                    for (int s = 0; s < ns; s++)
                                        if (std::fabs(P->nu[r][s]) > 0.0) W[s][q] += P->nu[r][s] * dr;
                                }
                            }
                        for (int s = 0; s < ns; s++) {
                            for (int q = 0; q < ns; q++) W[s][q] = -(g * h) * W[s][q];
                            W[s][s] += 1.0;
                        }
                        // LU with partial pivoting
                        for (int kk = 0; kk < ns; kk++) {
                            int p = kk;
                            for (int ii = kk + 1; ii < ns; ii++)
                                if (std::fabs(W[ii][kk]) > std::fabs(W[p][kk])) p = ii;
                            piv[kk] = p;
                            if (p != kk)
                                for (int jj = 0; jj < ns; jj++) std::swap(W[kk][jj], W[p][jj]);
                            for (int ii = kk + 1; ii < ns; ii++) {
                                W[ii][kk] /= W[kk][kk];
                                for (int jj = kk + 1; jj < ns; jj++) W[ii][jj] -= W[ii][kk] * W[kk][jj];
                            }
                        }
                        auto solve = [&](double* x) {
                            for (int kk = 0; kk < ns; kk++)
                                if (piv[kk] != kk) std::swap(x[kk], x[piv[kk]]);
                            for (int ii = 1; ii < ns; ii++)
                                for (int jj = 0; jj < ii; jj++) x[ii] -= W[ii][jj] * x[jj];
                            for (int ii = ns - 1; ii >= 0; ii--) {
                                for (int jj = ii + 1; jj < ns; jj++) x[ii] -= W[ii][jj] * x[jj];
                                x[ii] /= W[ii][ii];
                            }
                        };
                        for (int s = 0; s < ns; s++) k1[s] = f0[s];
                        solve(k1);
                        for (int s = 0; s < ns; s++) y1[s] = y[s] + h * k1[s];
                        compute_spec_source(c, y1, temp, k2);
                        for (int s = 0; s < ns; s++) k2[s] -= 2.0 * k1[s];
                        solve(k2);
                        double e2 = 0.0;
                        for (int s = 0; s < ns; s++) {
                            const double yn = y[s] + (1.5 * h) * k1[s] + (0.5 * h) * k2[s];
                            const double err = (0.5 * h) * (k1[s] + k2[s]);
                            const double sc = atol + rtol * std::max(std::fabs(y[s]), std::fabs(yn));
                            e2 += (err / sc) * (err / sc);
                            y1[s] = yn;
                        }
                        const double en = std::sqrt(e2 / ns);
                        if (en <= 1.0) {
                            for (int s = 0; s < ns; s++) y[s] = y1[s];
                            t += h;
                            if (last) done = true;
                        }
                        h *= (en > 0.0) ? std::min(5.0, std::max(0.2, 0.9 / std::sqrt(en))) : 5.0;
                    }
                    if (!done) status = MFG_ERR_TIMEOUT;
                    for (int s = 0; s < ns; s++) sn(i, j, k, FLO_NVARS + s) = y[s];
                }
    }
    return status;
}

// mflo::Advance_chemistry (Source/mflo_splitchem.cpp:177-199), after its
// swap: the stage-1 source on the incoming s_old, the midpoint
// 1*X + (half dt) F in the s_new buffer, the stage-2 source there, then
// s_new = 1*X + dt F; s_old ends holding X, the incoming s_new.
int oracle_chem_advance_rk2(const mfg_params* P, const mfg_box* boxes, int nbox, double dt) {
    Ctx c{P, P->nspec};
    const int nc = ncomp_of(P);
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        ValidFab X, F;
        X.define(b, nc);
        F.define(b, nc);
        copy_valid(b, X.a, b.s_new, nc);
        A4 x(X.a), f(F.a), sn(b.s_new);
        chem_rhs_box(c, b, A4(b.s_old), f);  // compute_dsdt_chemistry(lev, .., S_new (= old phi_old))
        copy_valid(b, b.s_old, X.a, nc);     // the swap: phi_old = current
        for (int n = 0; n < nc; n++)
            for (int k = b.lo[2]; k <= b.hi[2]; k++)
                for (int j = b.lo[1]; j <= b.hi[1]; j++)
                    for (int i = b.lo[0]; i <= b.hi[0]; i++) sn(i, j, k, n) = one * x(i, j, k, n) + half * dt * f(i, j, k, n);
        chem_rhs_box(c, b, sn, f);
        for (int n = 0; n < nc; n++)
            for (int k = b.lo[2]; k <= b.hi[2]; k++)
                for (int j = b.lo[1]; j <= b.hi[1]; j++)
                    for (int i = b.lo[0]; i <= b.hi[0]; i++) sn(i, j, k, n) = one * x(i, j, k, n) + dt * f(i, j, k, n);
    }
    return MFG_OK;
}

// mflo::store_inertgas_conc (Source/mflo_splitchem.cpp:150-175).
int oracle_store_inertgas_conc(const mfg_params* P, const mfg_box* boxes, int nbox) {
    Ctx c{P, P->nspec};
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 s(b.s_new);
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    if (!(s(i, j, k, VFRAC_INDX) >= one)) continue;
                    double spec[MAXS];
                    for (int sp = 0; sp < P->nspec; sp++) spec[sp] = s(i, j, k, FLO_NVARS + sp);
                    s(i, j, k, DENS_INDX) = get_bgasconc_from_rc(c, s(i, j, k, RHO_INDX), spec);
                }
    }
    return MFG_OK;
}

// mflo::update_vars_after_chemsolve (Source/mflo_splitchem.cpp:74-148).
int oracle_update_vars_after_chemsolve(const mfg_params* P, const mfg_box* boxes, int nbox, int bg) {
    Ctx c{P, P->nspec};
    int status = MFG_OK;
    for (int ib = 0; ib < nbox; ib++) {
        const mfg_box& b = boxes[ib];
        A4 s(b.s_new);
        double minp = 1e300;
        for (int k = b.lo[2]; k <= b.hi[2]; k++)
            for (int j = b.lo[1]; j <= b.hi[1]; j++)
                for (int i = b.lo[0]; i <= b.hi[0]; i++) {
                    if (s(i, j, k, VFRAC_INDX) >= one) {
                        double spec[MAXS], u[MAXC], p[NCVARS];
                        for (int sp = 0; sp < P->nspec; sp++) spec[sp] = s(i, j, k, sp + FLO_NVARS);
                        s(i, j, k, RHO_INDX) = get_r_from_c(c, spec, bg ? s(i, j, k, DENS_INDX) : zeroval);
                        s(i, j, k, DENS_INDX) = s(i, j, k, RHO_INDX);
                        s(i, j, k, RHOU_INDX) = s(i, j, k, RHO_INDX) * s(i, j, k, VELX_INDX);
                        s(i, j, k, RHOV_INDX) = s(i, j, k, RHO_INDX) * s(i, j, k, VELY_INDX);
                        s(i, j, k, RHOW_INDX) = s(i, j, k, RHO_INDX) * s(i, j, k, VELZ_INDX);
                        for (int q = 0; q < NCVARS; q++) u[q] = s(i, j, k, q + RHO_INDX);
                        for (int q = 0; q < P->nspec; q++) u[q + NCVARS] = s(i, j, k, q + FLO_NVARS);
                        cons_to_prim(c, u, p);
                        for (int q = 0; q < NCVARS; q++) s(i, j, k, q + DENS_INDX) = p[q];
                        s(i, j, k, TEMP_INDX) = get_t_from_rpc(c, s(i, j, k, DENS_INDX), s(i, j, k, PRES_INDX), u + NCVARS);
                    }
                    minp = std::min(minp, s(i, j, k, PRES_INDX));
                }
        if (minp < 0 && P->do_ns) status = MFG_ERR_NEG_PRESSURE;
    }
    return status;
}

// One coarse step of a multi-level run: the step body of mflo::EvolveAMR
// (Source/mflo_evolve.cpp:26-58) around timeStep's subcycling (:174-247):
// level l advances with dt0 / (ratio_1 ... ratio_l), its face fluxes feed the
// flux registers of both of its interfaces, and after the substeps of the
// finer level it is refluxed and averaged down onto; then the primitive
// refresh and species clipping of every level.  boxes[].level selects the
// level; geoms holds one geometry per level (ratio = dx[l-1] / dx[l]); fine
// boxes must be aligned to the ratio and properly nested (MFG_ERR_ARG
// otherwise).  On exit s_new holds the new state and s_old phi_old.
int oracle_advance_amr(const mfg_params* P, const mfg_geom* geoms, const mfg_box* boxes, int nbox, int nlev,
                       double time, double dt0, int only_flow, int clip) {
    if (nlev < 1) return MFG_ERR_ARG;
    Amr A;
    A.P = P;
    A.c = Ctx{P, P->nspec};
    A.nlev = nlev;
    A.nc = ncomp_of(P);
    A.only_flow = only_flow != 0;
    A.G.resize(nlev);
    A.ratio.assign(nlev, 1);
    A.lv.resize(nlev);
    A.flux.resize(nlev);
    A.reg.resize(nlev);
    for (int l = 0; l < nlev; l++) {
        A.G[l] = &geoms[l];
        if (l > 0) {
            A.ratio[l] = (int)(geoms[l - 1].dx[0] / geoms[l].dx[0] + 0.5);
            if (A.ratio[l] < 2) return MFG_ERR_ARG;
        }
    }
    for (int b = 0; b < nbox; b++) {
        const int l = boxes[b].level;
        if (l < 0 || l >= nlev) return MFG_ERR_ARG;
        for (int d = 0; d < 3; d++)
            if (l > 0 && (floor_div(boxes[b].lo[d], A.ratio[l]) * A.ratio[l] != boxes[b].lo[d] ||
                          floor_div(boxes[b].hi[d] + 1, A.ratio[l]) * A.ratio[l] != boxes[b].hi[d] + 1))
                return MFG_ERR_ARG;
        A.lv[l].push_back(boxes[b]);
    }
    for (int l = 0; l < nlev; l++) A.flux[l].resize(A.lv[l].size());
    A.t_old.assign(nlev, time);
    A.t_new.assign(nlev, time);
    A.dt.assign(nlev, dt0);
    for (int l = 1; l < nlev; l++) A.dt[l] = A.dt[l - 1] / A.ratio[l];
    int rc;
    for (int l = 1; l < nlev; l++)
        if ((rc = build_registers(A, l))) return rc;
    if ((rc = amr_time_step(A, 0, time))) return rc;
    for (int l = 0; l < nlev; l++) {
        Level L{P, &geoms[l], A.lv[l].data(), (int)A.lv[l].size()};
        if ((rc = update_prims(A.c, L))) return rc;
        if (clip) clip_species(A.c, L);
    }
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
