/*
 * mflo_gpu.h — C ABI of the GB300 (sm_103a) implementation of mesoflow's
 * per-box explicit right-hand side and SSP-RK3 stage update.
 *
 * The boundary is plain C: raw device pointers, strides, sizes and POD
 * parameter tables.  An AMReX-based mesoflow driver calls these entry points
 * in place of the bodies of
 *   mflo::compute_dsdt_flow        Source/mflo_evolve.cpp:543-682
 *   mflo::update_cutcell_data      Source/mflo_evolve.cpp:495-519
 *   RK3 stage algebra              Source/mflo_evolve.cpp:276-311
 *   mflo::compute_dsdt_chemistry   Source/mflo_evolve.cpp:684-720
 *   mflo::compute_residual_norms   Source/mflo_evolve.cpp:91-112
 *   mflo::update_primitive_vars    Source/mflo_evolve.cpp:114-171
 *   mflo::clip_neg_speciesconc     Source/mflo_evolve.cpp:521-540
 *   mflo::EstTimeStep              Source/mflo_timestep.cpp:53-153
 *   mflo::FillPatch (single level) Source/mflo_gridwork.cpp:135-146 + Source/mflo_bcfill.H
 * keeping the reference's state layout (Source/globalDefines.H:5-32):
 * component-major AMReX Array4<Real> boxes, FP64.
 *
 * Memory: the caller owns every state array.  The library owns only its
 * scratch (face-flux and reconstruction buffers, box tables, graphs), which it
 * allocates on first use and frees in mfg_finalize().
 *
 * Errors: every entry point returns an int status (MFG_OK on success).  Faults
 * detected on the device (NaN in dsdt, negative pressure, bad box, bounded
 * wait timeout) become sticky bits read by mfg_status(); kernels never trap.
 *
 * Threading: entry points are asynchronous on the caller's stream (passed as
 * void*, a cudaStream_t) except those that return host values, which
 * synchronize that stream.  mfg_init() is not thread-safe.
 */
#ifndef MFLO_GPU_H_
#define MFLO_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- layout constants (Source/globalDefines.H:5-32) -------------------- */
#define MFG_RHO_INDX    0
#define MFG_RHOU_INDX   1
#define MFG_RHOV_INDX   2
#define MFG_RHOW_INDX   3
#define MFG_RHOE_INDX   4
#define MFG_DENS_INDX   5
#define MFG_VELX_INDX   6
#define MFG_VELY_INDX   7
#define MFG_VELZ_INDX   8
#define MFG_PRES_INDX   9
#define MFG_TEMP_INDX   10
#define MFG_VFRAC_INDX  11
#define MFG_FLO_NVARS   12
#define MFG_NCVARS      5

#define MFG_MAX_SPECIES   16
#define MFG_MAX_REACTIONS 16
#define MFG_NGROW         3      /* ghost width of Sborder (mflo_evolve.cpp:253) */

/* ---- status codes --------------------------------------------------------- */
#define MFG_OK                0
#define MFG_ERR_ARG           1   /* bad argument / box descriptor */
#define MFG_ERR_NAN           2   /* "NaN detected in dsdt" (div_3d.H:72-75) */
#define MFG_ERR_NEG_PRESSURE  3   /* "Pressure has gone negative" (mflo_evolve.cpp:162-167) */
#define MFG_ERR_SCHEME        4   /* "unknown hyperbolics scheme" (compute_flux_3d.H:273-276) */
#define MFG_ERR_TIMEOUT       5   /* a bounded device wait gave up */
#define MFG_ERR_CUDA          6   /* a CUDA runtime call failed */
#define MFG_ERR_STATE         7   /* called before mfg_init / unsupported configuration */
#define MFG_ERR_SIZE          8   /* a box needs more scratch than mfg_compute_dsdt_flow_noalloc's static array */

/* capacity of the static scratch array of mfg_compute_dsdt_flow_noalloc (32 MiB) */
#define MFG_NOALLOC_SCRATCH_DOUBLES 4194304

/* sticky device status bits (mfg_status) */
#define MFG_STATUS_NAN           0x1u
#define MFG_STATUS_NEG_PRESSURE  0x2u
#define MFG_STATUS_TIMEOUT       0x4u
#define MFG_STATUS_BAD_BOX       0x8u
#define MFG_STATUS_CHEM_STEPS    0x10u  /* implicit chemistry needed more than max_substeps in a cell */

/* ---- thermo / transport / boundary enums ---------------------------------- */
/* thermo families found in the reference's per-case thermo.H plugins */
#define MFG_THERMO_MOLAR        0  /* calorically perfect molar mixture:
                                      models/catalystCylinder/thermo.H:36-156,
                                      tests/Cartesian/ShockTube_N2/thermo.H:38-132 */
#define MFG_THERMO_MASS_SINGLE  1  /* single gas, p=(gamma-1) rho e:
                                      tests/Cartesian/TaylorGreen/thermo.H:36-80,
                                      models/porousParticle/thermo.H */
#define MFG_THERMO_BG_GAS       2  /* molar mixture plus untracked background gas:
                                      py_utils/rxnscheme_writer/example/thermo.H */

/* energy form of get_e_from_rpc for the molar family */
#define MFG_EFORM_MOLAR_CV  0      /* sum(cv_k c_k) T / rho   (catalystCylinder/thermo.H:131-156) */
#define MFG_EFORM_MASS_CV   1      /* T * sum(cv_k/W_k x_k)    (ShockTube_N2/thermo.H:110-132) */

#define MFG_TRANSPORT_CONST        0  /* coefficient = gas value */
#define MFG_TRANSPORT_VFRAC_BLEND  1  /* gas*vfrac + solid*(1-vfrac) (catalystCylinder/transport.H) */

/* physical boundary kinds, numbered as mflo.lo_bc / mflo.hi_bc (Source/mflo.cpp:86-142) */
#define MFG_BC_INT_DIR   0  /* periodic */
#define MFG_BC_FOEXTRAP  2
#define MFG_BC_EXT_DIR   3
#define MFG_BC_WALL      6  /* reflect_even, reflect_odd for momenta/velocities */

/* ext_dir ghost-state templates (the per-case externalbc functor, externbc.H) */
#define MFG_EXT_FIXED_STATE      0  /* s_ext = given state; optionally PRES from the interior
                                       (tests/Cartesian/ShockTube_N2/externbc.H) */
#define MFG_EXT_PRESSURE_INLET   1  /* dens,pres,species fixed; normal velocity = |u_int|
                                       (models/porousParticle/externbc.H:25-43) */
#define MFG_EXT_PRESSURE_OUTLET  2  /* pres fixed; dens,velocity,species from the interior
                                       (models/porousParticle/externbc.H:44-58) */
#define MFG_EXT_VELOCITY_INLET   3  /* dens,velocity,pres,species fixed (conserved from prim) */
#define MFG_EXT_SPECIES_DIRICHLET 4 /* flow components from the interior, vfrac 1 (or from the
                                       interior), species 2 spec - s_int (value spec on the face)
                                       or zero gradient per species
                                       (tests/Cartesian/SpeciesEqTests/externbc.H:20-52,
                                       models/blockCatalyst1d/externbc.H:18-55) */

/* ---- views ---------------------------------------------------------------- */
/* Mirror of amrex::Array4<Real>: p[(i-begin0) + (j-begin1)*jstride
 * + (k-begin2)*kstride + n*nstride]; end is exclusive. */
typedef struct mfg_array4 {
    double*  p;
    int64_t  jstride;
    int64_t  kstride;
    int64_t  nstride;
    int      begin[3];
    int      end[3];
    int      ncomp;
} mfg_array4;

/* One AMReX box of a level (the body of one MFIter iteration). */
typedef struct mfg_box {
    int        lo[3];       /* valid cells, inclusive (Box::smallEnd)              */
    int        hi[3];       /* valid cells, inclusive (Box::bigEnd)                */
    mfg_array4 sborder;     /* state grown by >= MFG_NGROW ghost cells (Sborder)   */
    mfg_array4 dsdt;        /* RHS on the valid box; p == NULL: not stored          */
    mfg_array4 s_old;       /* phi_old on the valid box (RK base state)            */
    mfg_array4 s_new;       /* phi_new on the valid box (RK stage output)          */
    mfg_array4 flux[3];     /* face fluxes, nodal in d (for reflux); p == NULL: skip */
    int        level;       /* index into the geometry array of batched calls      */
    int        pad_;
} mfg_box;

typedef struct mfg_geom {
    double dx[3];
    double prob_lo[3];
    int    domain_lo[3];
    int    domain_hi[3];
    int    is_periodic[3];
    int    pad_;
} mfg_geom;

typedef struct mfg_extbc {
    int    kind;                  /* MFG_EXT_* */
    int    keep_interior_pres;    /* FIXED_STATE: PRES_INDX copied from the boundary cell */
    int    spec_zero_grad_mask;   /* SPECIES_DIRICHLET: bit s set = species s copied from the boundary cell */
    int    vfrac_interior;        /* SPECIES_DIRICHLET: VFRAC copied from the boundary cell (else 1) */
    double dens, pres;
    double vel[3];
    double spec[MFG_MAX_SPECIES];
    double state[MFG_FLO_NVARS + MFG_MAX_SPECIES];   /* FIXED_STATE ghost state */
} mfg_extbc;

/* The per-case plugin headers and mflo.* runtime parameters, as tables. */
typedef struct mfg_params {
    /* species + thermo (species.H, species.cpp, thermo.H) */
    int    nspec;                              /* NUM_SPECIES (1..MFG_MAX_SPECIES) */
    int    ngas;                               /* NUM_GAS_SPECIES: species [0,ngas) are gas */
    int    thermo_kind;                        /* MFG_THERMO_* */
    int    energy_form;                        /* MFG_EFORM_* (molar family) */
    double R_univ;                             /* gas constant of the molar / bg families */
    double gas_R;                              /* specific gas constant (mass-single family) */
    double gamma_single;                       /* gamma (mass-single family) */
    double bg_molwt;                           /* BG_GAS_MWT (bg family) */
    double molwt[MFG_MAX_SPECIES];
    double gamma[MFG_MAX_SPECIES + 1];         /* gas species; [ngas] = background gas */
    double advect_flag[MFG_MAX_SPECIES];
    /* transport (transport.H compute_spec_dcoeff, userfuncs.H compute_fluid_transport) */
    int    visc_mode, cond_mode;               /* MFG_TRANSPORT_* */
    double visc_gas, visc_solid;
    double cond_gas, cond_solid;
    int    diff_mode[MFG_MAX_SPECIES];
    double diff_gas[MFG_MAX_SPECIES];
    double diff_solid[MFG_MAX_SPECIES];
    /* numerics (Source/mflo.H:227-259) */
    int    order_hyp;                          /* 1, 2, 4 or 5 */
    int    do_ns;                              /* mflo.solve_navier_stokes */
    int    species_in_solid;
    int    conj_ht;                            /* mflo.conjugate_heat_transfer */
    double dissfactor;
    double solid_temp;                         /* get_solid_t_from_rhoe */
    double cfl;
    /* chemistry (chemistry.H compute_spec_source) */
    int    chem_on;
    int    nreact;
    double nu[MFG_MAX_REACTIONS][MFG_MAX_SPECIES];    /* net stoichiometry (rxnarray) */
    double order[MFG_MAX_REACTIONS][MFG_MAX_SPECIES]; /* concentration exponents (|rxnarray| of reactants) */
    double A[MFG_MAX_REACTIONS];               /* rateconsts, or Arrhenius pre-exponential */
    double Ea[MFG_MAX_REACTIONS];              /* activation energy J/mol; 0 = table form */
    /* boundaries (mflo.lo_bc / mflo.hi_bc, externbc.H) */
    int    bc_lo[3], bc_hi[3];                 /* MFG_BC_* */
    mfg_extbc ext_lo[3], ext_hi[3];
} mfg_params;

/* ---- library lifetime ----------------------------------------------------- */

/* Validates the parameter tables and uploads them to device constant memory.
 * Replaces the compile-time plugin includes (thermo.H, transport.H,
 * chemistry.H, species.cpp) and mflo::ReadParameters (Source/mflo.cpp:263-307). */
int mfg_init(const mfg_params* params);

/* Frees the library's scratch (face fluxes, box tables, graphs) and forgets
 * the device addresses cached by mfg_compute_dsdt_flow_noalloc. */
int mfg_finalize(void);

/* Reads (and optionally clears) the sticky device status bits.  Synchronizes. */
int mfg_status(uint32_t* flags, int clear);

/* Library version string. */
const char* mfg_version(void);

/* ---- per-level operations on a box list (all boxes share geom) ------------ */

/* Single-level ghost fill of every box's sborder from the level's valid data
 * (s_src selects which array of each box holds the valid data: 0 = s_old,
 * 1 = s_new) plus the physical boundary conditions.
 * Replaces FillPatch(lev, time, Sborder, 0, ncomp) at level 0
 * (Source/mflo_gridwork.cpp:135-146, Source/mflo_bcfill.H:13-129). */
int mfg_fill_patch(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                   int s_src, double time, void* stream);

/* Immersed-boundary cut-cell ghost treatment, in place on sborder (valid cells).
 * Replaces mflo::update_cutcell_data (Source/mflo_evolve.cpp:495-519)
 * -> update_cutcells (Source/Src_3d/ib_utils.H:272-436).  The level-wide form
 * of the pass keeps its cut-cell lists in one library buffer: calls must be
 * ordered on one stream (or synchronized); calls that overlap on the GPU race. */
int mfg_cutcells(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                 double time, void* stream);

/* Flow RHS dsdt from sborder (and face fluxes when flux[d].p != NULL).
 * Replaces mflo::compute_dsdt_flow (Source/mflo_evolve.cpp:543-682):
 * compute_flux (compute_flux_3d.H:88-430) + update_residual (div_3d.H:13-76). */
int mfg_compute_dsdt_flow(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                          double time, double dt, void* stream);

/* Fused RHS + RK3 stage algebra (stage = 1, 2 or 3), writing s_new:
 *   1: s_new = sborder + dt*L(sborder)                       (mflo_evolve.cpp:283)
 *   2: s_new = ((s_new + dt*L(sborder)) + 3*s_old) * 1/4     (mflo_evolve.cpp:296-298)
 *   3: s_new = (s_old + 2*(s_new + dt*L(sborder))) * third   (mflo_evolve.cpp:309-311)
 * dsdt is also stored when dsdt.p != NULL. */
int mfg_rk3_stage(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                  int stage, double time, double dt, void* stream);

/* Species reaction source added to dsdt on the valid box (s_new holds the
 * state).  Replaces compute_dsdt_chemistry (Source/mflo_evolve.cpp:684-720). */
int mfg_chem_source(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                    double time, void* stream);

/* Strang chemistry sub-step over dt: s_old = state after the flow stages,
 * s_new = result; explicit SSP-RK3 of the reaction source, as the AMReX
 * TimeIntegrator default (Source/mflo_evolve.cpp:470-493, Source/mflo.cpp:300-305). */
int mfg_chem_substep(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                     double time, double dt, void* stream);

/* cons -> prim refresh of s_new plus the negative-pressure check
 * (Source/mflo_evolve.cpp:114-171); returns MFG_ERR_NEG_PRESSURE. Synchronizes. */
int mfg_update_primitive_vars(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                              void* stream);

/* Negative species concentrations of s_new set to 0 (Source/mflo_evolve.cpp:521-540). */
int mfg_clip_species(const mfg_box* boxes, int nbox, void* stream);

/* L2 norms of (s_new - s_old)/dt (components < VFRAC scaled by s_old VFRAC) per
 * component into out[ncomp] (host).  Source/mflo_evolve.cpp:91-112. Synchronizes. */
int mfg_residual_norms(const mfg_box* boxes, int nbox, double dt,
                       double* out, void* stream);

/* CFL / diffusion time-step estimate of s_new, cfl applied
 * (Source/mflo_timestep.cpp:53-153).  *dt_out on the host.  Synchronizes. */
int mfg_est_timestep(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                     double time, double* dt_out, void* stream);

/* One coarse step of a single level (Source/mflo_evolve.cpp:251-318 with the
 * bookends of mflo::EvolveAMR :33-58): phi_old <- phi_new; three RK3 stages of
 * fill patch, cut cells and the fused RHS + stage update; the Strang
 * chemistry sub-step unless only_flow; primitive refresh (negative pressure
 * -> MFG_ERR_NEG_PRESSURE); species clipping when clip != 0; residual norms
 * into resnorms[ncomp] when non-NULL.  Returns MFG_ERR_NAN when the "NaN
 * detected in dsdt" condition occurred.  Synchronizes the stream. */
int mfg_advance_level(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                      double time, double dt, int only_flow, int clip,
                      double* resnorms, void* stream);

/* mfg_advance_level for a driver whose state FABs live in host memory (the
 * reference's CPU build: its per-box MFIter bodies of mflo_evolve.cpp:251-318
 * read host Array4s).  h_state[b] is a host view with the layout of
 * boxes[b].s_new (same strides, begin, end and ncomp; else MFG_ERR_ARG); it
 * holds phi_new on entry and receives it on return.  Each box's view is copied
 * in on the stream before the step, and copied back on an internal copy
 * stream as soon as that box's last kernels (its stage-3 update and bookends)
 * are done, so the copies back overlap the later boxes' compute.  Results are
 * bitwise those of copy-in + mfg_advance_level + copy-out.  Pinned
 * (page-locked) host memory moves at link speed; pageable memory works but is
 * staged by the driver.  Synchronizes the stream. */
int mfg_advance_level_host(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                           double time, double dt, int only_flow, int clip,
                           const mfg_array4* h_state, double* resnorms, void* stream);

/* Selects the WENO5 nonlinear-weight normalisation: fast != 0 uses one
 * division per reconstructed value (default), 0 follows the reference's
 * four reciprocals (flux_schemes.H:407-414) operation for operation. */
int mfg_set_weno_mode(int fast);

/* The cut-cell lists and inverse-distance weights depend on the volume
 * fraction only, which the solver never changes; update_cutcells
 * (ib_utils.H:272-436) recomputes them every stage.  With the cache on
 * (default) the first mfg_cutcells / mfg_advance_level call for a box keeps
 * them in device memory (synchronizes twice; 24 B per cut cell plus 20 B per
 * fluid neighbour, about 0.3 KiB per cut cell in a sphere pack), and
 * every later call checks the box's grown volume fraction against a stored
 * copy on the device (exact) before using them: a changed geometry falls back
 * to recomputation in the same call and is dropped from the cache.  Results
 * are bitwise the same either way.  enable = 0 frees the cache.  Synchronizes. */
int mfg_set_cutcell_cache(int enable);

/* Form of the face pass of orders 1 and 2 with Navier-Stokes terms
 * (compute_flux, compute_flux_3d.H:88-430, whose faces on the solid side,
 * face vfrac < 1/2, carry conduction and diffusion only): 1 (default) writes
 * those faces in one pass and runs the flux branch over a compacted list of
 * the others, 0 runs every face in one kernel.  Bitwise the same results.
 * Synchronizes. */
int mfg_set_face_compaction(int on);

/* Integrator of the chemistry sub-step (mfg_chem_substep, mfg_advance_level,
 * the box-list steps): kind 0 (default) the explicit SSP-RK3 of the
 * reference's AMReX TimeIntegrator (rk.type 3); kind 1 an implicit, L-stable,
 * adaptive second-order Rosenbrock method (ROS2, gamma = 1 + 1/sqrt 2, with
 * the analytic Jacobian of the mass-action source and the embedded
 * first-order error estimate, error norm RMS(err / (atol + rtol max|c|)))
 * for stiff chemistry, where the reference uses SUNDIALS CVODE
 * (integration.type = SUNDIALS, Source/mflo_evolve.cpp:455-469), which is not
 * available here.  A cell that needs more than max_substeps substeps raises
 * MFG_STATUS_CHEM_STEPS.  Applies from the next launch, kept across mfg_init. */
int mfg_set_chem_integrator(int kind, double rtol, double atol, int max_substeps);

/* ---- split-chemistry pieces (mflo::Evolve_split, Source/mflo_splitchem.cpp:24-72:
 * flow to steady state, then chemistry sub-steps of the frozen flow, the flow
 * variables brought back to the new concentrations, flow again) -------------- */

/* mflo::Advance_chemistry (Source/mflo_splitchem.cpp:177-199): explicit
 * midpoint step of the reaction source with the reference's phi_old/phi_new
 * swap first, so the stage-1 source is evaluated on the incoming s_old and
 * the stage-2 source on the midpoint: s_new <- s_new + dt F(s_new +
 * dt/2 F(s_old)); on exit s_old holds the incoming s_new.  Asynchronous. */
int mfg_chem_advance_rk2(const mfg_box* boxes, int nbox, double time, double dt, void* stream);

/* mflo::store_inertgas_conc (Source/mflo_splitchem.cpp:150-175): in fluid
 * cells the untracked background-gas concentration (thermo.H
 * get_bgasconc_from_rc) goes to the density component.  Asynchronous. */
int mfg_store_inertgas_conc(const mfg_box* boxes, int nbox, void* stream);

/* mflo::update_vars_after_chemsolve (Source/mflo_splitchem.cpp:74-148): in
 * fluid cells rho = get_r_from_c(species[, stored background gas when
 * using_bg_inertgas]), momenta = rho x velocities, energy kept, primitives
 * and temperature recomputed.  Synchronizes; MFG_ERR_NEG_PRESSURE where the
 * reference aborts with "Pressure has gone negative". */
int mfg_update_vars_after_chemsolve(const mfg_box* boxes, int nbox, int using_bg_inertgas, void* stream);

/* Same result as mfg_compute_dsdt_flow, for callers that may not allocate
 * device memory (for example an AMReX application, whose arena reserves most
 * of the GPU at start-up, or a code with a fixed device-memory budget): the
 * scratch comes from one static device array of MFG_NOALLOC_SCRATCH_DOUBLES
 * doubles inside the library, and the call makes no cudaMalloc or cudaFree.
 * A box whose scratch exceeds the array returns MFG_ERR_SIZE (any 32^3 box
 * fits, for every species count; a 40^3 box does not).  All calls share the array: calls that overlap on
 * the GPU race.  The first call on each device looks up the array's device
 * address; make it before any stream capture (after a cudaDeviceReset, call
 * mfg_finalize first so that the address is looked up again).  No counterpart in the
 * reference, which allocates its flux and transport FABs per box
 * (Source/mflo_evolve.cpp:566-591). */
int mfg_compute_dsdt_flow_noalloc(const mfg_box* boxes, int nbox, const mfg_geom* geom,
                                  double time, double dt, void* stream);

/* ---- batched AMR form --------------------------------------------------------
 * All boxes of all levels (uneven sizes; boxes[b].level indexes geoms) uploaded
 * once into device tables; every phase of the step is one launch over a tile
 * list spanning all boxes, and the whole step can be replayed from one CUDA
 * graph.  Levels advance with a common dt (no subcycling); level-L ghost cells
 * not covered at level L are injected from level L-1.  Replaces the per-box
 * MFIter loops of Source/mflo_evolve.cpp:509-519 and :579-651 (and the
 * FillPatch calls :278-302) for a whole hierarchy at once. */
typedef struct mfg_boxlist mfg_boxlist;

/* Builds the device box tables, per-level owner maps, per-box scratch and tile
 * lists.  The arrays named by the descriptors must stay valid until destroy. */
int mfg_boxlist_create(const mfg_box* boxes, int nbox, const mfg_geom* geoms, int nlev,
                       mfg_boxlist** out);
int mfg_boxlist_destroy(mfg_boxlist* list);

/* One step of every level (phi_old <- phi_new, three RK3 stages of fill + cut
 * cells + RHS + stage update, chemistry sub-step, primitive refresh, clipping).
 * mode 0: plain per-box launches of the same kernels; 1: batched launches over
 * tile lists; 2: the batched step replayed from a CUDA graph (captured on first
 * use and when dt changes; needs a non-default stream).  Asynchronous. */
int mfg_boxlist_step(mfg_boxlist* list, double time, double dt, int mode, void* stream);

/* mflo::EvolveAMR's loop on the device for the common-dt step of the list
 * (Source/mflo_evolve.cpp:18-89; for one level exactly the reference's loop):
 * while *istep < max_step and *time < final_time: ComputeDt (EstTimeStep of
 * every level with cfl, at most 1.1 x the previous dt, the minimum over the
 * levels, clamped so that time does not pass stop_time, mflo_timestep.cpp:
 * 18-153), one batched step (as mfg_boxlist_step mode 1), time += dt; stop
 * when time >= stop_time - 1e-6 dt or a NaN / negative-pressure status is
 * raised.  The whole loop is one CUDA graph with a device-side loop condition:
 * no step waits for the host.  *time, *dt (the previous step's dt; 1e100
 * before the first step) and *istep are read and updated.  Needs a
 * non-default stream and profiling off; synchronizes at the end; returns
 * MFG_ERR_NAN / MFG_ERR_NEG_PRESSURE where the reference aborts. */
int mfg_boxlist_evolve(mfg_boxlist* list, double final_time, double stop_time, int max_step, double* time,
                       double* dt, int* istep, void* stream);

/* The same device-resident loop for the subcycled hierarchy (mfg_boxlist_step_amr
 * steps): ComputeDt with subcycling on the device (per level EstTimeStep x cfl
 * capped at 1.1 x the level's previous dt, dt0 = min over levels of the ratio
 * product x that, stop-time clamp, dt_l = dt_{l-1} / ratio_l), the fill
 * coefficients of the coarse step computed on the device, then the step.
 * dt holds nlev doubles: each level's previous dt (1e100 before the first). */
int mfg_boxlist_evolve_amr(mfg_boxlist* list, double final_time, double stop_time, int max_step, double* time,
                           double* dt, int* istep, void* stream);

/* One coarse step of the reference's multi-level time stepping over the whole
 * hierarchy (mflo::EvolveAMR's step, Source/mflo_evolve.cpp:26-58, and
 * mflo::timeStep, :174-247): level l advances with dt0 / (ratio_1 ... ratio_l)
 * (ratio_l substeps of level l per step of level l-1), each RK3 stage filling
 * the level's ghost cells as FillPatch does (Source/mflo_gridwork.cpp:135-173):
 * level-l data, else cell_cons_interp from level l-1 at the stage time
 * (old / new / linear in time, mflo::GetData, Source/mflo.cpp:310-330), then
 * the physical boundaries; the stage's face fluxes go to the flux registers
 * (weights 1/6, 1/6, 2/3, :655-681); after the substeps of level l+1, level l
 * is refluxed and level l+1 averaged down onto it; then the chemistry
 * sub-steps, primitive refresh and clipping as in mfg_boxlist_step.  Needs
 * refinement ratios 2 to 4, fine boxes aligned to the ratio and properly nested (each fine
 * box's ghost cells and their interpolation stencil, inside the domain, lie
 * on the next coarser level): MFG_ERR_ARG otherwise.  mode 0 plain per-box
 * launches, 1 batched per level, 2 replay of a CUDA graph of the whole coarse
 * step (captured on first use and when dt0 changes; non-default stream).
 * AMReX is not vendored in the reference: the interpolation, register and
 * average-down semantics are restated from AMReX's documented behaviour. */
int mfg_boxlist_step_amr(mfg_boxlist* list, double time, double dt0, int mode, void* stream);

/* Chooses tile size and grid size for each batched phase by timing candidates
 * (CUDA events) on this machine list, and for WENO5 the flux form (column sweep
 * or per face, bitwise equal); results (optional, 16 doubles): per phase
 * (fill, cut, face, flux, update) tile items, grid blocks, best ms, then the
 * flux kernel (2 column sweep, 1 WENO5 per face, 0 generic).  Synchronizes. */
int mfg_boxlist_autotune(mfg_boxlist* list, double dt, double* results, void* stream);

/* Number of valid cells in the list. */
long long mfg_boxlist_cells(const mfg_boxlist* list);

/* ---- adjoint form --------------------------------------------------------------
 * No counterpart in the reference (its solver is forward only).  The
 * objective is the integrated surface reaction rate
 *     J = dx dy dz * sum_valid_cells sum_r k_r(T) prod_s c_s^order[r][s]
 * with k_r = A_r, or A_r exp(-Ea_r/(RU T)) when Ea_r != 0 (the rate law of
 * the chemistry source, chemistry.H compute_spec_source). */

/* Form of the adjoint's hyperbolic-flux reversal: 1 (default) a column sweep
 * over all boxes of a stage (edge adjoints summed in registers, one scatter
 * per cell), 0 one thread per face and component; the two differ only in the
 * order of the floating-point sums. */
int mfg_set_adjoint_flux_form(int form);

/* J on the boxes' s_new.  Synchronizes. */
int mfg_reaction_objective(const mfg_box* boxes, int nbox, const mfg_geom* geom, double* J,
                           void* stream);

/* Advances the level nsteps steps of dt from s_new, exactly as nsteps calls of
 * mfg_advance_level(only_flow = 0, clip = 1), evaluates J on the result and
 * returns it with its gradients from a hand-written discrete adjoint of the
 * whole step: grad_logA[r] = dJ/dlog A_r (nreact values), grad_uin = dJ/d(the
 * normal velocity of the velocity-inlet boundaries, the initial state held
 * fixed).  Both gradient pointers may be null.  checkpoint_every > 0: the
 * state is kept every checkpoint_every steps and the steps between are
 * recomputed during the reverse sweep.  When one segment's intermediates fit
 * in free device memory (about checkpoint_every x (6 level-sized and 6 grown
 * arrays) plus nsteps/checkpoint_every level-sized ones), each segment but
 * the last is recomputed once with its intermediates kept and then reversed
 * (the last segment keeps them from the first forward sweep); otherwise each
 * step is recomputed once more before its reverse (about
 * nsteps/checkpoint_every + checkpoint_every + 10 level-sized arrays and 5
 * grown ones).  checkpoint_every = 0: every step's intermediates are kept and
 * nothing is recomputed (about 3 level-sized and 3 grown arrays per step).
 * The gradients do not depend on the choice beyond rounding.  Supported: order_hyp 5,
 * do_ns 1, molar or mass-single thermo, constant viscosity and conductivity,
 * no conj_ht, ext_dir boundaries of kind VELOCITY_INLET or FIXED_STATE; other
 * configurations return MFG_ERR_STATE.  On return s_new holds the state after
 * nsteps; s_old and sborder hold intermediates.  Synchronizes. */
int mfg_adjoint_objective(const mfg_box* boxes, int nbox, const mfg_geom* geom, int nsteps,
                          double dt, int checkpoint_every, double* J, double* grad_logA,
                          double* grad_uin, void* stream);

/* ---- diagnostics (no counterpart in the reference beyond BL_PROFILE) ------ */

/* Enables (1) or disables (0) CUDA-event timing of every kernel launch and
 * resets the accumulated times. */
int mfg_profile(int enable);

/* Accumulated milliseconds and launch counts per kernel kind (synchronizes);
 * returns the number of kinds. */
int mfg_profile_read(double* ms, long long* count, int nkinds);

/* Name of a kernel kind of mfg_profile_read. */
const char* mfg_profile_name(int kind);

/* Description of the last failed CUDA call behind an MFG_ERR_CUDA ("" if none). */
const char* mfg_last_error(void);

/* Total kernel launches issued by the library since it was loaded. */
unsigned long long mfg_launch_count(void);

/* Measures this GPU's FP64 FMA issue rate (TFLOP/s, FMA = 2 flop) with a
 * register-resident DFMA loop timed by CUDA events; the roof of the RHS
 * kernels.  Allocates a small buffer.  Synchronizes. */
int mfg_measure_fp64_peak(double* tflops, void* stream);

/* Self-test of the integer-pipe form of x + 0.0 that the stage update uses
 * (the sum of a state value and a rate of exactly +0): compares it bit for
 * bit with the FP64 add on n values (boundary values, then pseudo-random bit
 * patterns; NaN skipped) and returns the number of mismatches.
 * Synchronizes. */
int mfg_selftest_exact_ops(unsigned long long n, unsigned* mismatches);

#ifdef __cplusplus
}
#endif
#endif /* MFLO_GPU_H_ */
