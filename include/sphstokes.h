/*
 * sphstokes.h — C ABI of libsphstokes, a GB300 (sm_103a) implementation of the
 * pseudo-transient (PT) Stokes iteration of PTsolvers/SphericalStokes.
 *
 * The reference is a set of Julia scripts; its "interface" for the hot path is
 * the sequence of ParallelStencil kernels launched inside the PT loop of each
 * script (e.g. scripts_diapir/SphericalStokes_diapir.jl:409-443) and the
 * arrays they mutate in place.  This library replaces that loop: the caller
 * passes grid and physics parameters, the library owns the device arrays,
 * runs the loop, and hands back converged P, velocities, stresses, effective
 * viscosity and the error history.  Julia code binds it with `ccall`; arrays
 * cross the boundary as plain `double*` in the reference's own column-major
 * layout and sizes (so `pointer(A)` of a Julia Array{Float64,3} is passed
 * as is).
 *
 * Conventions
 *  - Every entry point returns int: 0 (SPH_OK) or a negative sph_status.
 *    No exceptions or aborts cross the ABI; sph_strerror() names the code and
 *    sph_last_error() gives the message of the last failure on this thread.
 *  - A context is used by one host thread at a time.  All device work of a
 *    context is issued on one CUDA stream (default: a stream the library
 *    creates; sph_set_stream() installs the caller's).
 *  - Index convention of fields: (ix,iy,iz) 1-based as in the reference,
 *    ix fastest.  Field sizes are those of the reference's @zeros calls
 *    (SphericalStokes_diapir.jl:381-399), see sph_field_dims().
 */
#ifndef SPHSTOKES_H
#define SPHSTOKES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 2

typedef enum sph_status {
    SPH_OK = 0,
    SPH_ERR_INVALID = -1,        /* bad argument or parameter */
    SPH_ERR_CUDA = -2,           /* a CUDA call failed (message in sph_last_error) */
    SPH_ERR_NOT_CONVERGED = -3,  /* maxiter reached before the tolerance */
    SPH_ERR_DIVERGED = -4,       /* NaN/Inf in a norm (reference: error("NaN"), SphericalStokes_mxpu.jl:426) */
    SPH_ERR_NOMEM = -5,          /* device or host allocation failed */
    SPH_ERR_UNSUPPORTED = -6,    /* combination of options not implemented */
    SPH_ERR_NO_DEVICE = -7       /* no CUDA device / the sm_103a kernels cannot run here */
} sph_status;

/* coordinate system: scripts_diapir/{Spherical,Cylindrical,Cartesian}Stokes_diapir.jl */
typedef enum sph_geometry { SPH_GEOM_SPHERICAL = 0, SPH_GEOM_CYLINDRICAL = 1, SPH_GEOM_CARTESIAN = 2 } sph_geometry;

/* arithmetic of the PT sweeps */
typedef enum sph_precision {
    SPH_PREC_FP64 = 0,  /* plain FP64 PT (the reference's Data.Number = Float64) */
    SPH_PREC_FP32 = 1,  /* plain FP32 PT (storage and arithmetic) */
    SPH_PREC_MIXED = 2  /* FP32 PT sweeps inside an FP64 defect-correction loop */
} sph_precision;

/* boundary-condition set */
typedef enum sph_bc {
    SPH_BC_DIAPIR = 0,     /* simple shear of the diapir scripts (sph: SphericalStokes_diapir.jl:61-99,
                              cyl: CylindricalStokes_diapir.jl:358-366, cart: CartesianStokes_diapir.jl:371-379) */
    SPH_BC_FREE_SLIP = 1,  /* free slip on all faces (SphericalStokes_plateau.jl:64-92); spherical only */
    SPH_BC_STRESS = 2,     /* free slip on the x1 faces, prescribed total normal stress sig_bc[1] on the x2
                              faces and sig_bc[2] on the x3 faces (not in the reference); spherical only */
    SPH_BC_FREE_SURFACE = 3 /* free-surface-stabilised top (not in the reference; the plateau's topography load
                              without sticky air): on the top x1 face the traction of the surface load q
                              (field SPH_FIELD_TOP_LOAD, top cells) plus fs_kappa * V_r, zero shear traction;
                              free slip on the bottom and the x2, x3 faces; spherical only */
} sph_bc;

/* rheology update after the stress update */
typedef enum sph_rheology {
    SPH_RHEO_LINEAR = 0,           /* eta = eta_ini, no update */
    SPH_RHEO_TAU_POWER = 1,        /* compute_TII! + power_law! (SphericalStokes_diapir.jl:243-265) */
    SPH_RHEO_TAU_POWER_RELAX = 2,  /* the same with log-space relaxation of eta_PL
                                      (CylindricalStokes_diapir.jl:185-192, CartesianStokes_diapir.jl:210-221) */
    SPH_RHEO_EDOT_POWER_RELAX = 3  /* eta_t = 2/(1/eta_ini + 1/(eta_ini (edot_II/edot_bg)^((1-n)/n))),
                                      eta <- eta^(1-relax) eta_t^relax (not in the reference) */
} sph_rheology;

/* initial state */
typedef enum sph_init {
    SPH_INIT_NONE = 0,       /* zeros; eta = eta_ini = eta0, rho = rho0; the caller sets fields */
    SPH_INIT_INCLUSION = 1   /* initialize_inclusion! on rho and eta plus the shear initial velocity
                                (SphericalStokes_diapir.jl:401-404 and the cyl/cart equivalents) */
} sph_init;

/* kernel variant of the FP32 sweeps (FP64 always uses one kernel per reference step) */
typedef enum sph_kernels { SPH_KERNELS_AUTO = 0, SPH_KERNELS_SIMPLE = 1 } sph_kernels;

/* stopping criterion of sph_solve */
typedef enum sph_criterion {
    SPH_CRIT_REFERENCE = 0,  /* max_f max|V_f - V_f(previous iteration)| / max|V_f| < tol and iter > 20
                                (SphericalStokes_diapir.jl:427-439) */
    SPH_CRIT_RESIDUAL = 1,   /* FP64 Stokes residual: max(max|R_mom|/f_scale, max|div V| l1/max|V|) < tol */
    SPH_CRIT_REFERENCE_PLATEAU = 2  /* SPH_CRIT_REFERENCE with the plateau script's rule: a NaN V3 ratio
                                       (max|V3| = 0) is left out of the max (SphericalStokes_plateau.jl:540-552) */
} sph_criterion;

typedef enum sph_field {
    SPH_FIELD_P = 0,
    SPH_FIELD_V1 = 1,      /* VR / VR / VX   (n1+1, n2, n3) */
    SPH_FIELD_V2 = 2,      /* Vθ / Vθ / VY   (n1, n2+1, n3) */
    SPH_FIELD_V3 = 3,      /* Vφ / VZ / VZ   (n1, n2, n3+1) */
    SPH_FIELD_TAU11 = 4,   /* τ_RR           (n1, n2, n3) */
    SPH_FIELD_TAU22 = 5,
    SPH_FIELD_TAU33 = 6,
    SPH_FIELD_TAU12 = 7,   /* τ_Rθ           (n1-1, n2-1, n3-2) */
    SPH_FIELD_TAU13 = 8,   /* τ_Rφ           (n1-1, n2-2, n3-1) */
    SPH_FIELD_TAU23 = 9,   /* τ_θφ           (n1-2, n2-1, n3-1) */
    SPH_FIELD_ETA = 10,    /* effective viscosity η */
    SPH_FIELD_ETA_INI = 11,
    SPH_FIELD_ETA_SM = 12, /* ηSM = local 7-point maximum of η */
    SPH_FIELD_DT_R = 13,   /* velocity pseudo-time step */
    SPH_FIELD_TII = 14,    /* second invariant of τ */
    SPH_FIELD_RHO = 15,
    SPH_FIELD_PHASE = 16,  /* 1 = linear cell for the power laws, 0 = power law (values 0/1 as double) */
    SPH_FIELD_ETA_PL = 17, /* η_PL state of SPH_RHEO_TAU_POWER_RELAX */
    SPH_FIELD_TOP_LOAD = 18, /* SPH_BC_FREE_SURFACE: surface load q (normal stress of the topography's weight)
                                on the top cells (i = n1); a cell-size array, the other layers unused */
    SPH_FIELD_COUNT = 19
} sph_field;

/* grid, physics and PT parameters.  sph_params_default() fills the values of
 * the reference script of the given geometry (e.g. SphericalStokes_diapir.jl:348-367). */
typedef struct sph_params {
    int32_t abi_version;   /* = SPH_ABI_VERSION */
    int32_t geometry;      /* sph_geometry */
    int32_t precision;     /* sph_precision */
    int32_t bc;            /* sph_bc */
    int32_t rheology;      /* sph_rheology */
    int32_t init;          /* sph_init */
    int32_t n1, n2, n3;    /* cells (P nodes) along x1, x2, x3 = nr, nθ, nφ (or nz / nx, ny, nz) */
    double c1, c2, c3;     /* domain centre: (r, π/2, 0) sph, (r, 0, 0) cyl, (0, 0, 0) cart */
    double l1, l2, l3;     /* domain lengths: (lr, lθ, lφ) etc.; node coordinates span c ± l/2 */
    double l_ref;          /* length in KBDT/GSDT (lr, or lx in Cartesian) */
    double vpdt;           /* PT step length: dr*CFL in the reference (:400) */
    double dmp;            /* damping parameter (:10) */
    double g;              /* gravity (radial for sph/cyl, along x3 for cart) */
    double tau_C;          /* characteristic stress of the stress power laws */
    double n_exp;          /* power-law exponent */
    double n_exp_late;     /* exponent switched to once the error drops below switch_err (cyl script :342-344) */
    double switch_err;     /* 0 disables the switch */
    double relax;          /* relaxation factor of the relaxed laws */
    double edot_bg;        /* background strain rate of SPH_RHEO_EDOT_POWER_RELAX */
    double r;              /* sphere / cylinder radius used by the shear BCs and the inclusion test */
    double sh;             /* shearing velocity of the diapir BCs */
    double sig_bc[3];      /* SPH_BC_STRESS: prescribed total normal stress on the x1 (unused), x2, x3 faces */
    /* SPH_INIT_INCLUSION */
    double eta0, vr;       /* matrix viscosity; inclusion viscosity = eta0 / vr */
    double rho0, rho_in;   /* matrix and inclusion density */
    double radius;         /* compared with the SQUARED distance, as the reference does (:132) */
    int32_t incl_linear;   /* 1: inclusion cells are linear (phase = 1) */
    int32_t kernels;       /* sph_kernels: FP32 sweeps fused (default) or one kernel per reference step */
    int32_t etasm_passes;  /* passes of the 7-point max filter that gives ηSM (reference: 1; 0 means 1) */
    int32_t reserved_i;
    double fs_kappa;       /* SPH_BC_FREE_SURFACE: stabilisation coefficient θ Δt Δρ g of the free-surface
                              stabilisation algorithm (the load of the surface's rise over a step; 0: none) */
    double reserved[7];
} sph_params;

/* solve controls and result */
typedef struct sph_solve_opts {
    int32_t criterion;     /* sph_criterion */
    int32_t nout;          /* check every nout iterations (reference: 100) */
    int64_t maxiter;       /* cap on PT iterations (all precisions; inner sweeps in MIXED) */
    double tol;            /* stopping tolerance (reference: 5e-7 on the velocity change) */
    /* MIXED only */
    double inner_rtol;     /* inner FP32 sweeps stop when their residual drops by this factor */
    int32_t max_outer;     /* cap on FP64 defect-correction steps */
    int32_t inner_max;     /* cap on FP32 sweeps per correction step */
    double warm_tol;       /* FP32 nonlinear warm start runs to this FP64 residual first (0 = skip) */
    double reserved[6];
} sph_solve_opts;

typedef struct sph_solve_info {
    int64_t iters;         /* PT iterations done (FP32 + FP64 sweeps) */
    int32_t outer;         /* defect-correction steps (MIXED) */
    int32_t status;        /* sph_status of the solve */
    double err;            /* final error of the chosen criterion */
    double residual;       /* final FP64 residual (SPH_CRIT_RESIDUAL definition) */
    double seconds;        /* wall time of the solve */
    int64_t nhist;         /* entries written to hist_iter / hist_err */
    double device_ms;      /* device time of the solve (CUDA events on the context's stream) */
    double sweep_ms;       /* of which PT sweeps (MIXED: the FP32 correction sweeps) */
    double outer_ms;       /* of which FP64 outer work (MIXED: residual, coefficients) */
    int32_t flags;         /* SPH_SOLVE_WARM_ABANDONED: the FP32 warm start produced a NaN or an
                              infinite error and was abandoned (the correction loop started from the
                              FP64 state as it was; its iterations count in iters) */
    int32_t reserved_i;
    double reserved[3];
} sph_solve_info;

#define SPH_SOLVE_WARM_ABANDONED 1

/* defaults of the reference script of the given geometry (diapir setups) */
int sph_params_default(sph_params* p, int32_t geometry);

/* sizes (reference layout) of a field: dims[0..2] */
int sph_field_dims(const sph_params* p, int32_t field, int64_t dims[3]);

/* allocate device state, build coordinate tables, apply p->init */
int sph_create(const sph_params* p, void** ctx);
int sph_destroy(void* ctx);

/* run device work of this context on `stream` (a cudaStream_t); NULL restores the library's own */
int sph_set_stream(void* ctx, void* stream);

/* copy a field from / to host memory in the reference layout (count = product of sph_field_dims) */
int sph_set_field(void* ctx, int32_t field, const double* host, int64_t count);
int sph_get_field(void* ctx, int32_t field, double* host, int64_t count);

/* Changes the scalar parameters of a live context between solves (the continuation steps
 * of SphericalStokes_plateau.jl:485-522 change vpdt through vr, and n_exp): vpdt (<= 0:
 * from vr as in sph_create), dmp, l_ref, g, tau_C, n_exp, n_exp_late, switch_err, relax,
 * edot_bg, r, sh, sig_bc, vr, eta0, etasm_passes.  geometry, precision, bc, rheology,
 * kernels, n1..n3, c1..c3 and l1..l3 are fixed at sph_create (SPH_ERR_INVALID if they
 * differ); init, rho0, rho_in, radius and incl_linear only act in sph_create.  Fields are
 * kept; η and η_ini of a new step are set with sph_set_field. */
int sph_update_params(void* ctx, const sph_params* params);

/* Batch of independent solves (no counterpart in the reference, which solves one grid per
 * script run).  opts[i] and infos[i] belong to ctxs[i] (per-solve tolerance and iteration
 * budget in; status, iterations, outer steps and residual out); no history is recorded.  A
 * context may appear once.  Returns SPH_OK unless an argument or a CUDA call failed; the
 * outcome of each solve is infos[i].status.
 *  - Lockstep batch, when every solve is SPH_PREC_MIXED on SPH_CRIT_RESIDUAL without a warm
 *    start (warm_tol 0), with the TMA sweep and one even nout for all: the solves advance
 *    together, and one correction sweep of all of them is one launch per geometry over a
 *    work list of (solve, tile, x3 chunk) blocks plus one launch per BC stage, a round of
 *    nout sweeps replayed from one CUDA graph; each solve's FP64 outer steps, inner tests
 *    and budget are its own, and its results equal those of sph_solve alone.  infos[i].seconds
 *    and device_ms are those of the whole batch; `threads` is not used.
 *  - Otherwise: sph_solve of every context, handed out to `threads` host threads (<= 0: one
 *    per host core), each context on its own CUDA stream. */
int sph_batch_solve(void* const* ctxs, int32_t n, const sph_solve_opts* opts, sph_solve_info* infos, int32_t threads);

/* Autotuner of the fused FP32 sweep (no counterpart in the reference): times `sweeps`
 * correction sweeps for each candidate x3 chunk length (planes per block) and keeps
 * the fastest for this context and for every later context of the same geometry and
 * grid size.  MIXED with SPH_KERNELS_AUTO only; the FP64 state is not changed. */
int sph_autotune(void* ctx, int32_t sweeps, int32_t* best_chunk, double* best_ms_per_sweep);

/* exactly k reference PT iterations (equal3! ... BC_φ!, SphericalStokes_diapir.jl:413-425) */
int sph_step(void* ctx, int64_t k);

/* iterate to the tolerance; hist_* (may be NULL) receive up to hist_cap (iter, err) pairs */
int sph_solve(void* ctx, const sph_solve_opts* opts, sph_solve_info* info,
              int64_t* hist_iter, double* hist_err, int64_t hist_cap);

/* Wall-clock milliseconds from the start of the last sph_solve on this context to each of its
 * history entries (the (iter, err) pairs it wrote, in order; no counterpart in the reference,
 * whose scripts print the error at each check): *n = number of entries, ms[0 .. min(cap, *n))
 * filled.  For residual-against-time curves of a solve. */
int sph_solve_history_ms(void* ctx, double* ms, int64_t cap, int64_t* n);

/* MIXED only: k FP32 PT sweeps of the current defect-correction step (the hot path of
 * sph_solve).  The first call after the FP64 state changed prepares the step (FP64
 * residual, frozen viscosity, zero correction) outside the timed region;
 * sph_last_device_ms() then returns the device time of the k sweeps.
 * sph_sweep_apply() adds the correction to the FP64 state and ends the step. */
int sph_sweep(void* ctx, int64_t k);
int sph_sweep_apply(void* ctx);

/* Fields of the correction problem that sph_sweep iterates (MIXED only; no counterpart in the
 * reference: the FP32 state of the defect-correction step, for inspection and parity checks):
 * the correction δP, δV1..δV3, δτ11..δτ23 (the sizes of P, V1..V3, τ11..τ23), the frozen
 * viscosity η and ηSM (P's size) and the right-hand sides rP (P's size) and rV1..rV3 (the
 * velocity arrays' sizes).  Values cross the boundary as doubles in the reference layout and
 * are stored as FP32.  The first access after the FP64 state changed prepares the step as
 * sph_sweep does (FP64 residual into rP/rV, η_eff into η, ηSM from it, zero correction);
 * sph_corr_set then overwrites single fields of it, so a caller can pose its own correction
 * problem; sph_sweep and sph_sweep_apply act on what is stored. */
typedef enum sph_corr_field {
    SPH_CORR_DP = 0, SPH_CORR_DV1 = 1, SPH_CORR_DV2 = 2, SPH_CORR_DV3 = 3,
    SPH_CORR_DTAU11 = 4, SPH_CORR_DTAU22 = 5, SPH_CORR_DTAU33 = 6, SPH_CORR_DTAU12 = 7, SPH_CORR_DTAU13 = 8, SPH_CORR_DTAU23 = 9,
    SPH_CORR_ETA = 10, SPH_CORR_ETA_SM = 11, SPH_CORR_RP = 12, SPH_CORR_RV1 = 13, SPH_CORR_RV2 = 14, SPH_CORR_RV3 = 15,
    SPH_CORR_COUNT = 16
} sph_corr_field;
int sph_corr_get(void* ctx, int32_t field, double* host, int64_t count);
int sph_corr_set(void* ctx, int32_t field, const double* host, int64_t count);

/* Self-test of the sweeps' failure path (no counterpart in the reference): launches on the
 * context's stream a one-block kernel that waits, with the TMA sweeps' bounded wait cut to
 * about a millisecond, on a barrier that nothing completes, and records the time-out in the
 * context's error word as a sweep does.  Returns what a sweep call returns after such a
 * time-out: SPH_ERR_CUDA, with the context marked unusable (every later call that launches
 * work on it fails with SPH_ERR_CUDA; destroy it).  No copy or fault is involved. */
int sph_selftest_wait_timeout(void* ctx);

/* MIXED only (no counterpart in the reference: measurement): k sweeps as sph_sweep,
 * launched one at a time with a CUDA event pair on the library's stream around each
 * launch of the fused sweep kernel.  *sweep_ms = device time of the k sweeps (fused
 * kernel + boundary stages), *kernel_ms = summed device time of the k fused-kernel
 * launches.  Needs SPH_KERNELS_AUTO. */
int sph_sweep_profile(void* ctx, int64_t k, double* sweep_ms, double* kernel_ms);

/* Residual fields of the current state (FP64, the SPH_CRIT_RESIDUAL definition before the
 * norms), in the reference layout: rV1..rV3 with the velocity arrays' sizes (non-zero at
 * interior nodes only), rP = div V with the pressure array's size.  NULL skips a field.
 * (No counterpart in the reference, which monitors only the velocity change.) */
int sph_residual_fields(void* ctx, double* rV1, double* rV2, double* rV3, double* rP);

/* Adjoint of the residual (no counterpart in the reference): linear rheology exactly; for the
 * strain-rate law the full Jacobian, η's dependence on V included (sph_residual_vjp_law).
 * In: λ for the residual rows (lV1..lV3 velocity-array sizes, lP pressure size; NULL = 0).
 * Out (NULL skips): aV1..aV3, aP = (∂R/∂(V,P))ᵀ λ; g_eta = (∂R/∂η)ᵀ λ and g_rho = (∂R/∂ρ)ᵀ λ
 * per cell.  flags bit 0: compose with the transposed homogeneous BC program, i.e. the
 * derivative with respect to the interior velocities (boundary entries come out zero);
 * without it every velocity entry is an independent input. */
int sph_residual_vjp(void* ctx, const double* lV1, const double* lV2, const double* lV3, const double* lP, double* aV1,
                     double* aV2, double* aV3, double* aP, double* g_eta, double* g_rho, int32_t flags);

/* After sph_residual_vjp: its η contraction carried through the viscosity law, per cell
 * g_eta_ini = (∂R/∂η_ini)ᵀ λ and the total g_n = (∂R/∂n)ᵀ λ (strain-rate law, unrelaxed target
 * η_t; phase cells and the linear rheology: η = η_ini, g_n = 0).  NULL skips an output.  For
 * the strain-rate law sph_residual_vjp and sph_adjoint_solve include the law's dependence on
 * V (the Jacobian of the residual as the forward solver defines it). */
int sph_residual_vjp_law(void* ctx, double* g_eta_ini, double* g_n);

/* Explicit advection of nf <= 4 cell fields (pressure-array size, reference layout) by the
 * current velocities over dt: first-order upwinding written as a central difference plus a
 * |v|-scaled diffusion, with |v| smoothed to sqrt(v² + delta²) so that the step is
 * differentiable where a velocity component changes sign (delta = 0: plain upwinding);
 * cell-mean velocities and the geometry's metric factors (diapir ascent between solves; the
 * scripts run one time step, so there is no counterpart in the reference). */
int sph_advect(void* ctx, double dt, double delta, int32_t nf, const double* const* phi, double* const* phi_new);

/* Transpose of sph_advect at the same velocities, phi, dt and delta: mu = (∂phi_new/∂phi)ᵀ mu_new
 * per field, aV1..aV3 = (∂phi_new/∂V)ᵀ mu_new summed over the fields (velocity-array sizes,
 * every entry). */
int sph_advect_vjp(void* ctx, double dt, double delta, int32_t nf, const double* const* phi, const double* const* mu_new,
                   double* const* mu, double* aV1, double* aV2, double* aV3);

/* In place: the transposed homogeneous BC program on velocity adjoints (adjoint with respect to
 * every entry -> with respect to the interior entries; boundary entries come out zero). */
int sph_bc_vjp(void* ctx, double* aV1, double* aV2, double* aV3);

/* Transposed PT solve (no counterpart in the reference): λ with Aᵀ λ = b, A the residual's
 * Jacobian in the interior-unknown form of sph_residual_vjp, iterated on the device by the
 * forward scheme transposed: its pseudo-steps (DT_R for the velocity rows, KBDT for the
 * pressure rows) and its stress relaxation, applied to a transposed stress memory.
 * b and λ in the layouts of sph_residual_vjp; λ holds the initial guess on entry.  Stops when
 * max|Aᵀλ - b| <= opts->tol * max|b| (checked every opts->nout iterations) or after
 * opts->maxiter.  Returns the solve status (SPH_OK, SPH_ERR_NOT_CONVERGED, SPH_ERR_DIVERGED). */
int sph_adjoint_solve(void* ctx, const double* bV1, const double* bV2, const double* bV3, const double* bP, double* lV1,
                      double* lV2, double* lV3, double* lP, const sph_solve_opts* opts, sph_solve_info* info);

/* Writes the results in the scripts' output format (Save_infos, Save_phys, SaveArray,
 * SphericalStokes_diapir.jl:23-43, :461-485; CylindricalStokes_diapir.jl:18-37, :390-419;
 * CartesianStokes_diapir.jl:18-37, :404-425) into the directory `dir` (created if absent):
 * <num>_infos.inf, <num>_phys.inf and A_<name>.bin (raw little-endian Float64, column-major,
 * the scripts' array sizes): the coordinate grids, ETAS, RHO, P, the velocities, the six
 * stresses, TII, err_evo and iter_evo (from hist_*, nhist entries; NULL when nhist = 0),
 * and for cylindrical geometry RHOG, DIVV and D_* of the current velocities.  tol and
 * runtime_s fill the εnonl and run-time entries of <num>_infos.inf. */
int sph_save(void* ctx, const char* dir, int32_t num, double tol, double runtime_s, const int64_t* hist_iter,
             const double* hist_err, int64_t nhist);

/* Allocation-free exit check (no counterpart in the reference's interface: it restates
 * the reference's own check, check_err! and the three maximum(abs.(.)) ratios of
 * SphericalStokes_diapir.jl:332-344, :428-432, for caller-owned device arrays).
 * v[i], v_old[i]: DEVICE pointers to count[i] doubles each (any layout); i < m, with
 * 1 <= m <= SPH_NOALLOC_MAX_ARRAYS, beyond which it returns SPH_ERR_INVALID and
 * launches nothing.  *err (host) = max_i max|v[i] - v_old[i]| / max|v[i]|.  Work is
 * queued on `stream` (NULL: the legacy default stream), which the call synchronizes.
 * It allocates no memory: its reduction slots are a static device array of
 * 2 * SPH_NOALLOC_MAX_ARRAYS * 8 bytes shared by every call, so calls that overlap on
 * the GPU race.  The first call on a device looks the array up (cudaGetSymbolAddress)
 * with that device current.  The address is kept for the life of the process, so no call
 * may follow a cudaDeviceReset of that device.  A NaN in v[i] or v_old[i] makes *err NaN (Julia's maximum propagates NaN). */
#define SPH_NOALLOC_MAX_ARRAYS 8
int sph_check_err_noalloc(int32_t m, const double* const* v, const double* const* v_old, const int64_t* count, double* err,
                          void* stream);

/* FP64 Stokes residual of the current state: out[0..2] max|R_mom| per component,
 * out[3] max|div V|, out[4] max|V|, out[5] f_scale, out[6] the SPH_CRIT_RESIDUAL error */
int sph_residual(void* ctx, double out[7]);

/* single reference kernels on the context's state (per-kernel parity):
 * maxloc!+copy_BC!(ηSM), compute_P!, compute_TII!+copy_BC!(τII), power_law!/rheology,
 * compute_V!, BC_R!/BC_θ!/BC_φ! (all stages of the BC set) */
typedef enum sph_kernel {
    SPH_K_MAXLOC = 0, SPH_K_COMPUTE_P = 1, SPH_K_RHEOLOGY = 2, SPH_K_COMPUTE_V = 3, SPH_K_BC = 4
} sph_kernel;
int sph_run_kernel(void* ctx, int32_t kernel);

/* device time (ms) of the last sph_step / sph_solve call measured with CUDA events */
int sph_last_device_ms(void* ctx, double* ms);

const char* sph_strerror(int code);
const char* sph_last_error(void);
int sph_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SPHSTOKES_H */
