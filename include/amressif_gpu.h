/*
 * amressif_gb300 — C ABI of the GB300 (sm_103a) fractional-step advance of
 * AMRESSIF (milk-white-way/AMRESSIF, Source/src1_rever).
 *
 * The reference has no plugin layer: main_main (main.cpp:51-1213) calls free
 * functions over amrex::MultiFab. Each entry point below replaces one of
 * those call sites (cited per function, paths relative to
 * Source/src1_rever). The library owns its device buffers (an opaque
 * ns_ctx); an AMReX host moves MultiFab boxes in and out with
 * ns_put_box / ns_get_box, which take Array4-style strided views.
 *
 * All functions return an int status (NS_OK = 0, negative = error,
 * positive = warning) and never abort the process. All work is enqueued on
 * the stream given at creation.
 */
#ifndef AMRESSIF_GPU_H
#define AMRESSIF_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NS_OK 0
#define NS_WARN_PSEUDO_MAXITER 1  /* main.cpp:1030-1033: countIter > IterNum, step continued */
#define NS_WARN_PSEUDO_DIVERGED 2 /* main.cpp:1035-1038: normError > 1e2, step continued */
#define NS_ERR_ARG -1             /* bad argument or parameter */
#define NS_ERR_BC -2              /* BC code the reference aborts on (main.cpp:822,832, utilities.cpp:135-179) */
#define NS_ERR_CUDA -3            /* CUDA runtime error (message in ns_last_error) */
#define NS_ERR_MG_STALL -4        /* Poisson residual stopped decreasing before the tolerance */
#define NS_ERR_NOMEM -5           /* device allocation failed */
#define NS_ERR_STATE -6           /* call out of sequence (e.g. stage before step_begin) */
#define NS_ERR_UNSUPPORTED -7     /* valid reference input the library does not implement */
#define NS_ERR_NONFINITE -8       /* NaN in the pseudo-increment norm, or a non-finite Poisson right-hand side
                                     (e.g. NaN in the input fields): the step is abandoned where it was
                                     found; set a state before the next step. The reference's loop test
                                     (main.cpp:898) is false for NaN, so it would carry the NaN on silently */

/* ---- precision modes ----------------------------------------------------- */
#define NS_PREC_FP64_EXACT 0 /* reference operation order, no FMA: bit-exact stages */
#define NS_PREC_FP64 1       /* FP64 everywhere, FMA and reciprocal multiplies */
#define NS_PREC_MIXED 2      /* float-float anchors + FP32 increments in the predictor; FP32 V-cycles inside a
                                defect correction whose residual is float-float (dc_residual = 0) or FP64
                                (dc_residual = 1); FP64 projection, pressure update and divergence check */

/* ---- initial conditions of hybrid_grid_init (fn_init.cpp:30-631) ------- */
#define NS_INIT_CAVITY 0 /* all zero (the shipped source) */
#define NS_INIT_TGV 1    /* u = sin x cos y, v = -cos x sin y, p = (cos 2x + cos 2y)/4 */

/* ---- field identifiers for ns_put_box / ns_get_box ---------------------- */
#define NS_FIELD_VEL 0      /* velCont[comp] (face-centred) */
#define NS_FIELD_VEL_PREV 1 /* velContPrev[comp] */
#define NS_FIELD_PRESSURE 2 /* userCtx comp 0 */
#define NS_FIELD_PHI 3      /* userCtx comp 1 / poisson_sol */
#define NS_FIELD_VEL_STAR 4 /* velStar[comp] (current pseudo-iterate) */
#define NS_FIELD_POISSON_RHS 5
#define NS_FIELD_CART 6     /* velCart[comp] override for the first stage (cell-centred) */

/* Inputs-file keys of the reference (main.cpp:89-157) plus GPU options. */
typedef struct ns_params {
  int dim;                   /* AMREX_SPACEDIM: 2 or 3 (3: the whole-step API and the adjoint pair) */
  int n_cell;                /* cells per direction. Deviation: the reference takes any n_cell
                                (main.cpp:310-324); here it must be a multiple of 8 (else NS_ERR_ARG)
                                whose multigrid hierarchy, halving while n % 4 == 0 and n > 4, ends at
                                32 or less in 2D and 24 or less in 3D (else NS_ERR_UNSUPPORTED): e.g.
                                40, 128, 4096 are taken, 808 is not */
  int max_grid_size[3];      /* accepted for drop-in; the GPU runs one box */
  double prob_lo[3];         /* lo_phy_dim (default 0) */
  double prob_hi[3];         /* hi_phy_dim (default 1) */
  double ren;                /* Reynolds number */
  double vis;                /* read but unused, as in the reference */
  double cfl;                /* dt = cfl / (2 sum 1/dx^2) unless fixed_dt > 0 (main.cpp:285-294) */
  double fixed_dt;           /* -1 = use cfl rule */
  int iter_num;              /* IterNum */
  double momentum_tolerance; /* 1e-10 */
  int pseudo_timestepping;   /* 1 dual-time RK4, 0 explicit */
  int bc_lo[3], bc_hi[3];    /* phy_bc_lo / phy_bc_hi codes */
  double inflow_waveform[3];
  int nsteps;
  /* GPU options */
  int precision;             /* NS_PREC_* */
  int fix_quirks;            /* 0 = reproduce reference quirks (flux / pressure ghost mirroring in periodic directions) */
  double poisson_tol_rel;    /* max-norm residual relative to the RHS (MLMG tol_rel, 1e-10) */
  double poisson_tol_div;    /* additionally require max|div u| <= this after projection (0 = off) */
  int poisson_max_cycles;    /* V-cycle / defect-correction cap (MLMG maxiter 2000) */
  int dtau_clip;             /* 0: dtau = 0.4 dt (main.cpp:861); 1: also clip to 0.9 x RK4 stability limit */
  int poisson_solver;        /* 0: multigrid V-cycles; 1: restarted GMRES with one FP64 V-cycle as right
                                preconditioner (the GMRES option of GMRES_Poisson.cpp:56-131), 2D and 3D,
                                FP64 in every precision mode */
  int gmres_restart;         /* Krylov vectors per GMRES cycle (<= 31) */
  int dc_residual;           /* NS_PREC_MIXED Poisson: the defect correction's residual and phi in
                                0 = float-float (about 48 bits; FP64 once its floor is reached),
                                1 = FP64 from the first sweep (2D and 3D) */
  int poisson_warm_start;    /* NS_PREC_MIXED Poisson (2D, float-float defect correction): 1 = start from
                                the previous step's phi instead of zero (poisson.cpp:63 starts from zero).
                                The tolerance stays relative to the zero-guess residual max|f - mean f|,
                                so the solve meets the same residual bound in fewer V-cycles. The result
                                then depends on the previous step's phi at the tolerance level. 0 = off */
  int conv_scheme;           /* convective flux routine of the predictor (NS_CONV_*). main_main calls
                                convective_flux_calc_new_quick (main.cpp:909,936); the other two are the
                                reference's alternatives, FP64 modes only (NS_PREC_MIXED and the adjoint
                                give NS_ERR_UNSUPPORTED) */
} ns_params;

/* ns_params.conv_scheme */
#define NS_CONV_NEW_QUICK 0  /* convective_flux_calc_new_quick (fn_flux_calc.cpp:11-202): QUICK; the default */
#define NS_CONV_QUICK 1      /* convective_flux_calc_quick (fn_flux_calc.cpp:204-393) as written: its QUICK
                                weight Real(1/8) is 0 (first-order upwind faces), face N copies face 0, and
                                the y differences are taken at i+1 through the flat face fab. 2D, one box
                                (max_grid_size >= n_cell in x and y): with more boxes and in 3D the routine
                                reads and writes outside its fabs. Else NS_ERR_UNSUPPORTED */
#define NS_CONV_UMIST_FORM 2 /* convective_flux_calc (fn_flux_calc.cpp:395-692): forms fluxConvect, which
                                only Export_Fluxes reads, and never updates fluxTotal, so the predictor has
                                no convective term. 2D and 3D */

typedef struct ns_step_stats {
  int pseudo_iters;   /* K (countIter at exit) */
  double norm_error;  /* last pseudo-increment norm */
  double div_before;  /* max|div u*| (fn_rhs.cpp:103-104) */
  double rhs_sum;     /* sum of the Poisson RHS (fn_rhs.cpp:123-124) */
  int poisson_cycles; /* V-cycles (FP64) or defect-correction sweeps (mixed) */
  double poisson_res; /* final max-norm residual / max-norm RHS */
  double div_after;   /* post-step max|div u| (main.cpp:1180) */
  int status;         /* NS_OK or NS_WARN_* */
  double ms_predictor, ms_poisson, ms_project; /* device time of the phases */
  int poisson_fp64_fallback; /* mixed solve: 1 if the float-float residual floor forced FP64 sweeps */
  double ms_h2d, ms_d2h;      /* ns_step_host: device time of the host->device copies of (u, u_prev, p) and
                                 of the device->host copies after the step (2D: u and p; u_prev is copied
                                 while the step runs); 0 for ns_step */
} ns_step_stats;

typedef struct ns_ctx ns_ctx;

/* Defaults: the shipped Exec/inputs physics with a valid chk_int (no restart). */
void ns_params_default(ns_params* p);

/* Parse a reference inputs file (ParmParse key = value lines, '#' comments)
 * into p (keys it does not know are ignored). Returns NS_OK or NS_ERR_ARG. */
int ns_params_parse_file(ns_params* p, const char* path);

/* main.cpp:267-383 (geometry, BoxArray, MultiFab allocation). stream is a
 * cudaStream_t (NULL = the context creates its own). */
int ns_ctx_create(const ns_params* p, void* stream, ns_ctx** out);
void ns_ctx_destroy(ns_ctx* c);
const char* ns_last_error(const ns_ctx* c);
double ns_get_dt(const ns_ctx* c);
double ns_get_time(const ns_ctx* c);

/* hybrid_grid_init (fn_init.cpp:30-631) for init_case NS_INIT_*. In 3D the
 * Taylor-Green case is the reference's 2D vortex in every z plane (its z
 * factors are commented out): w = 0, and w = 0 in the analytic cell velocity.
 * Both dimensions give the first stage the analytic cell velocity, as the
 * reference does; the adjoint replaces it by cont2cart's. */
int ns_init_fields(ns_ctx* c, int init_case);

/* Move one box of a field between the caller and the device
 * (MultiFab::array(mfi) views, 2D and 3D). data is indexed
 *   data[(i-lo[0]) + (j-lo[1])*jstride + (k-lo[2])*kstride]
 * over the inclusive index box [lo, hi] in the field's own index space
 * (face fields extend to n_cell along their direction). An AMReX host passes
 * the Array4 of a ghosted FArrayBox offset to the valid box's lo, with the
 * Array4's jstride and kstride. NS_ERR_ARG if the box leaves the field, if
 * jstride is below the box width or, for boxes of more than one plane,
 * kstride below jstride times the box height; a 2D context takes only the
 * plane lo[2] = hi[2] = 0 (kstride unused). where_device = 1 if data is
 * device memory. ns_put_box from host memory and ns_get_box wait for the
 * stream before they return. NS_FIELD_CART (put only) is the cell velocity of
 * the next FP64 stage in place of cont2cart's; ns_set_state clears it. */
int ns_put_box(ns_ctx* c, int field, int comp, const double* data, const int lo[3], const int hi[3],
               long long jstride, long long kstride, int where_device);
int ns_get_box(ns_ctx* c, int field, int comp, double* data, const int lo[3], const int hi[3],
               long long jstride, long long kstride, int where_device);

/* Whole-state convenience (dense host arrays, x fastest): u[d] (d < dim) are
 * face arrays of extent n_cell+1 along d and n_cell along the others, p is a
 * cell array. */
int ns_set_state(ns_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time);
int ns_get_state(ns_ctx* c, double* const* u, double* const* u_prev, double* p, double* phi);

/* Checkpoint / restart state of SaveCheckpoint / LoadCheckpoint
 * (utilities.cpp:792-1023): u^n, u^{n-1}, p, the time and the number of steps
 * taken. phi is not part of it (the reference does not save it either; the
 * advance recomputes it every step). After ns_checkpoint_put the next ns_step
 * continues the saved run bit for bit: the cell velocity of the first stage
 * is rebuilt from the faces, as a restart of the reference does
 * (main.cpp:387-784). Host arrays as in ns_set_state. */
int ns_checkpoint_get(ns_ctx* c, double* const* u, double* const* u_prev, double* p, double* time, long long* step);
int ns_checkpoint_put(ns_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time,
                      long long step);
long long ns_get_step(const ns_ctx* c);

/* The cell-centred velocity velCart that Export_Flow_Field plots
 * (utilities.cpp:534-570): the face averages of cont2cart
 * (utilities.cpp:49-53) of the current u^n, computed on the device. cart[d]
 * (d < dim) are dense host arrays of n_cell^dim values, x fastest. */
int ns_get_cell_velocity(ns_ctx* c, double* const* cart);

/* ---- building blocks, one per reference call site ------------------------ */
int ns_step_begin(ns_ctx* c);                              /* main.cpp:879-887 */
int ns_rk_stage(ns_ctx* c, int sub);                       /* main.cpp:931-1017 (fused) */
int ns_pseudo_norm(ns_ctx* c, double* norm);               /* Error_Computation, main.cpp:1019-1026 */
int ns_explicit_predictor(ns_ctx* c, double* norm);        /* main.cpp:902-925 */
int ns_poisson_rhs(ns_ctx* c, double* divmax, double* sum);/* fn_rhs.cpp:71-125 on velStar */
int ns_poisson_solve(ns_ctx* c, int precision, int* cycles, double* res); /* poisson.cpp:41-186 */
int ns_project(ns_ctx* c, double* divmax);                 /* main.cpp:1078-1164 + main.cpp:1180 */

/* One full time step (main.cpp:877-1180); stats may be NULL. */
int ns_step(ns_ctx* c, ns_step_stats* stats);

/* End-to-end host call: upload (u, u_prev, p) from host memory, advance one
 * step, download (u, u_prev, p); the arrays are dense as in ns_set_state and
 * are updated in place. The copies and the step are enqueued on the context's
 * stream without intermediate waits; in 2D the outgoing u_prev (the incoming
 * u, which the step does not change) is copied back on a second stream while
 * the step runs. Use pinned buffers (ns_host_alloc) for full copy speed. */
int ns_step_host(ns_ctx* c, double* const* u, double* const* u_prev, double* p, ns_step_stats* stats);

/* Synchronise the context's stream. */
int ns_sync(ns_ctx* c);

/* ---- instrumentation (no reference counterpart: replaces TinyProfiler
 * regions, Exec/GNUmakefile:13, and the per-step timer of main.cpp:1173-1175)
 * Per-kernel-kind device time from CUDA events around every launch on the
 * context's stream, and the number of kernels launched. */
#define NS_PROF_STAGE_EXACT 0
#define NS_PROF_STAGE_FAST 1
#define NS_PROF_ANCHOR 2
#define NS_PROF_INC 3
#define NS_PROF_EXPLICIT 4
#define NS_PROF_STEP_BEGIN 5
#define NS_PROF_POISSON_RHS 6
#define NS_PROF_PROJECT 7
#define NS_PROF_MG_SMOOTH0 8   /* finest-level smoothing (+ prolongation) */
#define NS_PROF_MG_SMOOTH 9
#define NS_PROF_MG_RESTRICT0 10
#define NS_PROF_MG_RESTRICT 11
#define NS_PROF_MG_BOTTOM 12
#define NS_PROF_MG_RESNORM 13
#define NS_PROF_DC_UPDATE 14
#define NS_PROF_OTHER 15
#define NS_PROF_MG_CYCLE 16 /* one V-cycle replayed as a CUDA graph (its kernels are not timed one by one) */
#define NS_PROF_KINDS 17
/* Poisson right-hand side without any device allocation. No counterpart in
 * the reference. For callers that cannot call cudaMalloc: a host whose device
 * memory all belongs to its own arena allocator (AMReX's), or a job whose
 * memory budget is fixed once it starts. Computes f = (1.5/dt) div u from
 * caller-owned device arrays, all with row pitch `pitch` elements
 * (pitch >= n_cell + 1; element (i, j) at j * pitch + i):
 *   u: x faces, n_cell rows of n_cell + 1 values;
 *   v: y faces, n_cell + 1 rows of n_cell values;
 *   f: cells, n_cell rows of n_cell values (written).
 * Returns {max|div u|, sum f} in divmax_sum[2] (host memory). The call
 * synchronises `stream` (a cudaStream_t, NULL = default stream) before it
 * returns, so it cannot be made during a stream capture. dx, dy and dt must be
 * finite and positive (NS_ERR_ARG otherwise). The reduction scratch is a fixed
 * device array of about 128 KB inside the library, held on every GPU that
 * loads it until the process exits: n_cell above 4096 is rejected with
 * NS_ERR_UNSUPPORTED. Each call looks up that array's device address on the
 * current device and clears its counter. All calls share the array, so calls
 * that overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. Results are bit-identical to ns_poisson_rhs. */
int ns_poisson_rhs_noalloc(const double* u, const double* v, double* f, int n_cell, long long pitch, double dx, double dy,
                           double dt, double* divmax_sum, void* stream);

/* Page-locked host memory for the ns_step_host / ns_put_box buffers of a
 * host that keeps its fields in CPU memory (cudaMallocHost). */
void* ns_host_alloc(unsigned long long bytes);
void ns_host_free(void* p);

/* ns_profile_enable(c, 1) waits for the stream and creates the event pool
 * (two events per launch, filled once), so switch it on outside a timed
 * region. The event pairs are read out only by ns_profile_read (which waits
 * for the stream), by ns_profile_enable, and when several thousand launches
 * are pending, never at the syncs inside a step. */
int ns_profile_enable(ns_ctx* c, int on);
int ns_profile_read(ns_ctx* c, double* ms, long long* counts, int nkinds, int reset);
long long ns_launch_count(const ns_ctx* c);

/* Bounds-check build (libamressif_gb300_check.so, compiled with
 * -DNS_BOUNDS_CHECK; the counterpart of the reference's DEBUG=TRUE build,
 * Exec/GNUmakefile:12): the column-marching predictor kernels and the
 * multigrid smoothers test every index they form by hand against the array
 * it addresses, skip a failing access and record it. status[0] = number of
 * failed tests, status[1] = the first failing index, status[2] = its site
 * (bounds.cuh). Waits for the stream; reset = 1 clears the words. The normal
 * build returns NS_ERR_UNSUPPORTED (and zeros). */
int ns_bounds_check_read(ns_ctx* c, unsigned long long* status, int reset);

/* ---- Discrete adjoint of the time advance (2D wall / lid boxes) ----------
 *
 * The differentiated map is one converged step of main_main's loop
 * (main.cpp:875-1164): the BDF2 predictor u* solving G(u*) = 0 with the
 * QUICK upwind switches frozen at u*, the Poisson solve and the projection.
 * Tangent and adjoint linear solves run in FP64 (BiCGStab on the interior
 * faces); the Poisson solves reuse the FP64 multigrid (self-adjoint). The
 * forward steps use the context's precision. Periodic boxes and the explicit
 * predictor (PSEUDO_TIMESTEPPING = 0) return NS_ERR_UNSUPPORTED.
 *
 * Controls: the north inlet's u is a piecewise-constant lid profile of nseg
 * segments of n_cell / nseg columns; the north ghost becomes 2 c_k - phi
 * (generalising the uniform inflow_waveform[0] of utilities.cpp:255).
 *
 * Objective: J = 1/2 sum over the cells of [lo, lo + L/2]^2 of
 * (phi_u^2 + phi_v^2) dx dy at the final step (phi: cont2cart cell average). */

typedef struct ns_adjoint_opts {
  int nsteps;          /* steps of the forward run */
  int nsnap;           /* device state snapshots incl. the initial state (>= 1); >= nsteps keeps every step */
  double lin_tol;      /* BiCGStab: ||r|| <= lin_tol ||b|| */
  int lin_max_iters;   /* BiCGStab iteration cap per solve */
} ns_adjoint_opts;

typedef struct ns_adjoint_stats {
  double J;                 /* objective of the forward run */
  int nsteps, nsnap;
  long long steps_advanced; /* forward steps, first sweep and recomputation */
  long long predictor_runs; /* predictor-only recomputations of u* */
  long long adjoint_steps;
  long long lin_iters;      /* BiCGStab iterations, all solves */
  int lin_max_iters_seen;
  double lin_max_res;       /* largest final relative residual: ||r|| / ||b||, or max|r| / max|b| for the
                               mixed-precision (refined) 3D solves */
  long long poisson_cycles; /* adjoint Poisson V-cycles */
  double ms_forward;        /* wall time of ns_step_adjoint_fwd */
  double ms_backward;       /* wall time of ns_step_adjoint_bwd */
  int status;
} ns_adjoint_stats;

void ns_adjoint_opts_default(ns_adjoint_opts* o);

/* Sets the lid controls (host array of nseg values; nseg divides n_cell). nseg
 * = 0 restores the uniform inflow_waveform lid. */
int ns_set_controls(ns_ctx* c, int nseg, const double* controls);

/* Forward half of the pair (the analogue of an autograd Function's forward):
 * sets the controls, runs opts->nsteps steps from the current state keeping
 * opts->nsnap snapshots (placed by a dynamic-programming schedule, the
 * binomial one as fallback), and returns J. 2D: J = kinetic energy of the
 * lower-left quarter, with nseg lid controls. 3D (periodic boxes,
 * fix_quirks = 1): J = the final enstrophy 1/2 sum |curl u|^2 dV, nseg = 0.
 * The context is left at the final state. */
int ns_step_adjoint_fwd(ns_ctx* c, const ns_adjoint_opts* opts, int nseg, const double* controls, double* J,
                        ns_adjoint_stats* stats);

/* Backward half: reverse sweep from the snapshots of the last
 * ns_step_adjoint_fwd, returning dJ/dcontrols (host, nseg values). The
 * gradient with respect to the initial state is kept and can be read with
 * ns_adjoint_get_state_grad. The context is left at the final state. */
int ns_step_adjoint_bwd(ns_ctx* c, double* grad, ns_adjoint_stats* stats);

/* dJ/d(u^0, u^{-1}, p^0) of the last backward sweep (host arrays in the
 * ns_set_state layout; any pointer may be NULL). */
int ns_adjoint_get_state_grad(ns_ctx* c, double* const* ubar, double* const* uprevbar, double* pbar);

/* One linearised step at the current state (which is not advanced):
 * tangent: (du, du_prev, dp, dc) -> (du', du_prev', dp') and
 * adjoint: (ubar', uprevbar', pbar') -> (ubar, uprevbar, pbar, cbar).
 * Host arrays in the ns_set_state layout; dc / cbar have nseg values (NULL
 * when no controls are set). */
int ns_step_jvp(ns_ctx* c, const double* const* du, const double* const* duprev, const double* dp, const double* dc,
                double* const* du_out, double* const* duprev_out, double* dp_out);
int ns_step_vjp(ns_ctx* c, const double* const* ubar_out, const double* const* uprevbar_out, const double* pbar_out,
                double* const* ubar, double* const* uprevbar, double* pbar, double* cbar);

/* The predictor Jacobian at the current state's u*: y = J x (transpose = 0)
 * or y = J^T x (transpose = 1), plus the lid term (dc in, cbar out; NULL to
 * skip). Faces in the ns_set_state layout. */
int ns_adjoint_op(ns_ctx* c, int transpose, const double* const* x, const double* dc, double* const* y, double* cbar);

#ifdef __cplusplus
}
#endif
#endif
