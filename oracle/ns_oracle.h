/*
 * CPU oracle for the AMRESSIF fractional-step advance (test infrastructure).
 *
 * This is the checker, never the product: only the tests, the smoke check and
 * the CPU-baseline leg of bench.py load it. It restates, function by function,
 * the reference's single-level MAC-grid advance (Source/src1_rever of
 * milk-white-way/AMRESSIF) in plain C++17 (+ optional OpenMP), FP64, with
 * -ffp-contract=off so that x86 and Arm builds give identical bits.
 *
 * Parity status: UNPINNED. The reference ships no golden vectors or tests for
 * this path, and it cannot be built here (AMReX is not vendored and its
 * version is not pinned). The restatement is instead checked against the
 * known answers the reference's own formulas give: the discrete Taylor-Green
 * decay, zero discrete divergence after projection, zero wall-normal velocity,
 * the BDF2 fixed-point identity of the pseudo-time loop, and an independent
 * DCT/FFT solve of the same discrete Poisson problem; against the RK
 * coefficient vector that the reference's only test prints
 * (Tests/loop_test/forloopforvec.cpp); and, bit for bit, against independent
 * vectorised restatements of the RK stage (2D and 3D, every ghost rule and
 * convective routine), the explicit predictor, the Poisson right-hand side,
 * the projection and the box-weighted pseudo-norm (see tests/).
 *
 * Field exchange layout (all arrays dense, x fastest, no ghosts):
 *   face array of direction d : extent N+1 along d, N along the others
 *   cell array                : N^dim
 * Index = i + nx*(j + ny*k) with (nx, ny) the array's own extents.
 */
#ifndef AMRESSIF_NS_ORACLE_H
#define AMRESSIF_NS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Inputs-file keys of the reference (main.cpp:89-157) plus oracle options. */
typedef struct orc_params {
  int dim;                 /* 2 or 3 (AMREX_SPACEDIM) */
  int n_cell;              /* cells per side */
  int max_grid_size[3];    /* box split (only the pseudo-norm summation order depends on it) */
  double prob_lo[3];       /* lo_phy_dim */
  double prob_hi[3];       /* hi_phy_dim */
  double ren;              /* Reynolds number */
  double dt;               /* time step (fixed_dt, or cfl rule evaluated by the caller) */
  int iter_num;            /* IterNum: pseudo-iteration cap */
  double momentum_tolerance;
  int pseudo_timestepping; /* 1: dual-time RK4, 0: explicit mode */
  int bc_lo[3];            /* phy_bc_lo: 111 periodic, 135 no-slip, -135 slip, 165/-165 inlet */
  int bc_hi[3];            /* phy_bc_hi (east code 1 = slip, reference quirk) */
  double inflow[3];        /* inflow_waveform (north inlet only) */
  int fix_quirks;          /* 0: reproduce reference quirks Q1/Q2/Q5/Q6; 1: physically consistent variant */
  double poisson_tol;      /* relative max-norm residual target of the exact solve (<= 1e-12) */
  int nthreads;            /* OpenMP threads (0 = runtime default) */
  int dtau_clip;           /* 1: clip dtau to 0.9 x the RK4 stability limit (grids where 0.4 dt is unstable) */
  int conv_scheme;         /* convective flux routine the predictor calls: 0 convective_flux_calc_new_quick
                              (main.cpp:909,936), 1 convective_flux_calc_quick (fn_flux_calc.cpp:204-393; 2D,
                              one box), 2 convective_flux_calc (fn_flux_calc.cpp:395-692) */
} orc_params;

typedef struct orc_step_stats {
  int pseudo_iters;        /* countIter at loop exit (K) */
  double norm_error;       /* last pseudo-increment norm */
  double div_before;       /* max|div u*| (norm0 printed by poisson_righthand_side_calc) */
  double rhs_sum;          /* sum of Poisson RHS */
  int poisson_iters;       /* oracle Poisson iterations */
  double poisson_res;      /* final relative max-norm residual */
  double div_after;        /* post-step max|div u| (main.cpp:1180) */
  int status;              /* 0 ok, 1 pseudo max-iter warning, 2 pseudo diverged warning */
} orc_step_stats;

typedef struct orc_ctx orc_ctx;

/* Error codes */
#define ORC_OK 0
#define ORC_ERR_ARG -1
#define ORC_ERR_BC -2

int orc_create(const orc_params* p, orc_ctx** out);
void orc_destroy(orc_ctx* c);
const char* orc_last_error(const orc_ctx* c);

/* hybrid_grid_init (fn_init.cpp:30-631): case 0 = lid-driven cavity (zeros),
 * case 1 = Taylor-Green (u = sin x cos y, v = -cos x sin y, p = (cos2x+cos2y)/4,
 * u_prev = exact(t - dt) with nu = 1 as in the reference, or nu = 1/Re with fix_quirks). */
int orc_init(orc_ctx* c, int init_case);

/* State exchange. u[d] are face arrays, p is a cell array. set_state rebuilds
 * velCart by cont2cart(velCont) and the userCtx ghosts; phi is set to zero. */
int orc_set_state(orc_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time);
int orc_get_state(const orc_ctx* c, double* const* u, double* const* u_prev, double* p, double* phi);
/* Optional cell-centred velocity (dim comps, N^dim each) used by the first
 * stage instead of cont2cart(u): the reference's init sets velCart analytically. */
int orc_set_cart(orc_ctx* c, const double* const* cart);

/* One full time step (main.cpp:877-1180). */
int orc_step(orc_ctx* c, orc_step_stats* st);

/* Building blocks, for stage-level parity tests. */
int orc_step_begin(orc_ctx* c);                     /* main.cpp:879-887 */
int orc_rk_stage(orc_ctx* c, int sub);              /* main.cpp:931-1017 */
double orc_pseudo_norm(orc_ctx* c);                 /* Error_Computation + copy back (main.cpp:1019-1026) */
int orc_explicit_predictor(orc_ctx* c, double* norm);/* main.cpp:902-925 */
int orc_poisson_rhs(orc_ctx* c, double* divmax, double* sum); /* fn_rhs.cpp:71-125 on velStar */
int orc_poisson_solve(orc_ctx* c, int* iters, double* res);    /* exact discrete solve of L phi = f */
int orc_project(orc_ctx* c, double* divmax);        /* main.cpp:1078-1164 + divergence check */

/* Raw access for tests: which = 0 velStar, 1 velCont (u_base), 2 velContPrev, 3 velContDiff,
 * 4 momentum_rhs; cell fields: 10 pressure, 11 phi, 12 poisson_rhs, 13+m velCart comp m,
 * 20+m fluxTotal comp m. Copies the valid region into out (face or cell layout). */
int orc_get_field(const orc_ctx* c, int which, int comp, double* out);
int orc_put_field(orc_ctx* c, int which, int comp, const double* in);

/* Solve L phi = f (5/7-point, Neumann/periodic as configured) for a given RHS:
 * f and phi are cell arrays. Mean of f is removed as AMReX MLMG does for singular problems. */
int orc_solve_poisson_array(orc_ctx* c, const double* f, double* phi, int* iters, double* res);

#ifdef __cplusplus
}
#endif
#endif
