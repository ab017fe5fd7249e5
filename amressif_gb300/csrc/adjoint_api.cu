// Host side of the discrete adjoint of the time advance (C ABI of the
// ns_step_adjoint_fwd / ns_step_adjoint_bwd pair, the single-step tangent and
// adjoint, and the predictor Jacobian).
//
// One step of main_main (main.cpp:875-1164) maps (u^n, u^{n-1}, p^n; c) to
// (u^{n+1}, u^n, p^{n+1}):
//   u*      solves G(u*) = S(u^n, u^{n-1}, p^n) + A(u*; c) - (1.5/dt) u* = 0,
//   psi     solves L psi = P0 D u* (L = D G, the Neumann Laplacian of the
//           multigrid; phi = (1.5/dt) psi),
//   u^{n+1} = u* - G psi,  p^{n+1} = p^n + (1.5/dt) psi.
// With J = dG/du* (QUICK switches frozen at u*), the adjoint of one step is
//   ubar*   = ubar' - G L^-1 P0 (D ubar' + (1.5/dt) pbar'),
//   J^T mu  = -ubar*,
//   ubar^n  = uprevbar' + (2/dt) mu,  uprevbar^n = -(0.5/dt) mu,
//   pbar^n  = pbar' + D mu,           cbar += (dA/dc)^T mu,
// (G^T = -D on the interior faces; the S coefficients are those of the step
// source of main.cpp:931-1017). Only u* of step k enters the adjoint of step
// k. A snapshot keeps a time level and the u* of the step that produced it;
// the reverse sweep follows a checkpoint schedule over the snapshot slots
// (dynamic programming on the step / predictor costs, Griewank's binomial
// split for long runs) and recomputes u*_k with the predictor alone only
// inside segments left without a free slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

// argument structs only: the kernels are compiled in kernels_adjoint.cu
#define NS_ADJOINT_ARGS_ONLY
#include "adjoint2d.cuh"
#include "ctx.h"
#include "launch.h"
#include "schedule.h"
#include "state3d.h"

using namespace ns;
using namespace nsh;

namespace nsh {

struct AdjState {
  std::vector<void*> allocs;
  double* US[2] = {nullptr, nullptr};    // u* of the step being differentiated
  double* PHG[2] = {nullptr, nullptr};   // ghosted cell velocity of u*
  double* GH[2] = {nullptr, nullptr};    // ghosted tangent / adjoint cell velocity
  double* FL[4] = {nullptr, nullptr, nullptr, nullptr};  // face flux tangents / adjoints
  double* CT[2] = {nullptr, nullptr};    // cell totals
  double* UADV[2] = {nullptr, nullptr};  // advecting-velocity adjoint
  double* OUT[2] = {nullptr, nullptr};   // operator output scratch
  double* ZERO[2] = {nullptr, nullptr};  // zero faces
  // BiCGStab vectors and scalars
  double* X[2] = {nullptr, nullptr};
  double* R[2] = {nullptr, nullptr};
  double* RH[2] = {nullptr, nullptr};
  double* PV[2] = {nullptr, nullptr};
  double* V[2] = {nullptr, nullptr};
  double* SV[2] = {nullptr, nullptr};
  double* T[2] = {nullptr, nullptr};
  double* BV[2] = {nullptr, nullptr};
  double* sc = nullptr;
  double* sc_h = nullptr;
  // adjoint of the state (u, u_prev, p) and the face / cell scratch
  double* UB[2] = {nullptr, nullptr};
  double* UPB[2] = {nullptr, nullptr};
  double* PB = nullptr;
  double* AUS[2] = {nullptr, nullptr};
  double* TL_DU[2] = {nullptr, nullptr};
  double* TL_DUP[2] = {nullptr, nullptr};
  double* TL_DP = nullptr;
  // lid: per-column tangent / adjoint, per-segment tangent / gradient
  double* DLIDCOL = nullptr;
  double* LIDB = nullptr;
  double* DSEG = nullptr;
  double* SEGACC = nullptr;
  // state snapshots: slot k holds U[2], UP[2], Pp of its time level and u*[2]
  // of the step that produced that level
  double* snap = nullptr;
  int nslots = 0;
  std::vector<int> slot_step;  // -1: free
  std::vector<double> slot_time;
  int final_slot = -1;
  double* ORPH[2] = {nullptr, nullptr};  // u* of a released snapshot, not yet consumed
  // previous adjoint Poisson solution (warm start of the next one)
  double* PSI_PREV = nullptr;
  bool psi_valid = false;
  Schedule sched;  // checkpoint schedule of the last forward run
  // last forward run
  bool have_fwd = false;
  int nsteps = 0, nsnap = 0;
  long long step0 = 0;  // step counter of the context at the start of the forward run
  ns_adjoint_opts opts;
  ns_adjoint_stats st;
};

void free_adjoint(ns_ctx* c) {
  if (!c->adj) return;
  for (void* p : c->adj->allocs) cudaFree(p);
  if (c->adj->snap) cudaFree(c->adj->snap);
  if (c->adj->sc_h) cudaFreeHost(c->adj->sc_h);
  delete c->adj;
  c->adj = nullptr;
}

}  // namespace nsh

namespace {

int adj_alloc(ns_ctx* c, double** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc (adjoint) failed");
  c->adj->allocs.push_back(*p);
  CK(cudaMemsetAsync(*p, 0, bytes, c->st), "memset");
  return NS_OK;
}

int ensure_adj(ns_ctx* c) {
  if (c->adj) return NS_OK;
  c->adj = new AdjState();
  AdjState& A = *c->adj;
  std::memset(&A.opts, 0, sizeof(A.opts));
  std::memset(&A.st, 0, sizeof(A.st));
  const int N = c->N;
  const size_t fb = c->fbytes, gb = (size_t)(N + 4) * (N + 4) * sizeof(double);
  int r = NS_OK;
  for (int m = 0; m < 2 && r == NS_OK; ++m) {
    double** faces[] = {&A.US[m], &A.CT[m], &A.UADV[m], &A.OUT[m], &A.ZERO[m], &A.X[m], &A.R[m], &A.RH[m],
                        &A.PV[m], &A.V[m], &A.SV[m], &A.T[m], &A.BV[m], &A.UB[m], &A.UPB[m], &A.AUS[m],
                        &A.TL_DU[m], &A.TL_DUP[m], &A.FL[2 * m], &A.FL[2 * m + 1], &A.ORPH[m]};
    for (double** p : faces)
      if (r == NS_OK) r = adj_alloc(c, p, fb);
    if (r == NS_OK) r = adj_alloc(c, &A.PHG[m], gb);
    if (r == NS_OK) r = adj_alloc(c, &A.GH[m], gb);
  }
  if (r == NS_OK) r = adj_alloc(c, &A.PB, fb);
  if (r == NS_OK) r = adj_alloc(c, &A.TL_DP, fb);
  if (r == NS_OK) r = adj_alloc(c, &A.PSI_PREV, fb);
  if (r == NS_OK) r = adj_alloc(c, &A.DLIDCOL, (size_t)N * sizeof(double));
  if (r == NS_OK) r = adj_alloc(c, &A.LIDB, (size_t)N * sizeof(double));
  if (r == NS_OK) r = adj_alloc(c, &A.DSEG, (size_t)N * sizeof(double));
  if (r == NS_OK) r = adj_alloc(c, &A.SEGACC, (size_t)N * sizeof(double));
  if (r == NS_OK) r = adj_alloc(c, &A.sc, kBcN * sizeof(double));
  if (r == NS_OK && cudaMallocHost(&A.sc_h, kBcN * sizeof(double)) != cudaSuccess)
    r = fail(c, NS_ERR_NOMEM, "cudaMallocHost (adjoint) failed");
  if (r != NS_OK) free_adjoint(c);
  return r;
}

// ---- host <-> device copies in the ns_set_state layout ---------------------------
int put_faces(ns_ctx* c, int m, const double* h, double* d) {
  const int N = c->N;
  const size_t w = (size_t)(N + (m == 0)), rows = (size_t)(N + (m == 1));
  CK(cudaMemcpy2DAsync(d, c->pitch * sizeof(double), h, w * sizeof(double), w * sizeof(double), rows, cudaMemcpyHostToDevice,
                       c->st),
     "put faces");
  return NS_OK;
}

int get_faces(ns_ctx* c, int m, const double* d, double* h) {
  const int N = c->N;
  const size_t w = (size_t)(N + (m == 0)), rows = (size_t)(N + (m == 1));
  CK(cudaMemcpy2DAsync(h, w * sizeof(double), d, c->pitch * sizeof(double), w * sizeof(double), rows, cudaMemcpyDeviceToHost,
                       c->st),
     "get faces");
  return NS_OK;
}

int put_cells(ns_ctx* c, const double* h, double* d) {
  const int N = c->N;
  CK(cudaMemcpy2DAsync(d, c->pitch * sizeof(double), h, N * sizeof(double), N * sizeof(double), N, cudaMemcpyHostToDevice, c->st),
     "put cells");
  return NS_OK;
}

int get_cells(ns_ctx* c, const double* d, double* h) {
  const int N = c->N;
  CK(cudaMemcpy2DAsync(h, N * sizeof(double), d, c->pitch * sizeof(double), N * sizeof(double), N, cudaMemcpyDeviceToHost, c->st),
     "get cells");
  return NS_OK;
}

int check_supported(ns_ctx* c) {
  if (c->P.dim == 3) return fail(c, NS_ERR_UNSUPPORTED, "adjoint: 2D only");
  if (c->P.conv_scheme != NS_CONV_NEW_QUICK)
    return fail(c, NS_ERR_UNSUPPORTED, "adjoint: differentiates the QUICK predictor (conv_scheme 0) only");
  if (c->g.periodic[0] || c->g.periodic[1])
    return fail(c, NS_ERR_UNSUPPORTED, "adjoint: periodic boxes are not supported");
  if (c->P.pseudo_timestepping == 0)
    return fail(c, NS_ERR_UNSUPPORTED, "adjoint: the explicit predictor is not supported");
  if (c->N % 2 != 0) return fail(c, NS_ERR_ARG, "adjoint: n_cell must be even");
  return NS_OK;
}

// ---- operators --------------------------------------------------------------------
AdjArgs adj_args(ns_ctx* c) {
  AdjState& A = *c->adj;
  AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  for (int m = 0; m < 2; ++m) {
    a.us[m] = A.US[m];
    a.phi[m] = A.PHG[m];
    a.dphi[m] = A.GH[m];
    a.phibar[m] = A.GH[m];
    a.dt_[m] = A.CT[m];
    a.tbar[m] = A.CT[m];
    a.uadv[m] = A.UADV[m];
  }
  for (int k = 0; k < 4; ++k) {
    a.dF[k] = A.FL[k];
    a.Fbar[k] = A.FL[k];
  }
  return a;
}

// ghosted cell velocity of u* (the linearisation point)
int base_cells(ns_ctx* c) {
  AdjState& A = *c->adj;
  LAUNCH(NS_PROF_OTHER, "adjoint base cells",
         launch_adj_cart(c->g, A.US[0], A.US[1], A.PHG[0], A.PHG[1], c->lid_col, 0, c->st));
  return NS_OK;
}

// y = J x + (dA/dc) dlid (transpose = 0) or y = J^T x, lidbar = (dA/dc)^T x
int apply_op(ns_ctx* c, int transpose, double* const* x, const double* dlid, double* const* y, double* lidbar) {
  AdjArgs a = adj_args(c);
  for (int m = 0; m < 2; ++m) a.out[m] = y[m];
  if (!transpose) {
    for (int m = 0; m < 2; ++m) a.v[m] = x[m];
    a.dlid = dlid;
    LAUNCH(NS_PROF_OTHER, "jvp", launch_jvp(a, c->st));
  } else {
    for (int m = 0; m < 2; ++m) a.w[m] = x[m];
    a.lidbar = lidbar;
    LAUNCH(NS_PROF_OTHER, "vjp", launch_vjp(a, c->st));
  }
  return NS_OK;
}

int read_scalars(ns_ctx* c) {
  AdjState& A = *c->adj;
  CK(cudaMemcpyAsync(A.sc_h, A.sc, kBcN * sizeof(double), cudaMemcpyDeviceToHost, c->st), "readback");
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

// BiCGStab for J x = BV (transpose = 0) or J^T x = BV, from the guess in X
int bicgstab(ns_ctx* c, int transpose, double tol, int maxit, int* iters, double* res) {
  AdjState& A = *c->adj;
  BcgArgs b;
  std::memset(&b, 0, sizeof(b));
  b.g = c->g;
  for (int m = 0; m < 2; ++m) {
    b.x[m] = A.X[m];
    b.r[m] = A.R[m];
    b.rh[m] = A.RH[m];
    b.p[m] = A.PV[m];
    b.v[m] = A.V[m];
    b.s[m] = A.SV[m];
    b.t[m] = A.T[m];
    b.b[m] = A.BV[m];
  }
  b.sc = A.sc;
  b.part = c->part;
  b.counter = c->counter;
  auto start = [&]() -> int {
    int r = apply_op(c, transpose, A.X, nullptr, A.V, nullptr);
    if (r != NS_OK) return r;
    LAUNCH(NS_PROF_OTHER, "bicgstab init", launch_bcg(kBcgInit, b, c->st));
    return read_scalars(c);
  };
  int r = start();
  if (r != NS_OK) return r;
  const double bb = A.sc_h[kBcBB];
  *iters = 0;
  if (!(bb > 0.0)) {
    for (int m = 0; m < 2; ++m) CK(cudaMemsetAsync(A.X[m], 0, c->fbytes, c->st), "memset");
    *res = 0.0;
    return NS_OK;
  }
  double rel = std::sqrt(A.sc_h[kBcRR] / bb);
  int it = 0, restarts = 0;
  while (rel > tol && it < maxit) {
    r = apply_op(c, transpose, A.PV, nullptr, A.V, nullptr);
    if (r != NS_OK) return r;
    LAUNCH(NS_PROF_OTHER, "bicgstab alpha", launch_bcg(kBcgAlpha, b, c->st));
    LAUNCH(NS_PROF_OTHER, "bicgstab s", launch_bcg(kBcgS, b, c->st));
    r = apply_op(c, transpose, A.SV, nullptr, A.T, nullptr);
    if (r != NS_OK) return r;
    LAUNCH(NS_PROF_OTHER, "bicgstab omega", launch_bcg(kBcgOmega, b, c->st));
    LAUNCH(NS_PROF_OTHER, "bicgstab x r", launch_bcg(kBcgXR, b, c->st));
    LAUNCH(NS_PROF_OTHER, "bicgstab p", launch_bcg(kBcgP, b, c->st));
    ++it;
    r = read_scalars(c);
    if (r != NS_OK) return r;
    rel = std::sqrt(A.sc_h[kBcRR] / bb);
    if (!std::isfinite(rel)) return fail(c, NS_ERR_CUDA, "BiCGStab: non-finite residual");
    if (A.sc_h[kBcBreak] != 0.0 && rel > tol) {
      // breakdown of the recurrence: restart from the current iterate
      if (++restarts > 8) break;
      r = start();
      if (r != NS_OK) return r;
      rel = std::sqrt(A.sc_h[kBcRR] / bb);
    }
  }
  *iters = it;
  *res = rel;
  return NS_OK;
}

void note_lin(ns_ctx* c, int it, double res) {
  ns_adjoint_stats& s = c->adj->st;
  s.lin_iters += it;
  s.lin_max_iters_seen = std::max(s.lin_max_iters_seen, it);
  s.lin_max_res = std::max(s.lin_max_res, res);
}

// L psi = P0 F with the FP64 multigrid (F, its sum in red[kRedSum] and max|F|
// in red[kRedF] are set), to poisson_tol_rel * max|F|; psi is left in
// PHI[phi_cur]. warm: start from the previous solution of the sweep (the
// adjoint fields change little from one step to the next).
int adj_poisson(ns_ctx* c, bool warm, const double** psi) {
  AdjState& A = *c->adj;
  const double keep = c->P.poisson_tol_div;
  c->P.poisson_tol_div = 0.0;
  c->phi_guess = (warm && A.psi_valid) ? A.PSI_PREV : nullptr;
  c->tol_from_f = true;
  int cyc = 0;
  double res = 0.0;
  const int r = ns_poisson_solve(c, NS_PREC_FP64, &cyc, &res);
  c->P.poisson_tol_div = keep;
  c->phi_guess = nullptr;
  c->tol_from_f = false;
  A.st.poisson_cycles += cyc;
  if (r != NS_OK && !(r == NS_ERR_MG_STALL && res < 1e-9)) return r;
  *psi = c->PHI[c->phi_cur];
  if (warm) {
    CK(cudaMemcpyAsync(A.PSI_PREV, *psi, c->fbytes, cudaMemcpyDeviceToDevice, c->st), "keep psi");
    A.psi_valid = true;
  }
  return NS_OK;
}

// u*_k of the current state (which is not advanced) into US
int predictor_ustar(ns_ctx* c) {
  ns_step_stats s;
  std::memset(&s, 0, sizeof(s));
  c->cart_pending = false;
  int r = run_predictor(c, &s);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m)
    CK(cudaMemcpyAsync(c->adj->US[m], face_ptr(c, c->cur, m), c->fbytes, cudaMemcpyDeviceToDevice, c->st), "copy u*");
  // undo the state rotation of ns_step_begin: the predictor did not write U
  for (int m = 0; m < 2; ++m) std::swap(c->U[m], c->UP[m]);
  c->time -= c->dt;
  c->in_step = false;
  c->adj->st.predictor_runs++;
  if (s.status != NS_OK) c->adj->st.status = s.status;
  return NS_OK;
}

// adjoint of one step at u* = US: (UB, UPB, PB) of state k+1 -> of state k;
// SEGACC += dJ/dc of this step. X holds the guess for mu (warm start).
int adjoint_step(ns_ctx* c) {
  AdjState& A = *c->adj;
  const Geom& g = c->g;
  LAUNCH(NS_PROF_OTHER, "adjoint div",
         launch_adj_div(g, A.UB[0], A.UB[1], A.PB, g.c15, c->F, c->part, c->counter, c->red + kRedSum, c->red + kRedF,
                        c->st));
  const double* psi = nullptr;
  int r = adj_poisson(c, true, &psi);
  if (r != NS_OK) return r;
  LAUNCH(NS_PROF_OTHER, "adjoint gradsub", launch_adj_gradsub(g, A.UB[0], A.UB[1], psi, 1.0, A.AUS[0], A.AUS[1], c->st));
  LAUNCH(NS_PROF_OTHER, "adjoint lincomb",
         launch_adj_lincomb(g, -1.0, A.AUS[0], A.AUS[1], 0.0, nullptr, nullptr, A.BV[0], A.BV[1], c->st));
  r = base_cells(c);
  if (r != NS_OK) return r;
  int it = 0;
  double res = 0.0;
  r = bicgstab(c, 1, A.opts.lin_tol, A.opts.lin_max_iters, &it, &res);
  if (r != NS_OK) return r;
  note_lin(c, it, res);
  if (c->lid_col) {
    r = apply_op(c, 1, A.X, nullptr, A.OUT, A.LIDB);
    if (r != NS_OK) return r;
    LAUNCH(NS_PROF_OTHER, "lid accum", launch_lid_accum(c->N, c->nseg, A.LIDB, 1.0, A.SEGACC, c->st));
  }
  LAUNCH(NS_PROF_OTHER, "adjoint lincomb",
         launch_adj_lincomb(g, 1.0, A.UPB[0], A.UPB[1], g.c15 + g.c05, A.X[0], A.X[1], A.UB[0], A.UB[1], c->st));
  LAUNCH(NS_PROF_OTHER, "adjoint lincomb",
         launch_adj_lincomb(g, -g.c05, A.X[0], A.X[1], 0.0, nullptr, nullptr, A.UPB[0], A.UPB[1], c->st));
  LAUNCH(NS_PROF_OTHER, "adjoint div",
         launch_adj_div(g, A.X[0], A.X[1], A.PB, 1.0, A.PB, c->part, c->counter, c->red + kRedScratch, nullptr, c->st));
  A.st.adjoint_steps++;
  return NS_OK;
}

// tangent of one step at u* = US: (TL_DU, TL_DUP, TL_DP, DLIDCOL if dlid) ->
// (OUT = du', TL_DP = dp'); du_prev' = TL_DU
int tangent_step(ns_ctx* c, bool dlid) {
  AdjState& A = *c->adj;
  const Geom& g = c->g;
  int r = base_cells(c);
  if (r != NS_OK) return r;
  if (dlid) {
    r = apply_op(c, 0, A.ZERO, A.DLIDCOL, A.OUT, nullptr);
    if (r != NS_OK) return r;
  }
  const double* jl[2] = {A.OUT[0], A.OUT[1]};
  const double* du[2] = {A.TL_DU[0], A.TL_DU[1]};
  const double* dup[2] = {A.TL_DUP[0], A.TL_DUP[1]};
  LAUNCH(NS_PROF_OTHER, "tangent rhs", launch_tlm_rhs(g, dlid ? jl : nullptr, A.TL_DP, du, dup, A.BV, c->st));
  int it = 0;
  double res = 0.0;
  r = bicgstab(c, 0, A.opts.lin_tol, A.opts.lin_max_iters, &it, &res);
  if (r != NS_OK) return r;
  note_lin(c, it, res);
  LAUNCH(NS_PROF_OTHER, "tangent div",
         launch_adj_div(g, A.X[0], A.X[1], nullptr, 0.0, c->F, c->part, c->counter, c->red + kRedSum, c->red + kRedF,
                        c->st));
  const double* psi = nullptr;
  r = adj_poisson(c, false, &psi);
  if (r != NS_OK) return r;
  LAUNCH(NS_PROF_OTHER, "tangent gradsub", launch_adj_gradsub(g, A.X[0], A.X[1], psi, 1.0, A.OUT[0], A.OUT[1], c->st));
  LAUNCH(NS_PROF_OTHER, "tangent p", launch_adj_cells(g, 1.0, A.TL_DP, g.c15, psi, A.TL_DP, c->st));
  return NS_OK;
}

// ---- snapshots and the checkpoint schedule ------------------------------------------
// slot k: fields 0-4 = U[2], UP[2], Pp of its time level; 5-6 = u*[2] of the
// step that produced the level
constexpr int kSlotFields = 7;

double* slot_field(ns_ctx* c, int slot, int f) {
  const size_t words = c->fbytes / sizeof(double);
  return c->adj->snap + ((size_t)slot * kSlotFields + f) * words;
}

int copy_pair(ns_ctx* c, double* const* dst, const double* const* src) {
  for (int m = 0; m < 2; ++m)
    CK(cudaMemcpyAsync(dst[m], src[m], c->fbytes, cudaMemcpyDeviceToDevice, c->st), "copy faces");
  return NS_OK;
}

// store the current state as time level `step`; ustar: u* of the step that
// produced it (the predictor buffer after ns_step), nullable
int store_state(ns_ctx* c, int slot, int step, const double* const* ustar) {
  AdjState& A = *c->adj;
  double* src[5] = {c->U[0], c->U[1], c->UP[0], c->UP[1], c->Pp};
  for (int f = 0; f < 5; ++f)
    CK(cudaMemcpyAsync(slot_field(c, slot, f), src[f], c->fbytes, cudaMemcpyDeviceToDevice, c->st), "snapshot store");
  if (ustar) {
    double* d[2] = {slot_field(c, slot, 5), slot_field(c, slot, 6)};
    int r = copy_pair(c, d, ustar);
    if (r != NS_OK) return r;
  }
  A.slot_step[slot] = step;
  A.slot_time[slot] = c->time;
  return NS_OK;
}

int restore_state(ns_ctx* c, int slot) {
  AdjState& A = *c->adj;
  double* dst[5] = {c->U[0], c->U[1], c->UP[0], c->UP[1], c->Pp};
  for (int f = 0; f < 5; ++f)
    CK(cudaMemcpyAsync(dst[f], slot_field(c, slot, f), c->fbytes, cudaMemcpyDeviceToDevice, c->st), "snapshot restore");
  c->time = A.slot_time[slot];
  c->step = A.step0 + A.slot_step[slot];
  c->in_step = false;
  c->cart_pending = false;
  return NS_OK;
}

int advance(ns_ctx* c, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    ns_step_stats s;
    const int r = ns_step(c, &s);
    if (r < 0) return r;
    if (r != NS_OK) c->adj->st.status = r;
    c->adj->st.steps_advanced++;
  }
  return NS_OK;
}

int find_slot(ns_ctx* c, int step) {
  AdjState& A = *c->adj;
  for (int k = 0; k < A.nslots; ++k)
    if (k != A.final_slot && A.slot_step[k] == step) return k;
  return -1;
}

int free_slot(ns_ctx* c) {
  AdjState& A = *c->adj;
  for (int k = 0; k < A.nslots; ++k)
    if (k != A.final_slot && A.slot_step[k] < 0) return k;
  return -1;
}

// adjoint of one step whose u* is in src
int adjoint_with(ns_ctx* c, const double* const* src) {
  int r = copy_pair(c, c->adj->US, src);
  return r != NS_OK ? r : adjoint_step(c);
}

// reverse the steps [a, b): the state of level a is in slot_a, s slots are
// free and ul holds u* of step b-1
int reverse(ns_ctx* c, int a, int b, int s, int slot_a, const double* const* ul) {
  AdjState& A = *c->adj;
  if (b - a <= 0) return NS_OK;
  if (b - a == 1) return adjoint_with(c, ul);
  const int m = A.sched.next(a, b, s);
  if (m < 0) {
    int r = adjoint_with(c, ul);
    for (int k = b - 2; k >= a && r == NS_OK; --k) {
      r = restore_state(c, slot_a);
      if (r == NS_OK) r = advance(c, k - a);
      if (r == NS_OK) r = predictor_ustar(c);
      if (r == NS_OK) r = adjoint_step(c);
    }
    return r;
  }
  int slot_m = find_slot(c, m);
  if (slot_m < 0) {
    slot_m = free_slot(c);
    if (slot_m < 0) return fail(c, NS_ERR_STATE, "checkpoint schedule: no free snapshot slot");
    int r = restore_state(c, slot_a);
    if (r == NS_OK) r = advance(c, m - a);
    const double* us[2] = {face_ptr(c, c->cur, 0), face_ptr(c, c->cur, 1)};
    if (r == NS_OK) r = store_state(c, slot_m, m, us);
    if (r != NS_OK) return r;
  }
  int r = reverse(c, m, b, s - 1, slot_m, ul);
  if (r != NS_OK) return r;
  // the slot's state is no longer needed, its u* (step m-1) is: the left
  // part reverses step m-1 before it releases any other snapshot
  const double* um[2] = {slot_field(c, slot_m, 5), slot_field(c, slot_m, 6)};
  r = copy_pair(c, A.ORPH, um);
  if (r != NS_OK) return r;
  A.slot_step[slot_m] = -1;
  return reverse(c, a, m, s, slot_a, A.ORPH);
}

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

int set_controls_impl(ns_ctx* c, int nseg, const double* controls) {
  if (nseg == 0) {
    c->nseg = 0;
    c->g.lid_u = nullptr;
    if (c->lid_col) cudaFree(c->lid_col);
    c->lid_col = nullptr;
    return NS_OK;
  }
  if (nseg < 0 || nseg > c->N || c->N % nseg != 0 || !controls) return fail(c, NS_ERR_ARG, "controls: nseg must divide n_cell");
  if (c->g.bc[3].rule[0] != kInlet) return fail(c, NS_ERR_BC, "controls: the north side is not an inlet (165)");
  if (!c->lid_col) {
    if (cudaMalloc(&c->lid_col, 2 * (size_t)c->N * sizeof(double)) != cudaSuccess)
      return fail(c, NS_ERR_NOMEM, "cudaMalloc (lid) failed");
  }
  double* seg = c->lid_col + c->N;
  CK(cudaMemcpyAsync(seg, controls, (size_t)nseg * sizeof(double), cudaMemcpyHostToDevice, c->st), "controls upload");
  LAUNCH(NS_PROF_OTHER, "lid expand", launch_lid_expand(c->N, nseg, seg, c->lid_col, c->st));
  CK(cudaStreamSynchronize(c->st), "stream sync");
  c->nseg = nseg;
  c->g.lid_u = c->lid_col;
  return NS_OK;
}

}  // namespace

extern "C" {

void ns_adjoint_opts_default(ns_adjoint_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->nsteps = 400;
  o->nsnap = 20;
  o->lin_tol = 1.0e-12;
  o->lin_max_iters = 500;
}

int ns_set_controls(ns_ctx* c, int nseg, const double* controls) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return fail(c, NS_ERR_UNSUPPORTED, "lid controls: 2D cavity only");
  return set_controls_impl(c, nseg, controls);
}

int ns_step_adjoint_fwd(ns_ctx* c, const ns_adjoint_opts* opts, int nseg, const double* controls, double* J,
                        ns_adjoint_stats* stats) {
  if (!c || !opts || opts->nsteps < 1 || opts->nsnap < 1 || opts->lin_max_iters < 1 || !(opts->lin_tol > 0))
    return NS_ERR_ARG;
  if (c->P.dim == 3) {
    if (nseg != 0) return fail(c, NS_ERR_ARG, "3D adjoint: no lid controls (the control is the initial state)");
    return adjoint_fwd3(c, opts, J, stats);
  }
  int r = check_supported(c);
  if (r != NS_OK) return r;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  const double t0 = now_ms();
  r = set_controls_impl(c, nseg, controls);
  if (r == NS_OK) r = ensure_adj(c);
  if (r != NS_OK) return r;
  AdjState& A = *c->adj;
  A.opts = *opts;
  std::memset(&A.st, 0, sizeof(A.st));
  A.have_fwd = false;
  A.nsteps = opts->nsteps;
  A.nsnap = opts->nsnap;
  A.step0 = c->step;
  // snapshot slots: min(nsnap, nsteps) for the schedule plus one for the final state
  const int nsched = std::min(opts->nsnap, opts->nsteps);
  const int nslots = nsched + 1;
  if (A.nslots != nslots) {
    if (A.snap) cudaFree(A.snap);
    A.snap = nullptr;
    A.nslots = 0;
    if (cudaMalloc(&A.snap, (size_t)nslots * kSlotFields * c->fbytes) != cudaSuccess)
      return fail(c, NS_ERR_NOMEM, "cudaMalloc (snapshots) failed");
    A.nslots = nslots;
  }
  A.slot_step.assign(nslots, -1);
  A.slot_time.assign(nslots, 0.0);
  A.final_slot = nslots - 1;
  A.sched.build(opts->nsteps, nsched - 1);
  // the first descent of the schedule stores its snapshots on the way
  std::vector<int> first;
  {
    int a = 0, s = nsched - 1;
    while (true) {
      const int m = A.sched.next(a, opts->nsteps, s);
      if (m < 0) break;
      first.push_back(m);
      a = m;
      --s;
    }
  }
  c->cart_pending = false;
  r = store_state(c, 0, 0, nullptr);
  if (r != NS_OK) return r;
  size_t next = 0;
  for (int k = 0; k < opts->nsteps; ++k) {
    if (next < first.size() && first[next] == k) {
      const int slot = free_slot(c);
      if (slot < 0) return fail(c, NS_ERR_STATE, "checkpoint schedule: no free snapshot slot");
      const double* us[2] = {face_ptr(c, c->cur, 0), face_ptr(c, c->cur, 1)};
      r = store_state(c, slot, k, us);
      if (r != NS_OK) return r;
      ++next;
    }
    r = advance(c, 1);
    if (r != NS_OK) return r;
  }
  // the final level, with u* of the last step (still in the predictor buffer)
  {
    const double* us[2] = {face_ptr(c, c->cur, 0), face_ptr(c, c->cur, 1)};
    r = store_state(c, A.final_slot, opts->nsteps, us);
    if (r != NS_OK) return r;
  }
  LAUNCH(NS_PROF_OTHER, "objective",
         launch_adj_objective(c->g, c->U[0], c->U[1], c->part, c->counter, c->red + kRedObj, c->st));
  // seed of the reverse sweep: dJ/du^N; zero adjoints of u^{N-1}, p^N, the controls and mu
  LAUNCH(NS_PROF_OTHER, "objective gradient", launch_adj_objective_grad(c->g, c->U[0], c->U[1], A.UB[0], A.UB[1], c->st));
  for (int m = 0; m < 2; ++m) {
    CK(cudaMemsetAsync(A.UPB[m], 0, c->fbytes, c->st), "memset");
    CK(cudaMemsetAsync(A.X[m], 0, c->fbytes, c->st), "memset");
  }
  CK(cudaMemsetAsync(A.PB, 0, c->fbytes, c->st), "memset");
  CK(cudaMemsetAsync(A.SEGACC, 0, (size_t)c->N * sizeof(double), c->st), "memset");
  r = sync_red(c, kRedObj, 1);
  if (r != NS_OK) return r;
  A.st.J = c->red_h[kRedObj];
  A.st.nsteps = opts->nsteps;
  A.st.nsnap = nsched;
  A.st.ms_forward = now_ms() - t0;
  A.have_fwd = true;
  if (J) *J = A.st.J;
  if (stats) *stats = A.st;
  return A.st.status < 0 ? A.st.status : NS_OK;
}

int ns_step_adjoint_bwd(ns_ctx* c, double* grad, ns_adjoint_stats* stats) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return adjoint_bwd3(c, stats);
  if (!c->adj || !c->adj->have_fwd) return fail(c, NS_ERR_STATE, "ns_step_adjoint_bwd needs ns_step_adjoint_fwd first");
  AdjState& A = *c->adj;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  const double t0 = now_ms();
  const int nsched = std::min(A.nsnap, A.nsteps);
  A.psi_valid = false;
  const double* ul[2] = {slot_field(c, A.final_slot, 5), slot_field(c, A.final_slot, 6)};
  int r = reverse(c, 0, A.nsteps, nsched - 1, 0, ul);
  if (r != NS_OK) return r;
  if (grad && c->nseg > 0)
    CK(cudaMemcpyAsync(grad, A.SEGACC, (size_t)c->nseg * sizeof(double), cudaMemcpyDeviceToHost, c->st), "gradient");
  r = restore_state(c, A.final_slot);
  if (r != NS_OK) return r;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  A.have_fwd = false;  // the snapshots of the schedule have been consumed
  A.st.ms_backward = now_ms() - t0;
  if (stats) *stats = A.st;
  return A.st.status < 0 ? A.st.status : NS_OK;
}

int ns_adjoint_get_state_grad(ns_ctx* c, double* const* ubar, double* const* uprevbar, double* pbar) {
  if (c && c->P.dim == 3) return adjoint_state_grad3(c, ubar, uprevbar, pbar);
  if (!c || !c->adj) return NS_ERR_ARG;
  AdjState& A = *c->adj;
  for (int m = 0; m < 2; ++m) {
    if (ubar && ubar[m]) { int r = get_faces(c, m, A.UB[m], ubar[m]); if (r) return r; }
    if (uprevbar && uprevbar[m]) { int r = get_faces(c, m, A.UPB[m], uprevbar[m]); if (r) return r; }
  }
  if (pbar) { int r = get_cells(c, A.PB, pbar); if (r) return r; }
  return ns_sync(c);
}

int ns_step_jvp(ns_ctx* c, const double* const* du, const double* const* duprev, const double* dp, const double* dc,
                double* const* du_out, double* const* duprev_out, double* dp_out) {
  if (!c || !du || !duprev || !dp) return NS_ERR_ARG;
  if (c->P.dim == 3) return step_jvp3(c, du, duprev, dp, du_out, duprev_out, dp_out);
  int r = check_supported(c);
  if (r == NS_OK) r = ensure_adj(c);
  if (r != NS_OK) return r;
  AdjState& A = *c->adj;
  if (A.opts.lin_max_iters == 0) ns_adjoint_opts_default(&A.opts);
  const Geom& g = c->g;
  for (int m = 0; m < 2; ++m) {
    r = put_faces(c, m, du[m], A.TL_DU[m]);
    if (r == NS_OK) r = put_faces(c, m, duprev[m], A.TL_DUP[m]);
    if (r != NS_OK) return r;
  }
  r = put_cells(c, dp, A.TL_DP);
  if (r != NS_OK) return r;
  // boundary faces carry no tangent
  LAUNCH(NS_PROF_OTHER, "mask", launch_adj_lincomb(g, 1.0, A.TL_DU[0], A.TL_DU[1], 0.0, nullptr, nullptr, A.TL_DU[0], A.TL_DU[1], c->st));
  LAUNCH(NS_PROF_OTHER, "mask", launch_adj_lincomb(g, 1.0, A.TL_DUP[0], A.TL_DUP[1], 0.0, nullptr, nullptr, A.TL_DUP[0], A.TL_DUP[1], c->st));
  const bool lid = dc && c->lid_col && c->nseg > 0;
  if (lid) {
    CK(cudaMemcpyAsync(A.DSEG, dc, (size_t)c->nseg * sizeof(double), cudaMemcpyHostToDevice, c->st), "dc upload");
    LAUNCH(NS_PROF_OTHER, "lid expand", launch_lid_expand(c->N, c->nseg, A.DSEG, A.DLIDCOL, c->st));
  }
  r = predictor_ustar(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) CK(cudaMemsetAsync(A.X[m], 0, c->fbytes, c->st), "memset");
  r = tangent_step(c, lid);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) {
    if (du_out && du_out[m]) { r = get_faces(c, m, A.OUT[m], du_out[m]); if (r) return r; }
    if (duprev_out && duprev_out[m]) { r = get_faces(c, m, A.TL_DU[m], duprev_out[m]); if (r) return r; }
  }
  if (dp_out) { r = get_cells(c, A.TL_DP, dp_out); if (r) return r; }
  return ns_sync(c);
}

int ns_step_vjp(ns_ctx* c, const double* const* ubar_out, const double* const* uprevbar_out, const double* pbar_out,
                double* const* ubar, double* const* uprevbar, double* pbar, double* cbar) {
  if (!c || !ubar_out || !uprevbar_out || !pbar_out) return NS_ERR_ARG;
  if (c->P.dim == 3) return step_vjp3(c, ubar_out, uprevbar_out, pbar_out, ubar, uprevbar, pbar);
  int r = check_supported(c);
  if (r == NS_OK) r = ensure_adj(c);
  if (r != NS_OK) return r;
  AdjState& A = *c->adj;
  if (A.opts.lin_max_iters == 0) ns_adjoint_opts_default(&A.opts);
  const Geom& g = c->g;
  A.have_fwd = false;
  for (int m = 0; m < 2; ++m) {
    r = put_faces(c, m, ubar_out[m], A.UB[m]);
    if (r == NS_OK) r = put_faces(c, m, uprevbar_out[m], A.UPB[m]);
    if (r != NS_OK) return r;
  }
  r = put_cells(c, pbar_out, A.PB);
  if (r != NS_OK) return r;
  LAUNCH(NS_PROF_OTHER, "mask", launch_adj_lincomb(g, 1.0, A.UB[0], A.UB[1], 0.0, nullptr, nullptr, A.UB[0], A.UB[1], c->st));
  LAUNCH(NS_PROF_OTHER, "mask", launch_adj_lincomb(g, 1.0, A.UPB[0], A.UPB[1], 0.0, nullptr, nullptr, A.UPB[0], A.UPB[1], c->st));
  CK(cudaMemsetAsync(A.SEGACC, 0, (size_t)c->N * sizeof(double), c->st), "memset");
  r = predictor_ustar(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) CK(cudaMemsetAsync(A.X[m], 0, c->fbytes, c->st), "memset");
  A.psi_valid = false;
  r = adjoint_step(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) {
    if (ubar && ubar[m]) { r = get_faces(c, m, A.UB[m], ubar[m]); if (r) return r; }
    if (uprevbar && uprevbar[m]) { r = get_faces(c, m, A.UPB[m], uprevbar[m]); if (r) return r; }
  }
  if (pbar) { r = get_cells(c, A.PB, pbar); if (r) return r; }
  if (cbar && c->nseg > 0)
    CK(cudaMemcpyAsync(cbar, A.SEGACC, (size_t)c->nseg * sizeof(double), cudaMemcpyDeviceToHost, c->st), "cbar");
  return ns_sync(c);
}

int ns_adjoint_op(ns_ctx* c, int transpose, const double* const* x, const double* dc, double* const* y, double* cbar) {
  if (!c || !x || !y) return NS_ERR_ARG;
  if (c->P.dim == 3) return adjoint_op3(c, transpose, x, y);
  int r = check_supported(c);
  if (r == NS_OK) r = ensure_adj(c);
  if (r != NS_OK) return r;
  AdjState& A = *c->adj;
  const Geom& g = c->g;
  for (int m = 0; m < 2; ++m) {
    r = put_faces(c, m, x[m], A.TL_DU[m]);
    if (r != NS_OK) return r;
  }
  LAUNCH(NS_PROF_OTHER, "mask", launch_adj_lincomb(g, 1.0, A.TL_DU[0], A.TL_DU[1], 0.0, nullptr, nullptr, A.TL_DU[0], A.TL_DU[1], c->st));
  const bool lid = c->lid_col && c->nseg > 0;
  if (lid && dc && !transpose) {
    CK(cudaMemcpyAsync(A.DSEG, dc, (size_t)c->nseg * sizeof(double), cudaMemcpyHostToDevice, c->st), "dc upload");
    LAUNCH(NS_PROF_OTHER, "lid expand", launch_lid_expand(c->N, c->nseg, A.DSEG, A.DLIDCOL, c->st));
  }
  A.have_fwd = false;
  r = predictor_ustar(c);
  if (r == NS_OK) r = base_cells(c);
  if (r != NS_OK) return r;
  if (!transpose) {
    r = apply_op(c, 0, A.TL_DU, (lid && dc) ? A.DLIDCOL : nullptr, A.OUT, nullptr);
  } else {
    r = apply_op(c, 1, A.TL_DU, nullptr, A.OUT, lid ? A.LIDB : nullptr);
    if (r == NS_OK && lid && cbar) {
      CK(cudaMemsetAsync(A.SEGACC, 0, (size_t)c->N * sizeof(double), c->st), "memset");
      LAUNCH(NS_PROF_OTHER, "lid accum", launch_lid_accum(c->N, c->nseg, A.LIDB, 1.0, A.SEGACC, c->st));
      CK(cudaMemcpyAsync(cbar, A.SEGACC, (size_t)c->nseg * sizeof(double), cudaMemcpyDeviceToHost, c->st), "cbar");
    }
  }
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) {
    r = get_faces(c, m, A.OUT[m], y[m]);
    if (r != NS_OK) return r;
  }
  return ns_sync(c);
}

}  // extern "C"
