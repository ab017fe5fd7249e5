// Host side of the 3D discrete adjoint (periodic boxes in the physical mode):
// the ns_step_adjoint_fwd / ns_step_adjoint_bwd pair for the final enstrophy
// E = 1/2 sum |curl u|^2 dV, the single-step tangent and adjoint, and the
// predictor Jacobian. The chain of one step and of its adjoint is the 2D one
// (adjoint_api.cu) with three components; the kernels are in adjoint3d.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#define NS_ADJOINT_ARGS_ONLY
#include "adjoint2d.cuh"  // BiCGStab scalar slots
#include "state3d.h"
#include "adjoint3d.cuh"
#include "schedule.h"

using namespace ns;
using namespace nsh;

namespace nsh {

struct Adj3 {
  std::vector<void*> allocs;
  double* US[3] = {};
  double* PHB[3] = {};
  double* Q[3][3] = {};
  double* DPH[3] = {};
  double* FL[3][3] = {};
  double* CT[3] = {};
  double* UADV[3] = {};
  double* OUT[3] = {};
  double* X[3] = {};
  double* R[3] = {};
  double* RH[3] = {};
  double* PV[3] = {};
  double* V[3] = {};
  double* SV[3] = {};
  double* T[3] = {};
  double* BV[3] = {};
  double* UB[3] = {};
  double* UPB[3] = {};
  double* AUS[3] = {};
  double* TL_DU[3] = {};
  double* TL_DUP[3] = {};
  double* OM[3] = {};
  double* ORPH[3] = {};
  // mixed-precision refinement: FP32 base operands and inner BiCGStab vectors
  bool mixed = false;
  float* US32[3] = {};
  float* PHB32[3] = {};
  float* Q32[3][3] = {};
  float* XF[3] = {};
  float* RF[3] = {};
  float* RHF[3] = {};
  float* PF[3] = {};
  float* VF[3] = {};
  float* SF[3] = {};
  float* TF[3] = {};
  double* PB = nullptr;
  double* TL_DP = nullptr;
  double* sc = nullptr;
  double* sc_h = nullptr;
  double* snap = nullptr;
  int nslots = 0, final_slot = -1;
  std::vector<int> slot_step;
  std::vector<double> slot_time;
  Schedule sched;
  bool have_fwd = false;
  int nsteps = 0, nsnap = 0;
  long long step0 = 0;
  ns_adjoint_opts opts;
  ns_adjoint_stats st;
};

void free_adj3(ns_ctx* c) {
  if (!c->s3 || !c->s3->adj) return;
  Adj3* A = c->s3->adj;
  for (void* p : A->allocs) cudaFree(p);
  if (A->snap) cudaFree(A->snap);
  if (A->sc_h) cudaFreeHost(A->sc_h);
  delete A;
  c->s3->adj = nullptr;
}

}  // namespace nsh

namespace {

constexpr int kSlot3 = 10;  // U[3], UP[3], p, u*[3]

inline dim3 cells_grid(int N) { return dim3((N + 31) / 32, (N + 7) / 8, N); }

int need3(ns_ctx* c) {
  const Geom& g = c->g;
  for (int d = 0; d < 3; ++d)
    if (!g.periodic[d] || g.flux_ghost[d] != kWrap || g.ctx_mirror[d] != 0)
      return fail(c, NS_ERR_UNSUPPORTED, "3D adjoint: periodic boxes in the physical mode (fix_quirks = 1) only");
  if (c->P.pseudo_timestepping == 0) return fail(c, NS_ERR_UNSUPPORTED, "3D adjoint: the explicit predictor is not built");
  if (c->P.conv_scheme != NS_CONV_NEW_QUICK)
    return fail(c, NS_ERR_UNSUPPORTED, "3D adjoint: differentiates the QUICK predictor (conv_scheme 0) only");
  return NS_OK;
}

int ensure3(ns_ctx* c) {
  State3D& S = *c->s3;
  if (S.adj) return NS_OK;
  S.adj = new Adj3();
  Adj3& A = *S.adj;
  std::memset(&A.opts, 0, sizeof(A.opts));
  std::memset(&A.st, 0, sizeof(A.st));
  auto al = [&](double** p, size_t bytes) -> int {
    if (cudaMalloc(p, bytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc (3D adjoint) failed");
    A.allocs.push_back(*p);
    CK(cudaMemsetAsync(*p, 0, bytes, c->st), "memset");
    return NS_OK;
  };
  int r = NS_OK;
  for (int m = 0; m < 3 && r == NS_OK; ++m) {
    double** fs[] = {&A.US[m], &A.PHB[m], &A.DPH[m], &A.CT[m], &A.UADV[m], &A.OUT[m], &A.X[m], &A.R[m], &A.RH[m],
                     &A.PV[m], &A.V[m], &A.SV[m], &A.T[m], &A.BV[m], &A.UB[m], &A.UPB[m], &A.AUS[m], &A.TL_DU[m],
                     &A.TL_DUP[m], &A.OM[m], &A.ORPH[m], &A.Q[0][m], &A.Q[1][m], &A.Q[2][m], &A.FL[0][m], &A.FL[1][m],
                     &A.FL[2][m]};
    for (double** p : fs)
      if (r == NS_OK) r = al(p, S.fb);
  }
  if (r == NS_OK) r = al(&A.PB, S.fb);
  if (r == NS_OK) r = al(&A.TL_DP, S.fb);
  if (r == NS_OK) r = al(&A.sc, kRfN * sizeof(double));
  if (r == NS_OK && cudaMallocHost(&A.sc_h, kRfN * sizeof(double)) != cudaSuccess)
    r = fail(c, NS_ERR_NOMEM, "cudaMallocHost (3D adjoint) failed");
  A.mixed = c->P.precision == NS_PREC_MIXED;
  for (int m = 0; m < 3 && r == NS_OK && A.mixed; ++m) {
    float** fs[] = {&A.US32[m], &A.PHB32[m], &A.Q32[0][m], &A.Q32[1][m], &A.Q32[2][m], &A.XF[m], &A.RF[m],
                    &A.RHF[m], &A.PF[m], &A.VF[m], &A.SF[m], &A.TF[m]};
    for (float** p : fs)
      if (r == NS_OK) r = al(reinterpret_cast<double**>(p), S.fb / 2);
  }
  if (r != NS_OK) free_adj3(c);
  return r;
}

A3Args a3(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  A3Args a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  a.c15 = c->g.c15;
  for (int m = 0; m < 3; ++m) {
    a.ix[m] = c->g.inv_dx[m];
    a.vc[m] = c->g.inv_dx2[m] * c->g.inv_ren;
    a.us[m] = A.US[m];
    a.phb[m] = A.PHB[m];
    a.dph[m] = A.DPH[m];
    a.ct[m] = A.CT[m];
    a.uadv[m] = A.UADV[m];
    for (int d = 0; d < 3; ++d) {
      a.q[d][m] = A.Q[d][m];
      a.fl[d][m] = A.FL[d][m];
    }
  }
  return a;
}

// FP32 operands: base in US32 / PHB32 / Q32, work arrays as float views of
// the FP64 ones (the FP64 and FP32 operators never run concurrently)
A3T<float> a3f(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  A3T<float> a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  a.c15 = (float)c->g.c15;
  for (int m = 0; m < 3; ++m) {
    a.ix[m] = (float)c->g.inv_dx[m];
    a.vc[m] = (float)(c->g.inv_dx2[m] * c->g.inv_ren);
    a.us[m] = A.US32[m];
    a.phb[m] = A.PHB32[m];
    a.dph[m] = reinterpret_cast<float*>(A.DPH[m]);
    a.ct[m] = reinterpret_cast<float*>(A.CT[m]);
    a.uadv[m] = reinterpret_cast<float*>(A.UADV[m]);
    for (int d = 0; d < 3; ++d) {
      a.q[d][m] = A.Q32[d][m];
      a.fl[d][m] = reinterpret_cast<float*>(A.FL[d][m]);
    }
  }
  return a;
}

#define L3(what, kernel, args)                                                                    \
  LAUNCH(NS_PROF_OTHER, what, (kernel<<<cells_grid(c->N), 256, 0, c->st>>> args, cudaGetLastError()))

// linearisation point: cell velocity and QUICK interpolants of u* (US)
int base3(ns_ctx* c) {
  const A3Args a = a3(c);
  L3("adjoint3 base cells", k3a_base_cells<double>, (a));
  L3("adjoint3 base q", k3a_base_q<double>, (a));
  if (c->s3->adj->mixed) {
    Adj3& A = *c->s3->adj;
    L3("adjoint3 base f32", k3r_to_f32, (c->g, A.US[0], A.US[1], A.US[2], A.US32[0], A.US32[1], A.US32[2]));
    const A3T<float> f = a3f(c);
    L3("adjoint3 base cells f32", k3a_base_cells<float>, (f));
    L3("adjoint3 base q f32", k3a_base_q<float>, (f));
  }
  return NS_OK;
}

template <typename T>
int apply_t(ns_ctx* c, int transpose, const A3T<T>& a) {
  if (!transpose) {
    L3("jvp3 cells", k3a_jv_cells<T>, (a));
    L3("jvp3 flux", k3a_jv_flux<T>, (a));
    L3("jvp3 total", k3a_jv_total<T>, (a));
    L3("jvp3 faces", k3a_jv_faces<T>, (a));
  } else {
    L3("vjp3 tbar", k3a_vj_tbar<T>, (a));
    L3("vjp3 flux", k3a_vj_flux<T>, (a));
    L3("vjp3 cells", k3a_vj_cells<T>, (a));
    L3("vjp3 faces", k3a_vj_faces<T>, (a));
  }
  return NS_OK;
}

// y = J x (transpose = 0) or J^T x
int apply3(ns_ctx* c, int transpose, double* const* x, double* const* y) {
  A3Args a = a3(c);
  for (int m = 0; m < 3; ++m) {
    a.v[m] = x[m];
    a.out[m] = y[m];
  }
  return apply_t(c, transpose, a);
}

// the same in FP32 on the FP32 base
int apply3f(ns_ctx* c, int transpose, float* const* x, float* const* y) {
  A3T<float> a = a3f(c);
  for (int m = 0; m < 3; ++m) {
    a.v[m] = x[m];
    a.out[m] = y[m];
  }
  return apply_t(c, transpose, a);
}

int scalars3(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  CK(cudaMemcpyAsync(A.sc_h, A.sc, kRfN * sizeof(double), cudaMemcpyDeviceToHost, c->st), "readback");
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

// BiCGStab for J x = BV (transpose = 0) or J^T x = BV from the guess in X
int bicg3(ns_ctx* c, int transpose, int* iters, double* res) {
  Adj3& A = *c->s3->adj;
  Bcg3 b;
  std::memset(&b, 0, sizeof(b));
  b.g = c->g;
  for (int m = 0; m < 3; ++m) {
    b.x[m] = A.X[m]; b.r[m] = A.R[m]; b.rh[m] = A.RH[m]; b.p[m] = A.PV[m];
    b.v[m] = A.V[m]; b.s[m] = A.SV[m]; b.t[m] = A.T[m]; b.b[m] = A.BV[m];
  }
  b.sc = A.sc;
  b.part = c->s3->part;
  b.counter = c->counter;
  auto start = [&]() -> int {
    int r = apply3(c, transpose, A.X, A.V);
    if (r != NS_OK) return r;
    L3("bicgstab3 init", k3b_init, (b));
    return scalars3(c);
  };
  int r = start();
  if (r != NS_OK) return r;
  const double bb = A.sc_h[kBcBB];
  *iters = 0;
  if (!(bb > 0.0)) {
    for (int m = 0; m < 3; ++m) CK(cudaMemsetAsync(A.X[m], 0, c->s3->fb, c->st), "memset");
    *res = 0.0;
    return NS_OK;
  }
  double rel = std::sqrt(A.sc_h[kBcRR] / bb);
  int it = 0, restarts = 0;
  const double tol = A.opts.lin_tol;
  while (rel > tol && it < A.opts.lin_max_iters) {
    r = apply3(c, transpose, A.PV, A.V);
    if (r != NS_OK) return r;
    L3("bicgstab3 alpha", k3b_alpha, (b));
    L3("bicgstab3 s", k3b_s, (b));
    r = apply3(c, transpose, A.SV, A.T);
    if (r != NS_OK) return r;
    L3("bicgstab3 omega", k3b_omega, (b));
    L3("bicgstab3 x r", k3b_xr, (b));
    L3("bicgstab3 p", k3b_p, (b));
    ++it;
    r = scalars3(c);
    if (r != NS_OK) return r;
    rel = std::sqrt(A.sc_h[kBcRR] / bb);
    if (!std::isfinite(rel)) return fail(c, NS_ERR_CUDA, "BiCGStab: non-finite residual");
    if (A.sc_h[kBcBreak] != 0.0 && rel > tol) {
      if (++restarts > 8) break;
      r = start();
      if (r != NS_OK) return r;
      rel = std::sqrt(A.sc_h[kBcRR] / bb);
    }
  }
  *iters = it;
  *res = rel;
  A.st.lin_iters += it;
  A.st.lin_max_iters_seen = std::max(A.st.lin_max_iters_seen, it);
  A.st.lin_max_res = std::max(A.st.lin_max_res, rel);
  return NS_OK;
}

// inner FP32 BiCGStab of the refinement: op(J) XF = RF from XF = 0 until the
// residual falls by rel_tol, a breakdown, or max_it iterations
int bicg3f(ns_ctx* c, int transpose, double rel_tol, int max_it, int* iters) {
  Adj3& A = *c->s3->adj;
  Bcg3f b;
  std::memset(&b, 0, sizeof(b));
  b.g = c->g;
  for (int m = 0; m < 3; ++m) {
    b.x[m] = A.XF[m]; b.r[m] = A.RF[m]; b.rh[m] = A.RHF[m]; b.p[m] = A.PF[m];
    b.v[m] = A.VF[m]; b.s[m] = A.SF[m]; b.t[m] = A.TF[m]; b.b[m] = A.RF[m];  // r starts as b, in place
  }
  b.sc = A.sc;
  b.part = c->s3->part;
  b.counter = c->counter;
  L3("bicgstab3 f32 init", k3c_init, (b));
  int r = scalars3(c);
  if (r != NS_OK) return r;
  const double rr0 = A.sc_h[kBcRR];
  int it = 0;
  double rel = rr0 > 0.0 ? 1.0 : 0.0;
  while (rel > rel_tol && it < max_it) {
    r = apply3f(c, transpose, A.PF, A.VF);
    if (r != NS_OK) return r;
    L3("bicgstab3 f32 alpha", k3c_alpha, (b));
    L3("bicgstab3 f32 s", k3c_s, (b));
    r = apply3f(c, transpose, A.SF, A.TF);
    if (r != NS_OK) return r;
    L3("bicgstab3 f32 omega", k3c_omega, (b));
    L3("bicgstab3 f32 x r", k3c_xr, (b));
    L3("bicgstab3 f32 p", k3c_p, (b));
    ++it;
    r = scalars3(c);
    if (r != NS_OK) return r;
    rel = std::sqrt(A.sc_h[kBcRR] / rr0);
    if (!std::isfinite(rel)) return fail(c, NS_ERR_CUDA, "BiCGStab (FP32): non-finite residual");
    if (A.sc_h[kBcBreak] != 0.0) break;
  }
  *iters = it;
  return NS_OK;
}

constexpr double kInnerTol = 1e-5;  // residual reduction of one inner FP32 solve
constexpr int kMaxRefine = 8;

// op(J) X = BV from the guess in X: FP64 BiCGStab, or (mixed precision) FP64
// residuals refined by inner FP32 solves; the relative residual of the
// refinement is max |r| / max |b|
int solve3(ns_ctx* c, int transpose, int* iters, double* res) {
  Adj3& A = *c->s3->adj;
  if (!A.mixed) return bicg3(c, transpose, iters, res);
  Ref3 f;
  std::memset(&f, 0, sizeof(f));
  f.g = c->g;
  for (int m = 0; m < 3; ++m) {
    f.b[m] = A.BV[m]; f.v[m] = A.V[m]; f.r32[m] = A.RF[m]; f.x[m] = A.X[m]; f.d[m] = A.XF[m];
  }
  f.sc = A.sc;
  f.part = c->s3->part;
  f.counter = c->counter;
  const double tol = A.opts.lin_tol;
  int inner = 0;
  double rel = 0.0;
  for (int outer = 0;; ++outer) {
    int r = apply3(c, transpose, A.X, A.V);
    if (r != NS_OK) return r;
    L3("refine residual max", k3r_resmax, (f));
    r = scalars3(c);
    if (r != NS_OK) return r;
    const double rmax = A.sc_h[kRfRR], bmax = A.sc_h[kRfBB];
    if (!(bmax > 0.0)) {
      for (int m = 0; m < 3; ++m) CK(cudaMemsetAsync(A.X[m], 0, c->s3->fb, c->st), "memset");
      rel = 0.0;
      break;
    }
    rel = rmax / bmax;
    if (!std::isfinite(rel)) return fail(c, NS_ERR_CUDA, "refinement: non-finite residual");
    if (rel <= tol || outer >= kMaxRefine || inner >= A.opts.lin_max_iters) break;
    L3("refine residual f32", k3r_scaled, (f, 1.0 / rmax));
    int it = 0;
    r = bicg3f(c, transpose, kInnerTol, A.opts.lin_max_iters, &it);
    if (r != NS_OK) return r;
    inner += it;
    L3("refine update", k3r_update, (f, rmax));
  }
  *iters = inner;
  *res = rel;
  A.st.lin_iters += inner;
  A.st.lin_max_iters_seen = std::max(A.st.lin_max_iters_seen, inner);
  A.st.lin_max_res = std::max(A.st.lin_max_res, rel);
  return NS_OK;
}

// F = D u + coef pb (sum into red[kRedSum]); psi = L^-1 P0 F in PHI
int poisson_adj3(ns_ctx* c, double* const* u, const double* pb, double coef, const double** psi) {
  State3D& S = *c->s3;
  L3("adjoint3 div", k3a_div, (c->g, u[0], u[1], u[2], pb, coef, S.F, S.part, c->counter, c->red + kRedSum, nullptr));
  const double keep = c->P.poisson_tol_div;
  c->P.poisson_tol_div = 0.0;
  int cyc = 0;
  double res = 0.0;
  const int r = poisson3d(c, &cyc, &res);
  c->P.poisson_tol_div = keep;
  S.adj->st.poisson_cycles += cyc;
  if (r != NS_OK && !(r == NS_ERR_MG_STALL && res < 1e-9)) return r;
  *psi = S.PHI;
  return NS_OK;
}

// u* of the current state (not advanced) into US
int ustar3(ns_ctx* c) {
  State3D& S = *c->s3;
  ns_step_stats s;
  std::memset(&s, 0, sizeof(s));
  int r = predictor3d(c, &s);
  if (r != NS_OK) return r;
  for (int m = 0; m < 3; ++m)
    CK(cudaMemcpyAsync(S.adj->US[m], face3_ptr(c, S.cur, m), S.fb, cudaMemcpyDeviceToDevice, c->st), "copy u*");
  for (int m = 0; m < 3; ++m) std::swap(S.U[m], S.UP[m]);
  c->time -= c->dt;
  S.adj->st.predictor_runs++;
  if (s.status != NS_OK) S.adj->st.status = s.status;
  return NS_OK;
}

// adjoint of one step at u* = US: (UB, UPB, PB) of level k+1 -> level k
int adj_step3(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  const Geom& g = c->g;
  const double* psi = nullptr;
  int r = poisson_adj3(c, A.UB, A.PB, g.c15, &psi);
  if (r != NS_OK) return r;
  A3Args ga = a3(c);
  for (int m = 0; m < 3; ++m) {
    ga.v[m] = A.UB[m];
    ga.out[m] = A.AUS[m];
  }
  L3("adjoint3 gradsub", k3a_gradsub, (ga, psi, 1.0));
  L3("adjoint3 rhs", k3a_lincomb, (g, -1.0, A.AUS[0], A.AUS[1], A.AUS[2], 0.0, nullptr, nullptr, nullptr, A.BV[0], A.BV[1], A.BV[2]));
  r = base3(c);
  if (r != NS_OK) return r;
  int it = 0;
  double res = 0.0;
  r = solve3(c, 1, &it, &res);
  if (r != NS_OK) return r;
  L3("adjoint3 ubar", k3a_lincomb, (g, 1.0, A.UPB[0], A.UPB[1], A.UPB[2], g.c15 + g.c05, A.X[0], A.X[1], A.X[2], A.UB[0], A.UB[1], A.UB[2]));
  L3("adjoint3 uprevbar", k3a_lincomb, (g, -g.c05, A.X[0], A.X[1], A.X[2], 0.0, nullptr, nullptr, nullptr, A.UPB[0], A.UPB[1], A.UPB[2]));
  L3("adjoint3 pbar", k3a_div, (g, A.X[0], A.X[1], A.X[2], A.PB, 1.0, A.PB, c->s3->part, c->counter, c->red + kRedScratch, nullptr));
  A.st.adjoint_steps++;
  return NS_OK;
}

// tangent of one step at u* = US: (TL_DU, TL_DUP, TL_DP) -> (OUT = du', TL_DP = dp')
int tan_step3(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  const Geom& g = c->g;
  int r = base3(c);
  if (r != NS_OK) return r;
  A3Args ta = a3(c);
  for (int m = 0; m < 3; ++m) {
    ta.v[m] = A.TL_DU[m];
    ta.out[m] = A.BV[m];
  }
  L3("tangent3 rhs", k3a_tlm_rhs, (ta, A.TL_DP, A.TL_DUP[0], A.TL_DUP[1], A.TL_DUP[2]));
  int it = 0;
  double res = 0.0;
  r = solve3(c, 0, &it, &res);
  if (r != NS_OK) return r;
  const double* psi = nullptr;
  r = poisson_adj3(c, A.X, nullptr, 0.0, &psi);
  if (r != NS_OK) return r;
  A3Args ga = a3(c);
  for (int m = 0; m < 3; ++m) {
    ga.v[m] = A.X[m];
    ga.out[m] = A.OUT[m];
  }
  L3("tangent3 gradsub", k3a_gradsub, (ga, psi, 1.0));
  L3("tangent3 p", k3a_cells, (g, 1.0, A.TL_DP, g.c15, psi, A.TL_DP));
  return NS_OK;
}

}  // namespace

namespace {

// ---- snapshots: slot k holds U[3], UP[3], p of a level and u*[3] of the step that produced it
double* slot3(ns_ctx* c, int slot, int f) {
  const size_t words = c->s3->fb / sizeof(double);
  return c->s3->adj->snap + ((size_t)slot * kSlot3 + f) * words;
}

int store3(ns_ctx* c, int slot, int step, bool with_ustar) {
  State3D& S = *c->s3;
  Adj3& A = *S.adj;
  double* src[7] = {S.U[0], S.U[1], S.U[2], S.UP[0], S.UP[1], S.UP[2], S.Pp};
  for (int f = 0; f < 7; ++f)
    CK(cudaMemcpyAsync(slot3(c, slot, f), src[f], S.fb, cudaMemcpyDeviceToDevice, c->st), "snapshot store");
  if (with_ustar)
    for (int m = 0; m < 3; ++m)
      CK(cudaMemcpyAsync(slot3(c, slot, 7 + m), face3_ptr(c, S.cur, m), S.fb, cudaMemcpyDeviceToDevice, c->st), "snapshot u*");
  A.slot_step[slot] = step;
  A.slot_time[slot] = c->time;
  return NS_OK;
}

int restore3(ns_ctx* c, int slot) {
  State3D& S = *c->s3;
  Adj3& A = *S.adj;
  double* dst[7] = {S.U[0], S.U[1], S.U[2], S.UP[0], S.UP[1], S.UP[2], S.Pp};
  for (int f = 0; f < 7; ++f)
    CK(cudaMemcpyAsync(dst[f], slot3(c, slot, f), S.fb, cudaMemcpyDeviceToDevice, c->st), "snapshot restore");
  c->time = A.slot_time[slot];
  c->step = A.step0 + A.slot_step[slot];
  c->in_step = false;
  return NS_OK;
}

int advance3(ns_ctx* c, int n) {
  for (int k = 0; k < n; ++k) {
    ns_step_stats s;
    const int r = step3d(c, &s);
    if (r < 0) return r;
    if (r != NS_OK) c->s3->adj->st.status = r;
    c->s3->adj->st.steps_advanced++;
  }
  return NS_OK;
}

int find3(ns_ctx* c, int step) {
  Adj3& A = *c->s3->adj;
  for (int k = 0; k < A.nslots; ++k)
    if (k != A.final_slot && A.slot_step[k] == step) return k;
  return -1;
}

int free3(ns_ctx* c) {
  Adj3& A = *c->s3->adj;
  for (int k = 0; k < A.nslots; ++k)
    if (k != A.final_slot && A.slot_step[k] < 0) return k;
  return -1;
}

int adjoint_with3(ns_ctx* c, double* const* src) {
  State3D& S = *c->s3;
  for (int m = 0; m < 3; ++m)
    CK(cudaMemcpyAsync(S.adj->US[m], src[m], S.fb, cudaMemcpyDeviceToDevice, c->st), "copy u*");
  return adj_step3(c);
}

// reverse the steps [a, b): level a in slot_a, s slots free, ul = u* of step b-1
int reverse3(ns_ctx* c, int a, int b, int s, int slot_a, double* const* ul) {
  Adj3& A = *c->s3->adj;
  if (b - a <= 0) return NS_OK;
  if (b - a == 1) return adjoint_with3(c, ul);
  const int m = A.sched.next(a, b, s);
  if (m < 0) {
    int r = adjoint_with3(c, ul);
    for (int k = b - 2; k >= a && r == NS_OK; --k) {
      r = restore3(c, slot_a);
      if (r == NS_OK) r = advance3(c, k - a);
      if (r == NS_OK) r = ustar3(c);
      if (r == NS_OK) r = adj_step3(c);
    }
    return r;
  }
  int slot_m = find3(c, m);
  if (slot_m < 0) {
    slot_m = free3(c);
    if (slot_m < 0) return fail(c, NS_ERR_STATE, "checkpoint schedule: no free snapshot slot");
    int r = restore3(c, slot_a);
    if (r == NS_OK) r = advance3(c, m - a);
    if (r == NS_OK) r = store3(c, slot_m, m, true);
    if (r != NS_OK) return r;
  }
  int r = reverse3(c, m, b, s - 1, slot_m, ul);
  if (r != NS_OK) return r;
  for (int q = 0; q < 3; ++q)
    CK(cudaMemcpyAsync(A.ORPH[q], slot3(c, slot_m, 7 + q), c->s3->fb, cudaMemcpyDeviceToDevice, c->st), "keep u*");
  A.slot_step[slot_m] = -1;
  return reverse3(c, a, m, s, slot_a, A.ORPH);
}

double now3() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// objective of the current U: enstrophy into red[kRedObj], dE/du into UB
int objective3(ns_ctx* c) {
  State3D& S = *c->s3;
  Adj3& A = *S.adj;
  A3Args a = a3(c);
  for (int m = 0; m < 3; ++m) {
    a.v[m] = S.U[m];
    a.out[m] = A.OM[m];
  }
  L3("vorticity", k3a_vort, (a));
  L3("enstrophy", k3a_enstrophy, (c->g, A.OM[0], A.OM[1], A.OM[2], S.part, c->counter, c->red + kRedObj));
  A3Args b = a3(c);
  for (int m = 0; m < 3; ++m) {
    b.v[m] = A.OM[m];
    b.out[m] = A.UB[m];
  }
  L3("enstrophy gradient", k3a_enstrophy_grad, (b));
  return NS_OK;
}

}  // namespace

namespace nsh {

int adjoint_fwd3(ns_ctx* c, const ns_adjoint_opts* opts, double* J, ns_adjoint_stats* stats) {
  int r = need3(c);
  if (r == NS_OK) r = ensure3(c);
  if (r != NS_OK) return r;
  // the adjoint differentiates the step with cont2cart's cell velocity (its
  // replays from the snapshots use it too): an analytic first-stage override
  // from ns_init_fields is not applied
  c->cart_pending = false;
  State3D& S = *c->s3;
  Adj3& A = *S.adj;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  const double t0 = now3();
  A.opts = *opts;
  std::memset(&A.st, 0, sizeof(A.st));
  A.have_fwd = false;
  A.nsteps = opts->nsteps;
  A.nsnap = opts->nsnap;
  A.step0 = c->step;
  const int nsched = std::min(opts->nsnap, opts->nsteps);
  const int nslots = nsched + 1;
  if (A.nslots != nslots) {
    if (A.snap) cudaFree(A.snap);
    A.snap = nullptr;
    A.nslots = 0;
    if (cudaMalloc(&A.snap, (size_t)nslots * kSlot3 * S.fb) != cudaSuccess)
      return fail(c, NS_ERR_NOMEM, "cudaMalloc (3D snapshots) failed");
    A.nslots = nslots;
  }
  A.slot_step.assign(nslots, -1);
  A.slot_time.assign(nslots, 0.0);
  A.final_slot = nslots - 1;
  A.sched.build(opts->nsteps, nsched - 1);
  std::vector<int> first;
  for (int a = 0, s = nsched - 1;;) {
    const int m = A.sched.next(a, opts->nsteps, s);
    if (m < 0) break;
    first.push_back(m);
    a = m;
    --s;
  }
  r = store3(c, 0, 0, false);
  if (r != NS_OK) return r;
  size_t next = 0;
  for (int k = 0; k < opts->nsteps; ++k) {
    if (next < first.size() && first[next] == k) {
      const int slot = free3(c);
      if (slot < 0) return fail(c, NS_ERR_STATE, "checkpoint schedule: no free snapshot slot");
      r = store3(c, slot, k, true);
      if (r != NS_OK) return r;
      ++next;
    }
    r = advance3(c, 1);
    if (r != NS_OK) return r;
  }
  r = store3(c, A.final_slot, opts->nsteps, true);
  if (r == NS_OK) r = objective3(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 3; ++m) {
    CK(cudaMemsetAsync(A.UPB[m], 0, S.fb, c->st), "memset");
    CK(cudaMemsetAsync(A.X[m], 0, S.fb, c->st), "memset");
  }
  CK(cudaMemsetAsync(A.PB, 0, S.fb, c->st), "memset");
  r = sync_red(c, kRedObj, 1);
  if (r != NS_OK) return r;
  A.st.J = c->red_h[kRedObj];
  A.st.nsteps = opts->nsteps;
  A.st.nsnap = nsched;
  A.st.ms_forward = now3() - t0;
  A.have_fwd = true;
  if (J) *J = A.st.J;
  if (stats) *stats = A.st;
  return A.st.status < 0 ? A.st.status : NS_OK;
}

int adjoint_bwd3(ns_ctx* c, ns_adjoint_stats* stats) {
  if (!c->s3->adj || !c->s3->adj->have_fwd) return fail(c, NS_ERR_STATE, "ns_step_adjoint_bwd needs ns_step_adjoint_fwd first");
  Adj3& A = *c->s3->adj;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  const double t0 = now3();
  const int nsched = std::min(A.nsnap, A.nsteps);
  double* ul[3] = {slot3(c, A.final_slot, 7), slot3(c, A.final_slot, 8), slot3(c, A.final_slot, 9)};
  int r = reverse3(c, 0, A.nsteps, nsched - 1, 0, ul);
  if (r == NS_OK) r = restore3(c, A.final_slot);
  if (r != NS_OK) return r;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  A.have_fwd = false;
  A.st.ms_backward = now3() - t0;
  if (stats) *stats = A.st;
  return A.st.status < 0 ? A.st.status : NS_OK;
}

int adjoint_state_grad3(ns_ctx* c, double* const* ubar, double* const* uprevbar, double* pbar) {
  if (!c->s3->adj) return NS_ERR_ARG;
  Adj3& A = *c->s3->adj;
  for (int m = 0; m < 3; ++m) {
    if (ubar && ubar[m]) { int r = copy_faces3(c, m, ubar[m], A.UB[m], false); if (r) return r; }
    if (uprevbar && uprevbar[m]) { int r = copy_faces3(c, m, uprevbar[m], A.UPB[m], false); if (r) return r; }
  }
  if (pbar) { int r = copy_cells3(c, pbar, A.PB, false); if (r) return r; }
  return ns_sync(c);
}

// the face-N images carry no degree of freedom: inputs there are ignored
// (zeroed), outputs there are 0
static int put_dofs3(ns_ctx* c, const double* const* h, double* const* d) {
  for (int m = 0; m < 3; ++m) {
    int r = copy_faces3(c, m, h[m], d[m], true);
    if (r != NS_OK) return r;
  }
  const Geom& g = c->g;
  L3("dofs", k3a_lincomb, (g, 1.0, d[0], d[1], d[2], 0.0, nullptr, nullptr, nullptr, c->s3->adj->OUT[0], c->s3->adj->OUT[1], c->s3->adj->OUT[2]));
  for (int m = 0; m < 3; ++m) {
    CK(cudaMemsetAsync(d[m], 0, c->s3->fb, c->st), "memset");
    CK(cudaMemcpyAsync(d[m], c->s3->adj->OUT[m], c->s3->fb, cudaMemcpyDeviceToDevice, c->st), "copy");
  }
  return NS_OK;
}

static int prepare3(ns_ctx* c) {
  int r = need3(c);
  if (r == NS_OK) r = ensure3(c);
  if (r != NS_OK) return r;
  c->cart_pending = false;  // as in adjoint_fwd3
  Adj3& A = *c->s3->adj;
  if (A.opts.lin_max_iters == 0) ns_adjoint_opts_default(&A.opts);
  A.have_fwd = false;
  for (int m = 0; m < 3; ++m) {
    CK(cudaMemsetAsync(A.OUT[m], 0, c->s3->fb, c->st), "memset");
    CK(cudaMemsetAsync(A.X[m], 0, c->s3->fb, c->st), "memset");
  }
  return NS_OK;
}

int step_jvp3(ns_ctx* c, const double* const* du, const double* const* duprev, const double* dp, double* const* du_out,
              double* const* duprev_out, double* dp_out) {
  int r = prepare3(c);
  if (r != NS_OK) return r;
  Adj3& A = *c->s3->adj;
  r = put_dofs3(c, du, A.TL_DU);
  if (r == NS_OK) r = put_dofs3(c, duprev, A.TL_DUP);
  if (r == NS_OK) r = copy_cells3(c, dp, A.TL_DP, true);
  if (r == NS_OK) r = ustar3(c);
  if (r == NS_OK) r = tan_step3(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 3; ++m) {
    if (du_out && du_out[m]) { r = copy_faces3(c, m, du_out[m], A.OUT[m], false); if (r) return r; }
    if (duprev_out && duprev_out[m]) { r = copy_faces3(c, m, duprev_out[m], A.TL_DU[m], false); if (r) return r; }
  }
  if (dp_out) { r = copy_cells3(c, dp_out, A.TL_DP, false); if (r) return r; }
  return ns_sync(c);
}

int step_vjp3(ns_ctx* c, const double* const* ubar_out, const double* const* uprevbar_out, const double* pbar_out,
              double* const* ubar, double* const* uprevbar, double* pbar) {
  int r = prepare3(c);
  if (r != NS_OK) return r;
  Adj3& A = *c->s3->adj;
  r = put_dofs3(c, ubar_out, A.UB);
  if (r == NS_OK) r = put_dofs3(c, uprevbar_out, A.UPB);
  if (r == NS_OK) r = copy_cells3(c, pbar_out, A.PB, true);
  if (r == NS_OK) r = ustar3(c);
  if (r == NS_OK) r = adj_step3(c);
  if (r != NS_OK) return r;
  for (int m = 0; m < 3; ++m) {
    if (ubar && ubar[m]) { r = copy_faces3(c, m, ubar[m], A.UB[m], false); if (r) return r; }
    if (uprevbar && uprevbar[m]) { r = copy_faces3(c, m, uprevbar[m], A.UPB[m], false); if (r) return r; }
  }
  if (pbar) { r = copy_cells3(c, pbar, A.PB, false); if (r) return r; }
  return ns_sync(c);
}

int adjoint_op3(ns_ctx* c, int transpose, const double* const* x, double* const* y) {
  int r = prepare3(c);
  if (r != NS_OK) return r;
  Adj3& A = *c->s3->adj;
  r = put_dofs3(c, x, A.TL_DU);
  if (r == NS_OK) r = ustar3(c);
  if (r == NS_OK) r = base3(c);
  if (r == NS_OK) r = apply3(c, transpose, A.TL_DU, A.OUT);
  if (r != NS_OK) return r;
  for (int m = 0; m < 3; ++m) {
    r = copy_faces3(c, m, y[m], A.OUT[m], false);
    if (r != NS_OK) return r;
  }
  return ns_sync(c);
}

}  // namespace nsh
