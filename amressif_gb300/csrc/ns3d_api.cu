// Host driver of the 3D advance (dim = 3): the time loop of main_main
// (main.cpp:875-1180) over the kernels of ns3d.cuh (FP64 predictor) and
// ns3d_mixed.cuh (mixed-precision predictor). The 3D context supports the
// whole-step API (ns_step, ns_set_state / ns_get_state, checkpoints), the
// per-call-site building blocks (step begin, FP64 RK stage, pseudo-norm,
// explicit predictor, Poisson right-hand side and solve, projection), the box
// transfers and the adjoint (adjoint3d_api.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "launch3d.h"
#include "state3d.h"

using namespace ns;
using namespace nsh;

namespace nsh {

void free3d(ns_ctx* c) {
  if (!c->s3) return;
  free_adj3(c);
  for (auto& G : c->s3->vg3)
    if (G.exec) cudaGraphExecDestroy(G.exec);
  for (void* p : c->s3->allocs) cudaFree(p);
  delete c->s3;
  c->s3 = nullptr;
}

}  // namespace nsh

namespace {

long rup(long x, long a) { return (x + a - 1) / a * a; }

template <typename P>
int alloc3(ns_ctx* c, P** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc (3D) failed");
  c->s3->allocs.push_back(*p);
  CK(cudaMemsetAsync(*p, 0, bytes, c->st), "memset");
  return NS_OK;
}

template <typename T>
int levels3(ns_ctx* c, MG3<T>& M, bool own0) {
  State3D& S = *c->s3;
  int n = c->N;
  M.L = 0;
  for (int d = 0; d < 3; ++d) M.periodic[d] = c->g.periodic[d];
  M.fmean = nullptr;
  double h[3] = {c->g.dx[0], c->g.dx[1], c->g.dx[2]};
  while (true) {
    const int l = M.L;
    if (l >= kMaxLevels3) return fail(c, NS_ERR_ARG, "too many multigrid levels");
    M.n[l] = n;
    M.pitch[l] = (l == 0) ? c->pitch : rup(n, 32);
    M.plane[l] = (l == 0) ? c->pitch * (c->N + 1) : M.pitch[l] * n;
    for (int d = 0; d < 3; ++d) M.ih[l][d] = (T)(1.0 / (h[d] * h[d]));
    M.x[l] = nullptr;
    M.f[l] = nullptr;
    if (l > 0 || own0) {
      const size_t bytes = (l == 0) ? S.fb / sizeof(double) * sizeof(T) : (size_t)M.plane[l] * n * sizeof(T);
      int r = alloc3(c, &M.x[l], bytes);
      if (r == NS_OK) r = alloc3(c, &M.f[l], bytes);
      if (r != NS_OK) return r;
    }
    M.L++;
    if (!(n % 4 == 0 && n > 4)) break;
    n /= 2;
    for (double& x : h) x *= 2;
  }
  return NS_OK;
}

Arg3 args(ns_ctx* c) {
  State3D& S = *c->s3;
  Arg3 a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  for (int m = 0; m < 3; ++m) {
    a.ph[m] = S.PH[m];
    a.t[m] = S.T[m];
    for (int d = 0; d < 3; ++d) a.fl[d][m] = S.FL[d][m];
  }
  a.part = S.part;
  a.counter = c->counter;
  return a;
}

double* face3(ns_ctx* c, int id, int m) { return id < 0 ? c->s3->UP[m] : c->s3->B[id][m]; }

int pick3(int base, int in) {
  for (int i = 0; i < 3; ++i)
    if (i != base && i != in) return i;
  return -2;
}

// the first level from which the V-cycle runs in the persistent coarse block
// (n <= kBottom3N down to the coarsest); M.L when the coarsest level is larger
template <typename T>
int coarse_level3(const MG3<T>& M) {
  int lb = 0;
  while (lb < M.L && M.n[lb] > kBottom3N) ++lb;
  return lb;
}

template <typename T>
int vcycle3(ns_ctx* c, MG3<T>& M) {
  const int lb = coarse_level3(M);
  if (lb < M.L) {
    // levels above lb as launches, lb and below in one block
    for (int l = 0; l < lb; ++l) {
      for (int s = 0; s < 4; ++s) LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg3 smooth", launch3_mg_rb<T>(M, l, s & 1, c->st));
      LAUNCH(l == 0 ? NS_PROF_MG_RESTRICT0 : NS_PROF_MG_RESTRICT, "mg3 restrict", launch3_mg_restrict<T>(M, l, c->st));
    }
    LAUNCH(NS_PROF_MG_BOTTOM, "mg3 coarse levels", launch3_mg_coarse<T>(M, lb, c->st));
    for (int l = lb - 1; l >= 0; --l) {
      LAUNCH(NS_PROF_MG_SMOOTH, "mg3 prolong", launch3_mg_prolong<T>(M, l, c->st));
      for (int s = 0; s < 4; ++s) LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg3 smooth", launch3_mg_rb<T>(M, l, (s + 1) & 1, c->st));
    }
    return NS_OK;
  }
  for (int l = 0; l + 1 < M.L; ++l) {
    for (int s = 0; s < 4; ++s) LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg3 smooth", launch3_mg_rb<T>(M, l, s & 1, c->st));
    LAUNCH(l == 0 ? NS_PROF_MG_RESTRICT0 : NS_PROF_MG_RESTRICT, "mg3 restrict", launch3_mg_restrict<T>(M, l, c->st));
  }
  LAUNCH(NS_PROF_MG_BOTTOM, "mg3 bottom", launch3_mg_bottom<T>(M, M.L - 1, 50, c->st));
  for (int l = M.L - 2; l >= 0; --l) {
    LAUNCH(NS_PROF_MG_SMOOTH, "mg3 prolong", launch3_mg_prolong<T>(M, l, c->st));
    for (int s = 0; s < 4; ++s) LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg3 smooth", launch3_mg_rb<T>(M, l, (s + 1) & 1, c->st));
  }
  return NS_OK;
}

// one V-cycle (FP32: preceded by zeroing the correction) replayed from a CUDA
// graph captured on first use; plain launches if the stream cannot be captured
template <typename T>
int vcycle3_graph(ns_ctx* c, MG3<T>& M) {
  State3D& S = *c->s3;
  ns_ctx::VGraph& G = S.vg3[sizeof(T) == 8 ? 1 : 0];
  auto body = [&]() -> int {
    if (sizeof(T) == 4) CK(cudaMemsetAsync(M.x[0], 0, S.fb / 2, c->st), "memset e");  // each correction starts from zero
    return vcycle3<T>(c, M);
  };
  if (G.unusable) return body();
  const void* key[4] = {M.x[0], M.f[0], M.fmean, nullptr};
  if (G.exec && std::memcmp(key, G.key, sizeof(key)) != 0) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  if (!G.exec) {
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      G.unusable = true;
      return body();
    }
    const long long l0 = c->launches;
    const bool prof = c->prof;
    c->prof = false;
    const int r = body();
    c->prof = prof;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->st, &g);
    if (r != NS_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    CK(e, "V-cycle capture");
    const cudaError_t ei = cudaGraphInstantiate(&G.exec, g, 0);
    cudaGraphDestroy(g);
    CK(ei, "V-cycle graph instantiate");
    G.nlaunch = c->launches - l0;
    c->launches = l0;
    std::memcpy(G.key, key, sizeof(key));
  }
  LAUNCH(NS_PROF_MG_CYCLE, "V-cycle graph", cudaGraphLaunch(G.exec, c->st));
  c->launches += G.nlaunch - 1;
  return NS_OK;
}

__global__ void k3_set_mean(double* red, double inv_n) { red[kRedMean] = red[kRedSum] * inv_n; }

// phi solves L phi = f - mean(f) to poisson_tol_rel (and the divergence
// tolerance); FP64 V-cycles, or FP32 V-cycles inside an FP64 defect correction
int poisson3(ns_ctx* c, bool mixed, int* cycles, double* res, long long* fallbacks) {
  State3D& S = *c->s3;
  const double n3 = (double)c->N * c->N * c->N;
  LAUNCH(NS_PROF_OTHER, "set mean", (k3_set_mean<<<1, 1, 0, c->st>>>(c->red, 1.0 / n3), cudaGetLastError()));
  S.M64.x[0] = S.PHI;
  S.M64.f[0] = S.F;
  S.M64.fmean = c->red + kRedMean;
  CK(cudaMemsetAsync(S.PHI, 0, S.fb, c->st), "memset phi");
  const int maxc = std::max(1, c->P.poisson_max_cycles);
  const double div_tol_res = c->P.poisson_tol_div > 0 ? c->P.poisson_tol_div * 1.5 / c->dt : 0.0;
  if (c->P.poisson_solver == 1) {
    // restarted GMRES with one FP64 V-cycle as right preconditioner
    // (GMRES_Poisson.cpp:56-131), in every precision mode as in 2D
    double g0 = 0.0, gn = 0.0;
    int its = 0;
    const int st = poisson_gmres(c, c->P.poisson_tol_rel, div_tol_res, maxc, &its, &g0, &gn);
    if (st != NS_OK && st != NS_ERR_MG_STALL) return st;
    *cycles = its;
    *res = g0 > 0 ? gn / g0 : 0.0;
    if (st != NS_OK) c->err = "GMRES residual did not reach the tolerance";
    return st;
  }
  // mixed: phi as float-float pairs in PHF[pf]; each sweep adds the FP32
  // correction and recomputes the residual (k3_dcff), phi goes to FP64 at the
  // end. dc_residual = 1: phi and the residual in FP64 from the first sweep
  // (k3_dc64), phi in P64[pf]
  DCff3 dc;
  std::memset(&dc, 0, sizeof(dc));
  int pf = 0;
  const bool dc64 = mixed && c->P.dc_residual == 1;
  double* P64[2] = {S.PHI, S.PHI2};
  if (mixed) {
    dc.n = c->N;
    dc.pitch = c->pitch;
    dc.plane = (long)c->pitch * (c->N + 1);
    for (int d = 0; d < 3; ++d) {
      dc.periodic[d] = c->g.periodic[d];
      dc.ih[d][0] = (float)(1.0 / (c->g.dx[d] * c->g.dx[d]));
      dc.ih[d][1] = (float)(1.0 / (c->g.dx[d] * c->g.dx[d]) - (double)dc.ih[d][0]);
    }
    dc.r32 = S.M32.f[0];
    dc.f = S.FF;
    dc.part = S.part;
    dc.counter = c->counter;
    dc.red_out = c->red + kRedRes;
    if (dc64) {
      dc.f64 = S.F;
      dc.fmean = c->red + kRedMean;
      for (int d = 0; d < 3; ++d) dc.ih64[d] = S.M64.ih[0][d];
    } else {
      LAUNCH(NS_PROF_DC_UPDATE, "f - mean (ff)", launch3_rhs_ff(c->N, dc.pitch, dc.plane, S.F, c->red + kRedMean, S.FF, c->st));
    }
  }
  auto residual = [&](bool first) -> int {
    if (mixed) {
      dc.first = first;
      dc.phin = S.PHF[pf];
      dc.phout = S.PHF[first ? pf : 1 - pf];
      dc.phin64 = P64[pf];
      dc.phout64 = P64[first ? pf : 1 - pf];
      dc.e = first ? nullptr : S.M32.x[0];
      LAUNCH(NS_PROF_DC_UPDATE, "dc update", dc64 ? launch3_dc64(dc, c->st) : launch3_dcff(dc, c->st));
      if (!first) pf = 1 - pf;
    } else {
      LAUNCH(NS_PROF_MG_RESNORM, "resnorm", launch3_mg_resnorm<double>(S.M64, S.part, c->counter, c->red + kRedRes, c->st));
    }
    return sync_red(c, kRedRes, 1);
  };
  int r = residual(true);
  if (r != NS_OK) return r;
  const double r0 = c->red_h[kRedRes];
  double rn = r0, best = r0;
  const double tol = c->P.poisson_tol_rel * r0;
  auto done = [&](double x) { return x <= tol && (div_tol_res <= 0 || x <= div_tol_res); };
  int ncyc = 0, stall = 0, status = NS_OK;
  while (!done(rn) && r0 > 0) {
    if (ncyc >= maxc) { status = NS_ERR_MG_STALL; break; }
    if (mixed) {
      r = vcycle3_graph<float>(c, S.M32);  // zeroes the correction first
    } else {
      r = vcycle3_graph<double>(c, S.M64);
    }
    if (r != NS_OK) return r;
    ++ncyc;
    r = residual(false);
    if (r != NS_OK) return r;
    rn = c->red_h[kRedRes];
    if (rn < 0.5 * best) { best = rn; stall = 0; } else if (++stall >= 6) { status = NS_ERR_MG_STALL; break; }
  }
  if (dc64) {
    if (P64[pf] != S.PHI) CK(cudaMemcpyAsync(S.PHI, P64[pf], S.fb, cudaMemcpyDeviceToDevice, c->st), "phi copy");
  } else if (mixed) {
    LAUNCH(NS_PROF_DC_UPDATE, "phi to FP64", launch3_ff_cells(c->N, dc.pitch, dc.plane, S.PHF[pf], S.PHI, c->st));
  }
  (void)fallbacks;
  *cycles = ncyc;
  *res = r0 > 0 ? rn / r0 : 0.0;
  if (status != NS_OK) c->err = "Poisson residual stalled before the tolerance";
  return status;
}

}  // namespace

namespace nsh {

// ns_set_state layout of face d: (N + [d==0]) x (N + [d==1]) x (N + [d==2]), x fastest
cudaMemcpy3DParms copy_parms(ns_ctx* c, int d, const double* host, double* dev, bool put) {
  const int N = c->N;
  const size_t nx = N + (d == 0), ny = N + (d == 1), nz = N + (d == 2);
  cudaMemcpy3DParms q;
  std::memset(&q, 0, sizeof(q));
  cudaPitchedPtr h = make_cudaPitchedPtr(const_cast<double*>(host), nx * sizeof(double), nx, ny);
  cudaPitchedPtr g = make_cudaPitchedPtr(dev, (size_t)c->pitch * sizeof(double), (size_t)c->pitch, (size_t)N + 1);
  q.srcPtr = put ? h : g;
  q.dstPtr = put ? g : h;
  q.extent = make_cudaExtent(nx * sizeof(double), ny, nz);
  q.kind = put ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  return q;
}

int copy_cells3(ns_ctx* c, const double* host, double* dev, bool put) {
  const int N = c->N;
  cudaMemcpy3DParms q;
  std::memset(&q, 0, sizeof(q));
  cudaPitchedPtr h = make_cudaPitchedPtr(const_cast<double*>(host), (size_t)N * sizeof(double), N, N);
  cudaPitchedPtr g = make_cudaPitchedPtr(dev, (size_t)c->pitch * sizeof(double), (size_t)c->pitch, (size_t)N + 1);
  q.srcPtr = put ? h : g;
  q.dstPtr = put ? g : h;
  q.extent = make_cudaExtent((size_t)N * sizeof(double), N, N);
  q.kind = put ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
  return NS_OK;
}

int copy_faces3(ns_ctx* c, int d, const double* host, double* dev, bool put) {
  cudaMemcpy3DParms q = copy_parms(c, d, host, dev, put);
  CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
  return NS_OK;
}

int create3d(ns_ctx* c) {
  const int N = c->N;
  c->s3 = new State3D();
  State3D& S = *c->s3;
  S.fb = (size_t)c->pitch * (N + 1) * (N + 1) * sizeof(double);
  c->fbytes = S.fb;
  int r = NS_OK;
  for (int m = 0; m < 3 && r == NS_OK; ++m) {
    double** fs[] = {&S.U[m], &S.UP[m], &S.DU[m], &S.S[m], &S.B[0][m], &S.B[1][m], &S.B[2][m], &S.T[m],
                     &S.FL[0][m], &S.FL[1][m], &S.FL[2][m]};
    for (double** p : fs)
      if (r == NS_OK) r = alloc3(c, p, S.fb);
    if (r == NS_OK) r = alloc3(c, &S.PH[m], (size_t)(N + 4) * (N + 4) * (N + 4) * sizeof(double));
  }
  if (r == NS_OK) r = alloc3(c, &S.Pp, S.fb);
  if (r == NS_OK) r = alloc3(c, &S.PHI, S.fb);
  if (r == NS_OK) r = alloc3(c, &S.F, S.fb);
  if (r == NS_OK) r = alloc3(c, &S.part, (size_t)4 * (blocks3_face(N) + 1024) * sizeof(double));
  if (r == NS_OK) r = levels3<double>(c, S.M64, false);
  if (r == NS_OK && c->P.precision == NS_PREC_MIXED) {
    r = levels3<float>(c, S.M32, true);
    const size_t f32 = S.fb / 2, g32 = (size_t)(N + 4) * (N + 4) * (N + 4) * sizeof(float);
    for (int m = 0; m < 3 && r == NS_OK; ++m) {
      float** fs[] = {&S.UB32[m], &S.UB32b[m], &S.G0[m], &S.G0b[m], &S.E[0][m], &S.E[1][m]};
      for (float** p : fs)
        if (r == NS_OK) r = alloc3(c, p, f32);
      if (r == NS_OK) r = alloc3(c, &S.PHB32[m], g32);
      for (int b = 0; b < 2 && r == NS_OK; ++b) r = alloc3(c, &S.BF[b][m], S.fb);
    }
    for (int b = 0; b < 2 && r == NS_OK; ++b) r = alloc3(c, &S.PHF[b], S.fb);
    if (r == NS_OK) r = alloc3(c, &S.FF, S.fb);
    if (r == NS_OK && c->P.dc_residual == 1) r = alloc3(c, &S.PHI2, S.fb);
  }
  return r;
}

int set_state3d(ns_ctx* c, const double* const* u, const double* const* up, const double* p, double time) {
  State3D& S = *c->s3;
  for (int d = 0; d < 3; ++d) {
    cudaMemcpy3DParms q = copy_parms(c, d, u[d], S.U[d], true);
    CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
    q = copy_parms(c, d, up[d], S.UP[d], true);
    CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
  }
  int r = copy_cells3(c, p, S.Pp, true);
  if (r != NS_OK) return r;
  CK(cudaMemsetAsync(S.PHI, 0, S.fb, c->st), "memset phi");
  c->time = time;
  c->in_step = false;
  c->cart_pending = false;
  return ns_sync(c);
}

int get_state3d(ns_ctx* c, double* const* u, double* const* up, double* p, double* phi) {
  State3D& S = *c->s3;
  for (int d = 0; d < 3; ++d) {
    if (u && u[d]) {
      cudaMemcpy3DParms q = copy_parms(c, d, u[d], S.U[d], false);
      CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
    }
    if (up && up[d]) {
      cudaMemcpy3DParms q = copy_parms(c, d, up[d], S.UP[d], false);
      CK(cudaMemcpy3DAsync(&q, c->st), "3D copy");
    }
  }
  if (p) { int r = copy_cells3(c, p, S.Pp, false); if (r) return r; }
  if (phi) { int r = copy_cells3(c, phi, S.PHI, false); if (r) return r; }
  return ns_sync(c);
}

double* face3_ptr(ns_ctx* c, int id, int m) { return face3(c, id, m); }

double* field_ptr3d(ns_ctx* c, int field, int comp, bool* is_face) {
  State3D& S = *c->s3;
  *is_face = false;
  if (comp < 0 || comp > 2) return nullptr;
  switch (field) {
    case NS_FIELD_VEL: *is_face = true; return S.U[comp];
    case NS_FIELD_VEL_PREV: *is_face = true; return S.UP[comp];
    case NS_FIELD_VEL_STAR: *is_face = true; return face3(c, S.cur, comp);
    case NS_FIELD_PRESSURE: return S.Pp;
    case NS_FIELD_PHI: return S.PHI;
    case NS_FIELD_POISSON_RHS: return S.F;
    case NS_FIELD_CART: return S.CART[comp];
    default: return nullptr;
  }
}

int ensure_cart3(ns_ctx* c) {
  State3D& S = *c->s3;
  for (int m = 0; m < 3; ++m)
    if (!S.CART[m]) {
      const int r = alloc3(c, &S.CART[m], S.fb);
      if (r != NS_OK) return r;
    }
  return NS_OK;
}

int poisson3d(ns_ctx* c, int* cycles, double* res) {
  long long fb = 0;
  return poisson3(c, c->P.precision == NS_PREC_MIXED, cycles, res, &fb);
}

void gm3_fields(ns_ctx* c, double** phi, const double** f, double ih[3]) {
  State3D& S = *c->s3;
  *phi = S.PHI;
  *f = S.F;
  for (int d = 0; d < 3; ++d) ih[d] = S.M64.ih[0][d];
}

int gm3_precond(ns_ctx* c, const double* in, double* out) {
  State3D& S = *c->s3;
  MG3<double>& M = S.M64;
  double* x0 = M.x[0];
  double* f0 = M.f[0];
  const double* fm = M.fmean;
  CK(cudaMemsetAsync(out, 0, S.fb, c->st), "memset");
  M.x[0] = out;
  M.f[0] = const_cast<double*>(in);
  M.fmean = nullptr;
  const int r = vcycle3<double>(c, M);
  M.x[0] = x0;
  M.f[0] = f0;
  M.fmean = fm;
  return r;
}

int gm3_resnorm(ns_ctx* c) {
  State3D& S = *c->s3;
  S.M64.x[0] = S.PHI;
  S.M64.f[0] = S.F;
  S.M64.fmean = c->red + kRedMean;
  LAUNCH(NS_PROF_MG_RESNORM, "resnorm", launch3_mg_resnorm<double>(S.M64, S.part, c->counter, c->red + kRedRes, c->st));
  return NS_OK;
}

}  // namespace nsh

namespace {

// (hi, lo) float pair of an FP64 constant
void split2(double x, float* out) {
  out[0] = (float)x;
  out[1] = (float)(x - (double)out[0]);
}

// the anchor is evaluated exactly (float-float) on the first iteration, at
// most kAnchorEvery3 iterations after the last exact one, and once the
// pseudo-norm has fallen below kAnchorDrop3 times its value after the last
// exact one; the others update it by an FP32 increment evaluation, as in the
// 2D predictor. (A drop of 1e-2 left 1.1e-11 relative error in the small w of
// a 16^3 cavity after four steps; 1e-1 leaves 1.8e-12.)
constexpr int kAnchorEvery3 = 16;
constexpr double kAnchorDrop3 = 1e-1;

// One pseudo-iteration of the mixed-precision predictor (ns3d_mixed.cuh):
// the anchor G0 = G(u_b), three FP32 increment stages, u_b + e4 (float-float)
// into the other base buffer, the pseudo-norm of e4 into red[kRedNorm].
// The anchor is exact (the float-float passes) on the first and every
// kAnchorEvery3-th iteration. In between it is updated:
//   G(u_b + e4) = G(u_b) + dG(u_b; e4),
// with dG from the FP32 increment passes at the old base (rk = 1, e4 kept by
// the previous iteration's last stage, which also wrote the moved base rounded
// to FP32 into the other buffer of the UB32 pair). The FP32 cell velocity of
// the moved base is then rebuilt from its float-float pairs. Each update rounds the stored G0
// to FP32, an error relative to |G0| at that iteration; the errors add up
// until the next exact anchor and shift the converged u* by their sum over
// 1.5/dt. Refreshing the anchor whenever the pseudo-norm has dropped by
// kAnchorDrop3 keeps that sum within a small multiple of the final norm,
// however few iterations the step takes.
int mixed_iteration3(ns_ctx* c) {
  State3D& S = *c->s3;
  const bool exact = S.bf < 0 || S.mix_it - S.mix_last_exact >= kAnchorEvery3 ||
                     !(S.mix_norm >= kAnchorDrop3 * S.mix_norm_exact);
  if (exact) S.mix_last_exact = S.mix_it;
  S.mix_exact = exact;
  ++S.mix_it;
  if (!exact) {
    Inc3 u;
    std::memset(&u, 0, sizeof(u));
    u.g = c->g;
    for (int m = 0; m < 3; ++m) {
      u.ub[m] = S.UB32b[m];  // the old base (the pair was swapped after the last stage)
      u.g0[m] = S.G0[m];
      u.phb[m] = S.PHB32[m];
      u.phe[m] = reinterpret_cast<float*>(S.PH[m]);
      u.dt[m] = reinterpret_cast<float*>(S.T[m]);
      for (int d = 0; d < 3; ++d) u.dfl[d][m] = reinterpret_cast<float*>(S.FL[d][m]);
      u.ein[m] = S.E[1][m];
      u.eout[m] = S.G0b[m];
      u.inv_dx[m] = (float)c->g.inv_dx[m];
      u.vcoef[m] = (float)(c->g.inv_dx2[m] * c->g.inv_ren);
    }
    u.c15 = (float)c->g.c15;
    u.rk_prev = 1.f;
    u.rk = 1.f;
    LAUNCH(NS_PROF_INC, "anchor update cart 3d", launch3i_cart(u, c->st));
    LAUNCH(NS_PROF_INC, "anchor update total 3d", launch3i_total(u, c->st));
    LAUNCH(NS_PROF_INC, "anchor update face 3d", launch3i_face(u, c->st));
    for (int m = 0; m < 3; ++m) std::swap(S.G0[m], S.G0b[m]);
    AncFF b;
    std::memset(&b, 0, sizeof(b));
    b.g = c->g;
    for (int m = 0; m < 3; ++m) {
      b.uff[m] = S.BF[S.bf][m];
      b.ph32[m] = S.PHB32[m];
    }
    LAUNCH(NS_PROF_OTHER, "fp32 base 3d", launch3f_base32(b, c->st));
  }
  AncFF f;
  std::memset(&f, 0, sizeof(f));
  f.g = c->g;
  const int nb = S.bf < 0 ? 0 : 1 - S.bf;
  for (int m = 0; m < 3; ++m) {
    f.u[m] = face3(c, S.base, m);
    f.uff[m] = S.bf < 0 ? nullptr : S.BF[S.bf][m];
    f.S[m] = S.S[m];
    f.ph[m] = reinterpret_cast<float2*>(S.PH[m]);
    f.ph32[m] = S.PHB32[m];
    f.t[m] = reinterpret_cast<float2*>(S.T[m]);
    for (int d = 0; d < 3; ++d) f.fl[d][m] = reinterpret_cast<float2*>(S.FL[d][m]);
    f.g0[m] = S.G0[m];
    f.ub[m] = S.UB32[m];
    split2(c->g.inv_dx[m], f.inv_dx[m]);
    split2(c->g.inv_dx2[m] * c->g.inv_ren, f.vcoef[m]);
  }
  split2(c->g.c15, f.c15);
  if (exact) {
    LAUNCH(NS_PROF_ANCHOR, "anchor cart 3d", launch3f_cart(f, c->st));
    LAUNCH(NS_PROF_ANCHOR, "anchor total 3d", launch3f_total(f, c->st));
    LAUNCH(NS_PROF_ANCHOR, "anchor face 3d", launch3f_face(f, c->st));
  }
  Inc3 q;
  std::memset(&q, 0, sizeof(q));
  q.g = c->g;
  for (int m = 0; m < 3; ++m) {
    q.ub[m] = S.UB32[m];
    q.g0[m] = S.G0[m];
    q.phb[m] = S.PHB32[m];
    q.phe[m] = reinterpret_cast<float*>(S.PH[m]);
    q.dt[m] = reinterpret_cast<float*>(S.T[m]);
    for (int d = 0; d < 3; ++d) q.dfl[d][m] = reinterpret_cast<float*>(S.FL[d][m]);
    q.base64[m] = face3(c, S.base, m);
    q.baseff[m] = S.bf < 0 ? nullptr : S.BF[S.bf][m];
    q.outff[m] = S.BF[nb][m];
    q.inv_dx[m] = (float)c->g.inv_dx[m];
    q.vcoef[m] = (float)(c->g.inv_dx2[m] * c->g.inv_ren);
  }
  q.c15 = (float)c->g.c15;
  q.part = S.part;
  q.counter = c->counter;
  q.norm_out = c->red + kRedNorm;
  for (int s = 1; s <= 3; ++s) {
    for (int m = 0; m < 3; ++m) {
      q.ein[m] = s == 1 ? nullptr : S.E[s == 2 ? 0 : 1][m];
      q.eout[m] = S.E[s == 1 ? 0 : 1][m];
    }
    q.rk_prev = (float)c->rk[s - 1];
    q.rk = (float)c->rk[s];
    q.last = s == 3;
    q.keep_e = s == 3;
    for (int m = 0; m < 3; ++m) q.ubout[m] = s == 3 ? S.UB32b[m] : nullptr;
    LAUNCH(NS_PROF_INC, "increment cart 3d", launch3i_cart(q, c->st));
    LAUNCH(NS_PROF_INC, "increment total 3d", launch3i_total(q, c->st));
    LAUNCH(NS_PROF_INC, "increment face 3d", launch3i_face(q, c->st));
  }
  S.bf = nb;
  for (int m = 0; m < 3; ++m) std::swap(S.UB32[m], S.UB32b[m]);  // UB32: the moved base, UB32b: the old one
  return NS_OK;
}

// u* (float-float) to FP64 in a free buffer, once the iteration stops
int mixed_finalize3(ns_ctx* c) {
  State3D& S = *c->s3;
  if (S.bf < 0) return NS_OK;
  const int outb = pick3(S.base, S.base);
  const float2* in[3] = {S.BF[S.bf][0], S.BF[S.bf][1], S.BF[S.bf][2]};
  double* out[3] = {S.B[outb][0], S.B[outb][1], S.B[outb][2]};
  LAUNCH(NS_PROF_OTHER, "store u* 3d", launch3f_store(c->g, in, out, c->st));
  S.base = S.cur = outb;
  S.bf = -1;
  return NS_OK;
}

}  // namespace

namespace nsh {

// ---- the per-call-site building blocks in 3D (the 2D entry points dispatch
// here). The RK stage is the FP64 stage of the context's own predictor (three
// passes: ghosted cell velocity, fluxes and totals, face update with the
// pseudo-norm), so a step assembled from the blocks equals ns_step in FP64.

// main.cpp:879-887: du, S from (u^n, u^{n-1}, p); the u^{n-1} buffer becomes
// the target of the projection
int step_begin3d(ns_ctx* c) {
  State3D& S = *c->s3;
  Arg3 a = args(c);
  for (int m = 0; m < 3; ++m) {
    a.un[m] = S.U[m];
    a.uprev[m] = S.UP[m];
    a.du[m] = S.DU[m];
    a.S[m] = S.S[m];
  }
  a.p = S.Pp;
  LAUNCH(NS_PROF_STEP_BEGIN, "step begin 3d", launch3_step_begin(a, c->st));
  for (int m = 0; m < 3; ++m) std::swap(S.U[m], S.UP[m]);
  c->time += c->dt;
  S.base = S.cur = -1;
  c->in_step = true;
  c->norm_ready = false;
  return NS_OK;
}

// main.cpp:931-1017, one RK pseudo-stage (FP64)
int rk_stage3d(ns_ctx* c, int sub) {
  State3D& S = *c->s3;
  const int outb = pick3(S.base, S.cur);
  Arg3 b = args(c);
  for (int m = 0; m < 3; ++m) {
    b.u[m] = face3(c, S.cur, m);
    b.ub[m] = face3(c, S.base, m);
    b.S[m] = S.S[m];
    b.out[m] = S.B[outb][m];
  }
  b.rk = c->rk[sub];
  b.do_norm = (sub == 3);
  b.red_out = c->red + kRedNorm;
  const bool use_cart = c->cart_pending;
  for (int m = 0; m < 3; ++m) b.cart[m] = use_cart ? S.CART[m] : nullptr;
  LAUNCH(NS_PROF_STAGE_FAST, "cart 3d", launch3_cart(b, c->st));
  LAUNCH(NS_PROF_STAGE_FAST, "total 3d", launch3_total(b, c->st));
  LAUNCH(NS_PROF_STAGE_FAST, "face 3d", launch3_face(b, c->st));
  c->cart_pending = false;
  S.cur = outb;
  if (sub == 3) c->norm_ready = true;
  return NS_OK;
}

// explicit_time_marching (momentum.cpp:96-192, main.cpp:902-925): one pass
// from u* = u^n (step begin leaves base and u* on u^n), R = -grad p +
// avg(total) + du / (2 dt), u* += (dt / 1.5) R, then Error_Computation and
// velCont <- velStar. With S = -grad p + (0.5/dt) du + (1.5/dt) u^n, R is the
// face pass's S - (1.5/dt) u* + avg(total) at u* = u^n, so the RK passes run
// once with rk = dt / 1.5. The flux ghosts of this mode are set when the
// context is made: zero normal total at walls (no reflection, quirk Q3), the
// periodic wrap otherwise.
int explicit_predictor3d(ns_ctx* c, double* norm) {
  State3D& S = *c->s3;
  const int outb = pick3(S.base, S.cur);
  Arg3 b = args(c);
  for (int m = 0; m < 3; ++m) {
    b.u[m] = face3(c, S.cur, m);
    b.ub[m] = face3(c, S.cur, m);
    b.S[m] = S.S[m];
    b.out[m] = S.B[outb][m];
  }
  b.rk = c->dt / 1.5;
  b.do_norm = 1;
  b.red_out = c->red + kRedNorm;
  for (int m = 0; m < 3; ++m) b.cart[m] = c->cart_pending ? S.CART[m] : nullptr;
  LAUNCH(NS_PROF_EXPLICIT, "cart 3d", launch3_cart(b, c->st));
  LAUNCH(NS_PROF_EXPLICIT, "total 3d", launch3_total(b, c->st));
  LAUNCH(NS_PROF_EXPLICIT, "explicit face 3d", launch3_face(b, c->st));
  c->cart_pending = false;
  S.cur = outb;
  int r = sync_red(c, kRedNorm, 1);
  if (r != NS_OK) return r;
  if (norm) *norm = c->red_h[kRedNorm];
  S.base = S.cur;
  return NS_OK;
}

// Error_Computation and velCont <- velStar (main.cpp:1019-1026)
int pseudo_norm3d(ns_ctx* c, double* norm) {
  State3D& S = *c->s3;
  int r = sync_red(c, kRedNorm, 1);
  if (r != NS_OK) return r;
  if (norm) *norm = c->red_h[kRedNorm];
  S.base = S.cur;
  c->norm_ready = false;
  return NS_OK;
}

// poisson_righthand_side_calc (fn_rhs.cpp:71-125) on u*
int poisson_rhs3d(ns_ctx* c, double* divmax, double* sum) {
  State3D& S = *c->s3;
  Arg3 p = args(c);
  for (int m = 0; m < 3; ++m) p.u[m] = face3(c, S.cur, m);
  p.f = S.F;
  p.red_out = c->red + kRedDivBefore;
  LAUNCH(NS_PROF_POISSON_RHS, "rhs 3d", launch3_rhs(p, c->st));
  int r = sync_red(c, kRedDivBefore, 2);
  if (r != NS_OK) return r;
  if (divmax) *divmax = c->red_h[kRedDivBefore];
  if (sum) *sum = c->red_h[kRedSum];
  return NS_OK;
}

// poisson_advance (poisson.cpp:41-186): FP64 V-cycles, or (NS_PREC_MIXED in a
// mixed context) FP32 V-cycles inside the float-float defect correction
int poisson_solve3d(ns_ctx* c, int precision, int* cycles, double* res) {
  State3D& S = *c->s3;
  const bool mixed = precision == NS_PREC_MIXED && S.M32.L > 0;
  long long fb = 0;
  int cyc = 0;
  double rr = 0.0;
  const int r = poisson3(c, mixed, &cyc, &rr, &fb);
  if (cycles) *cycles = cyc;
  if (res) *res = rr;
  return r;
}

// main.cpp:1078-1164 (phi ghosts, update_solution) + the divergence check of
// main.cpp:1180
int project3d(ns_ctx* c, double* divmax) {
  State3D& S = *c->s3;
  Arg3 p = args(c);
  for (int m = 0; m < 3; ++m) {
    p.u[m] = face3(c, S.cur, m);
    p.out[m] = S.U[m];
  }
  p.p = S.Pp;
  p.pw = S.Pp;
  p.phi = S.PHI;
  p.red_out = c->red + kRedDivAfter;
  LAUNCH(NS_PROF_PROJECT, "project 3d", launch3_project(p, c->st));
  LAUNCH(NS_PROF_PROJECT, "div 3d", launch3_div(p, c->st));
  int r = sync_red(c, kRedDivAfter, 1);
  if (r != NS_OK) return r;
  if (divmax) *divmax = c->red_h[kRedDivAfter];
  c->in_step = false;
  return NS_OK;
}

// step begin and the dual-time pseudo-iterations: u* in face3(c, S.cur); the
// state (U, UP, time) is rotated as in ns_step_begin
int predictor3d(ns_ctx* c, ns_step_stats* sp) {
  State3D& S = *c->s3;
  ns_step_stats& s = *sp;
  int r = step_begin3d(c);
  if (r != NS_OK) return r;
  // ---- dual-time pseudo-iterations (main.cpp:898-1040)
  const bool mixed = c->P.precision == NS_PREC_MIXED && c->P.pseudo_timestepping != 0;
  S.bf = -1;
  S.mix_it = 0;
  S.mix_last_exact = 0;
  int count = 0;
  double norm = 1.e9;
  while (norm > c->P.momentum_tolerance) {
    if (c->P.pseudo_timestepping == 0) {  // one explicit pass, then break (main.cpp:902-925)
      r = explicit_predictor3d(c, &norm);
      if (r != NS_OK) return r;
      count = 1;
      break;
    }
    if (mixed && !c->cart_pending) {
      // the analytic first-stage cell velocity of ns_init_fields(TGV) is only
      // consumed by the FP64 stages, so that iteration runs in FP64 (the next
      // one starts its exact anchor from the FP64 base)
      r = mixed_iteration3(c);
      if (r != NS_OK) return r;
      r = sync_red(c, kRedNorm, 1);
      if (r != NS_OK) return r;
      norm = c->red_h[kRedNorm];
      S.mix_norm = norm;
      if (S.mix_exact) S.mix_norm_exact = norm;
      S.base = S.cur;
    } else {
      for (int sub = 0; sub < 4; ++sub) {
        r = rk_stage3d(c, sub);
        if (r != NS_OK) return r;
      }
      r = pseudo_norm3d(c, &norm);
      if (r != NS_OK) return r;
    }
    count++;
    if (std::isnan(norm)) return fail(c, NS_ERR_NONFINITE, "pseudo-increment norm is NaN (non-finite fields)");
    if (count > c->P.iter_num) { s.status = NS_WARN_PSEUDO_MAXITER; break; }
    if (norm > 1.e2) { s.status = NS_WARN_PSEUDO_DIVERGED; break; }
  }
  s.pseudo_iters = count;
  s.norm_error = norm;
  return mixed ? mixed_finalize3(c) : NS_OK;
}

int step3d(ns_ctx* c, ns_step_stats* stats) {
  ns_step_stats s;
  std::memset(&s, 0, sizeof(s));
  if (c->ev_ok) cudaEventRecord(c->ev[0], c->st);
  int r = predictor3d(c, &s);
  if (r != NS_OK) return r;
  if (c->ev_ok) cudaEventRecord(c->ev[1], c->st);
  // ---- Poisson right-hand side, solve, projection
  r = poisson_rhs3d(c, &s.div_before, &s.rhs_sum);
  if (r != NS_OK) return r;
  if (!std::isfinite(s.div_before) || !std::isfinite(s.rhs_sum))
    return fail(c, NS_ERR_NONFINITE, "Poisson right-hand side is not finite");
  long long fb = 0;
  const int mg = poisson3(c, c->P.precision == NS_PREC_MIXED, &s.poisson_cycles, &s.poisson_res, &fb);
  if (mg != NS_OK && mg != NS_ERR_MG_STALL) return mg;
  if (c->ev_ok) cudaEventRecord(c->ev[2], c->st);
  r = project3d(c, &s.div_after);
  if (r != NS_OK) return r;
  c->step++;
  if (c->ev_ok) {
    cudaEventRecord(c->ev[3], c->st);
    cudaEventSynchronize(c->ev[3]);
    float t0 = 0, t1 = 0, t2 = 0;
    cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&t2, c->ev[2], c->ev[3]);
    s.ms_predictor = t0; s.ms_poisson = t1; s.ms_project = t2;
  }
  if (stats) *stats = s;
  if (mg != NS_OK) return mg;
  return s.status;
}

}  // namespace nsh
