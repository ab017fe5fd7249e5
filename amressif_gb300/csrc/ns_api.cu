// C ABI and host driver of the GB300 fractional-step advance.
//
// The host side restates main_main's time loop (main.cpp:875-1202) over
// device-resident fields: one fused kernel per RK pseudo-stage, an 8-byte
// read-back of the pseudo-increment norm per pseudo-iteration (the loop
// condition of main.cpp:898), then the Poisson right-hand side, the
// multigrid solve and the projection.
#include <atomic>
#include <chrono>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/amressif_gpu.h"
#include "anchor_ff2d.cuh"
#include "ctx.h"
#include "dc_ff2d.cuh"
#define NS_GMRES_ARGS_ONLY  // structs and constants only: the kernels are compiled in kernels_fast.cu
#include "gmres2d.cuh"
#include "launch.h"
#include "stage_inc2d.cuh"

using namespace ns;
using namespace nsh;

namespace nsh {

int fail(ns_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_check(ns_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return NS_OK;
  return fail(c, NS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int alloc_field(ns_ctx* c, double** p) {
  if (cudaMalloc(p, c->fbytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc failed");
  if (cudaMemsetAsync(*p, 0, c->fbytes, c->st) != cudaSuccess) return fail(c, NS_ERR_CUDA, "memset failed");
  return NS_OK;
}

// The pseudo-norm of the iteration just queued, from the mapped note the
// reducing launch writes: poll its sequence number for up to kNoteWaitS
// seconds (the launches run meanwhile), then read the norm. Saves the
// device-to-host copy and the stream synchronisation per pseudo-iteration;
// false (the caller falls back to them) when there is no note or it is late.
constexpr double kNoteWaitS = 2.0;
bool read_note(ns_ctx* c, double* norm) {
  if (c->note_h == nullptr || c->note_d == nullptr) return false;
  const volatile double* nh = c->note_h;
  const auto t0 = std::chrono::steady_clock::now();
  for (unsigned spin = 0;; ++spin) {
    if (nh[1] == c->note_seq) {
      std::atomic_thread_fence(std::memory_order_acquire);
      *norm = nh[0];
      return true;
    }
    if ((spin & 1023u) == 1023u &&
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > kNoteWaitS)
      return false;
  }
}

int sync_red(ns_ctx* c, int first, int count) {
  CK(cudaMemcpyAsync(c->red_h + first, c->red + first, count * sizeof(double), cudaMemcpyDeviceToHost, c->st), "readback");
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

cudaEvent_t pool_get(ns_ctx* c) {
  if (!c->evpool.empty()) {
    cudaEvent_t e = c->evpool.back();
    c->evpool.pop_back();
    return e;
  }
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Fold completed launch timings into the per-kind totals (stream is idle).
void prof_resolve(ns_ctx* c) {
  for (auto& p : c->pend) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
      c->pms[p.first] += ms;
      c->pcnt[p.first] += 1;
    }
    c->evpool.push_back(p.second.first);
    c->evpool.push_back(p.second.second);
  }
  c->pend.clear();
}

}  // namespace nsh

namespace {

// ghost rule table of one velCart side (utilities.cpp:62-349)
int make_cart_bc(const ns_params& P, int d, int side, CartBC& b) {
  const int code = side == 0 ? P.bc_lo[d] : P.bc_hi[d];
  for (int m = 0; m < 3; ++m) { b.rule[m] = kNeg; b.add[m] = 0.0; }
  if (code == 111 || code == 135) return NS_OK;
  bool slip = (code == -135);
  if (d == 0 && side == 1) {
    // east wall: the reference tests slip as "== 1" (utilities.cpp:152)
    if (!P.fix_quirks && code == -135) return NS_ERR_UNSUPPORTED;
    slip = (code == 1) || (P.fix_quirks && code == -135);
  }
  if (slip) {
    for (int m = 0; m < 3; ++m) b.rule[m] = (m == d) ? kNeg : kPos;
    return NS_OK;
  }
  if (code == 165 || (code == -165 && d == 0 && side == 0)) {
    for (int m = 0; m < 3; ++m) { b.rule[m] = kInlet; b.add[m] = 2.0; }
    if (d == 1 && side == 1)
      for (int m = 0; m < 3; ++m) b.add[m] = 2 * P.inflow_waveform[m];
    return NS_OK;
  }
  return NS_ERR_BC;
}

long round_up(long x, long a) { return (x + a - 1) / a * a; }

void free_all(ns_ctx* c) {
  auto F = [](void* p) { if (p) cudaFree(p); };
  for (int m = 0; m < 2; ++m) {
    F(c->U[m]); F(c->UP[m]); F(c->DU[m]); F(c->S[m]); F(c->CART[m]); F(c->PHI[m]); F(c->CONV[m]);
    for (int i = 0; i < 3; ++i) F(c->B[i][m]);
    F(c->SH[m]); F(c->G0[m]); F(c->G0b[m]); F(c->E[0][m]); F(c->E[1][m]);
    F(c->BH[0][m]); F(c->BH[1][m]); F(c->BL[0][m]); F(c->BL[1][m]); F(c->SFh[m]); F(c->SFl[m]);
    F(c->PFh[m]); F(c->PFl[m]);
  }
  F(c->FFh); F(c->FFl);
  F(c->Pp); F(c->F);
  F(c->lid_col);
  F(c->cell_tmp);
  F(c->check);
  free3d(c);
  for (double* v : c->gm_v) F(v);
  F(c->gm_w); F(c->gm_z); F(c->gm_b); F(c->gm_part); F(c->gm_dev);
  if (c->gm_host) cudaFreeHost(c->gm_host);
  free_adjoint(c);
  for (int l = 1; l < c->M64.L; ++l) { F(c->M64.x[l]); F(c->M64.f[l]); }
  for (int l = 0; l < c->M64.L; ++l) F(c->M64.x2[l]);
  for (int l = 0; l < c->M32.L; ++l) { F(c->M32.x[l]); F(c->M32.f[l]); F(c->M32.x2[l]); }
  F(c->part); F(c->counter); F(c->red);
  if (c->red_h) cudaFreeHost(c->red_h);
  if (c->note_h) cudaFreeHost(c->note_h);
  if (c->ev_ok) for (auto& e : c->ev) cudaEventDestroy(e);
  for (auto& p : c->pend) { cudaEventDestroy(p.second.first); cudaEventDestroy(p.second.second); }
  for (auto& e : c->evpool) cudaEventDestroy(e);
  for (auto& row : c->vg)
    for (auto& G : row)
      if (G.exec) cudaGraphExecDestroy(G.exec);
  if (c->own_stream && c->st) cudaStreamDestroy(c->st);
  for (auto& e : c->side_ev)
    if (e) cudaEventDestroy(e);
  if (c->side) cudaStreamDestroy(c->side);
}

template <typename T>
int alloc_levels(ns_ctx* c, MGLevels<T>& M, bool own_level0) {
  int n = c->N;
  M.L = 0;
  M.periodic[0] = c->g.periodic[0];
  M.periodic[1] = c->g.periodic[1];
  M.fmean = nullptr;
  M.check = c->check;
  double hx = c->g.dx[0], hy = c->g.dx[1];
  while (true) {
    const int l = M.L;
    if (l >= kMaxLevels) return fail(c, NS_ERR_ARG, "too many multigrid levels");
    M.n[l] = n;
    // level 0 shares the row pitch of the velocity / pressure fields
    M.pitch[l] = (l == 0) ? c->pitch : round_up(n, 32);
    M.invh2[l][0] = 1.0 / (hx * hx);
    M.invh2[l][1] = 1.0 / (hy * hy);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        const double diag = a * M.invh2[l][0] + b * M.invh2[l][1];
        M.invdiag[l][a + 3 * b] = diag > 0 ? 1.0 / diag : 0.0;
        M.idg[l][a + 3 * b] = (T)M.invdiag[l][a + 3 * b];
      }
    M.ih[l][0] = (T)M.invh2[l][0];
    M.ih[l][1] = (T)M.invh2[l][1];
    M.x[l] = nullptr;
    M.x2[l] = nullptr;
    M.f[l] = nullptr;
    const size_t bytes = (size_t)M.pitch[l] * (n + 1) * sizeof(T);
    if (l > 0 || own_level0) {
      if (cudaMalloc(&M.x[l], bytes) != cudaSuccess || cudaMalloc(&M.f[l], bytes) != cudaSuccess)
        return fail(c, NS_ERR_NOMEM, "cudaMalloc (multigrid) failed");
      cudaMemsetAsync(M.x[l], 0, bytes, c->st);
      cudaMemsetAsync(M.f[l], 0, bytes, c->st);
    }
    if (cudaMalloc(&M.x2[l], bytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc (multigrid) failed");
    cudaMemsetAsync(M.x2[l], 0, bytes, c->st);
    M.L++;
    if (!(n % 4 == 0 && n > 4)) break;
    n /= 2;
    hx *= 2;
    hy *= 2;
  }
  return NS_OK;
}

StageArgs base_stage_args(ns_ctx* c) {
  StageArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  a.p = c->Pp;
  for (int m = 0; m < 2; ++m) {
    a.un[m] = c->UP[m];
    a.du[m] = c->DU[m];
    a.S[m] = c->S[m];
  }
  a.part = c->part;
  a.counter = c->counter;
  a.norm_out = c->red + kRedNorm;
  return a;
}

int pick_out(int base, int in) {
  for (int i = 0; i < 3; ++i)
    if (i != base && i != in) return i;
  return -2;
}

}  // namespace

extern "C" {

void ns_params_default(ns_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->dim = 2;
  p->n_cell = 32;
  p->max_grid_size[0] = 32; p->max_grid_size[1] = 16; p->max_grid_size[2] = 16;
  for (int d = 0; d < 3; ++d) { p->prob_lo[d] = 0.0; p->prob_hi[d] = 1.0; }
  p->ren = 100.0;
  p->vis = 1.0;
  p->cfl = 0.9;
  p->fixed_dt = 1.0e-3;
  p->iter_num = 100;
  p->momentum_tolerance = 1.e-10;
  p->pseudo_timestepping = 1;
  p->bc_lo[0] = 135; p->bc_lo[1] = 135; p->bc_lo[2] = 135;
  p->bc_hi[0] = 135; p->bc_hi[1] = 165; p->bc_hi[2] = 135;
  p->inflow_waveform[0] = 1.0;
  p->nsteps = 11;
  p->precision = NS_PREC_FP64_EXACT;
  p->fix_quirks = 0;
  p->poisson_tol_rel = 1.0e-10;
  p->poisson_tol_div = 0.0;
  p->poisson_max_cycles = 200;
  p->dtau_clip = 0;
  p->poisson_solver = 0;
  p->gmres_restart = 30;
  p->dc_residual = 0;
  p->poisson_warm_start = 0;
  p->conv_scheme = NS_CONV_NEW_QUICK;
}

int ns_params_parse_file(ns_params* p, const char* path) {
  std::ifstream in(path);
  if (!in) return NS_ERR_ARG;
  std::string line;
  while (std::getline(in, line)) {
    const size_t h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string key = line.substr(0, eq), val = line.substr(eq + 1);
    key.erase(0, key.find_first_not_of(" \t"));
    key.erase(key.find_last_not_of(" \t") + 1);
    std::istringstream vs(val);
    std::vector<double> v;
    std::string tok;
    bool bad = false;
    while (vs >> tok) {
      char* end = nullptr;
      const double x = std::strtod(tok.c_str(), &end);
      if (end == tok.c_str() || *end != '\0') { bad = true; break; }
      v.push_back(x);
    }
    if (bad || v.empty()) continue;  // e.g. "chk_int = = 10" of the shipped inputs
    auto I = [&](int k) { return (int)v[std::min<size_t>(k, v.size() - 1)]; };
    auto D = [&](int k) { return v[std::min<size_t>(k, v.size() - 1)]; };
    if (key == "n_cell") p->n_cell = I(0);
    else if (key == "max_grid_size_x") p->max_grid_size[0] = I(0);
    else if (key == "max_grid_size_y") p->max_grid_size[1] = I(0);
    else if (key == "max_grid_size_z") p->max_grid_size[2] = I(0);
    else if (key == "nsteps") p->nsteps = I(0);
    else if (key == "fixed_dt") p->fixed_dt = D(0);
    else if (key == "cfl") p->cfl = D(0);
    else if (key == "IterNum") p->iter_num = I(0);
    else if (key == "ren") p->ren = D(0);
    else if (key == "vis") p->vis = D(0);
    else if (key == "momentum_tolerance") p->momentum_tolerance = D(0);
    else if (key == "PSEUDO_TIMESTEPPING") p->pseudo_timestepping = I(0);
    else if (key == "phy_bc_lo") for (int d = 0; d < 3 && d < (int)v.size(); ++d) p->bc_lo[d] = I(d);
    else if (key == "phy_bc_hi") for (int d = 0; d < 3 && d < (int)v.size(); ++d) p->bc_hi[d] = I(d);
    else if (key == "inflow_waveform") for (int d = 0; d < 3 && d < (int)v.size(); ++d) p->inflow_waveform[d] = D(d);
    else if (key == "lo_phy_dim") for (int d = 0; d < 3 && d < (int)v.size(); ++d) p->prob_lo[d] = D(d);
    else if (key == "hi_phy_dim") for (int d = 0; d < 3 && d < (int)v.size(); ++d) p->prob_hi[d] = D(d);
  }
  return NS_OK;
}

int ns_ctx_create(const ns_params* p, void* stream, ns_ctx** out) {
  if (!p || !out) return NS_ERR_ARG;
  *out = nullptr;
  if (p->dim != 2 && p->dim != 3) return NS_ERR_UNSUPPORTED;
  if (p->n_cell < 8 || p->n_cell % 8 != 0) return NS_ERR_ARG;
  const int D = p->dim;
  {
    // the multigrid halves n while n % 4 == 0 and n > 4; its coarsest level
    // must fit the single-block bottom solve (2D: <= 32, 3D: <= 24)
    int nc = p->n_cell;
    while (nc % 4 == 0 && nc > 4) nc /= 2;
    if (nc > (D == 2 ? kBottomN : 24)) return NS_ERR_UNSUPPORTED;
  }
  if (!(p->ren > 0)) return NS_ERR_ARG;
  if (p->dc_residual != 0 && p->dc_residual != 1) return NS_ERR_ARG;
  if (p->poisson_warm_start != 0 && p->poisson_warm_start != 1) return NS_ERR_ARG;
  if (p->conv_scheme < NS_CONV_NEW_QUICK || p->conv_scheme > NS_CONV_UMIST_FORM) return NS_ERR_ARG;
  if (p->conv_scheme != NS_CONV_NEW_QUICK && p->precision == NS_PREC_MIXED) return NS_ERR_UNSUPPORTED;
  // convective_flux_calc_quick reads face 0 from boxes that do not hold it,
  // and in 3D writes component k of a one-component fab
  if (p->conv_scheme == NS_CONV_QUICK &&
      (D == 3 || p->max_grid_size[0] < p->n_cell || p->max_grid_size[1] < p->n_cell))
    return NS_ERR_UNSUPPORTED;
  ns_ctx* c = new ns_ctx();
  c->P = *p;
  const int N = p->n_cell;
  c->N = N;
  c->pitch = round_up(N + 1, 32);
  c->fbytes = (size_t)c->pitch * (N + 1) * sizeof(double);
  Geom& g = c->g;
  std::memset(&g, 0, sizeof(g));
  g.N = N;
  g.dim = 2;
  g.pitch = c->pitch;
  g.plane = c->pitch * (N + 1);
  for (int d = 0; d < 3; ++d) g.dx[d] = (p->prob_hi[d] - p->prob_lo[d]) / (double)N;
  g.conv_scheme = p->conv_scheme;
  for (int d = 0; d < D; ++d) {
    const bool lo111 = p->bc_lo[d] == 111, hi111 = p->bc_hi[d] == 111;
    if (lo111 != hi111) { delete c; return NS_ERR_BC; }
    g.periodic[d] = lo111 && hi111;
    if (p->pseudo_timestepping == 0)
      g.flux_ghost[d] = g.periodic[d] ? kWrap : kZero;  // explicit mode: no reflection (quirk Q3)
    else
      g.flux_ghost[d] = (g.periodic[d] && p->fix_quirks) ? kWrap : kReflect;
    g.ctx_mirror[d] = (g.periodic[d] && p->fix_quirks) ? 0 : 1;
    for (int side = 0; side < 2; ++side) {
      const int r = make_cart_bc(*p, d, side, g.bc[2 * d + side]);
      if (r != NS_OK) {
        delete c;
        return r;
      }
    }
  }
  // dt rule of main.cpp:285-294
  double coeff = 1.0 / (g.dx[0] * g.dx[0]) + 1.0 / (g.dx[1] * g.dx[1]);
  if (D == 3) coeff += 1.0 / (g.dx[2] * g.dx[2]);
#ifdef NS_BOUNDS_CHECK
  if (cudaMalloc(&c->check, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(c->check, 0, 4 * sizeof(unsigned long long)) != cudaSuccess) {
    if (c->check) cudaFree(c->check);
    delete c;
    return NS_ERR_NOMEM;
  }
  g.check = c->check;
#endif
  c->dt = p->fixed_dt != -1.0 ? p->fixed_dt : p->cfl / (2.0 * coeff);
  g.dt = c->dt;
  g.ren = p->ren;
  for (int d = 0; d < 3; ++d) {
    g.inv_dx[d] = 1.0 / g.dx[d];
    g.dx2[d] = g.dx[d] * g.dx[d];
    g.inv_dx2[d] = 1.0 / g.dx2[d];
  }
  g.inv_ren = 1.0 / p->ren;
  g.c15 = 1.5 / c->dt;
  g.c05 = 0.5 / c->dt;
  g.c2dt = 1.0 / (2.0 * c->dt);
  g.dt15 = c->dt / 1.5;
  // RK coefficients (main.cpp:861-870), optionally clipped to 0.9 x the RK4
  // real-axis stability limit of the stiffest mode
  double d_tau = 0.4 * c->dt;
  if (p->dtau_clip) {
    const double lam = 4.0 / p->ren * coeff + 1.5 / c->dt;
    d_tau = std::min(d_tau, 0.9 * 2.785 / lam);
  }
  c->rk[0] = d_tau * 0.25;
  c->rk[1] = d_tau * (1.0 / 3.0);
  c->rk[2] = d_tau * 0.5;
  c->rk[3] = d_tau * 1.0;

  if (stream) {
    c->st = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) { delete c; return NS_ERR_CUDA; }
    c->own_stream = true;
  }
  int r = NS_OK;
  g.dim = D;
  if (D == 3) r = create3d(c);
  for (int m = 0; m < 2 && r == NS_OK && D == 2; ++m) {
    r = alloc_field(c, &c->U[m]);
    if (r == NS_OK) r = alloc_field(c, &c->UP[m]);
    if (r == NS_OK) r = alloc_field(c, &c->DU[m]);
    if (r == NS_OK) r = alloc_field(c, &c->S[m]);
    if (r == NS_OK) r = alloc_field(c, &c->PHI[m]);
    for (int i = 0; i < 3 && r == NS_OK; ++i) r = alloc_field(c, &c->B[i][m]);
  }
  for (int m = 0; m < 2 && r == NS_OK && D == 2 && p->conv_scheme == NS_CONV_QUICK; ++m)
    r = alloc_field(c, &c->CONV[m]);
  if (r == NS_OK && D == 2) r = alloc_field(c, &c->Pp);
  if (r == NS_OK && D == 2) r = alloc_field(c, &c->F);
  if (r == NS_OK && D == 2) r = alloc_levels<double>(c, c->M64, false);
  if (r == NS_OK && D == 2) r = alloc_levels<float>(c, c->M32, true);
  if (r == NS_OK) {
    // reduction scratch: 2 partials per block of the largest launch
    const size_t nb = (size_t)((N + 31) / 32) * ((N + 7) / 8) + 1024;
    if (cudaMalloc(&c->part, 4 * nb * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->counter, 64 * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&c->red, 16 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&c->red_h, 16 * sizeof(double)) != cudaSuccess)
      r = fail(c, NS_ERR_NOMEM, "cudaMalloc (reductions) failed");
    else {
      cudaMemsetAsync(c->counter, 0, 64 * sizeof(unsigned), c->st);
      cudaMemsetAsync(c->red, 0, 16 * sizeof(double), c->st);
      if (cudaHostAlloc(&c->note_h, 2 * sizeof(double), cudaHostAllocMapped) != cudaSuccess) {
        c->note_h = nullptr;
        cudaGetLastError();
      } else if (cudaHostGetDevicePointer(&c->note_d, c->note_h, 0) != cudaSuccess) {
        c->note_d = nullptr;
        cudaGetLastError();
      } else {
        c->note_h[0] = c->note_h[1] = 0.0;
      }
    }
  }
  if (r == NS_OK) {
    bool ok = true;
    for (auto& e : c->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    c->ev_ok = ok;
    c->M64.x[0] = c->PHI[0];
    c->M64.f[0] = c->F;
    c->M64.fmean = c->red + kRedMean;
    c->lb = 0;
    while (c->lb < c->M64.L && c->M64.n[c->lb] > kBottomN) c->lb++;
    if (cudaStreamSynchronize(c->st) != cudaSuccess) r = fail(c, NS_ERR_CUDA, "init sync failed");
  }
  if (r != NS_OK) {
    free_all(c);
    delete c;
    return r;
  }
  *out = c;
  return NS_OK;
}

void ns_ctx_destroy(ns_ctx* c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  free_all(c);
  delete c;
}

const char* ns_last_error(const ns_ctx* c) { return c ? c->err.c_str() : "null context"; }
double ns_get_dt(const ns_ctx* c) { return c ? c->dt : 0.0; }
double ns_get_time(const ns_ctx* c) { return c ? c->time : 0.0; }

int ns_sync(ns_ctx* c) {
  if (!c) return NS_ERR_ARG;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

// ---- field movement -----------------------------------------------------------

static double* field_ptr(ns_ctx* c, int field, int comp, bool* is_face) {
  *is_face = false;
  switch (field) {
    case NS_FIELD_VEL: *is_face = true; return comp < 2 ? c->U[comp] : nullptr;
    case NS_FIELD_VEL_PREV: *is_face = true; return comp < 2 ? c->UP[comp] : nullptr;
    case NS_FIELD_VEL_STAR: *is_face = true; return comp < 2 ? face_ptr(c, c->cur, comp) : nullptr;
    case NS_FIELD_PRESSURE: return c->Pp;
    case NS_FIELD_PHI: return c->PHI[c->phi_cur];
    case NS_FIELD_POISSON_RHS: return c->F;
    case NS_FIELD_CART: return nullptr;
    default: return nullptr;
  }
}

// One box [lo, hi] of a field between the caller's Array4-style view and the
// device: one pitched 2D copy per k plane. The index box must lie inside the
// field's own index space; jstride must hold a row of the box, and in 3D
// kstride a plane of it (AMReX's Array4 strides satisfy both). A 2D context
// takes the single plane k = 0 (kstride is then unused).
static int box_copy(ns_ctx* c, int field, int comp, double* data, const int lo[3], const int hi[3], long long jstride,
                    long long kstride, int where_device, bool put) {
  if (!c || !data || !lo || !hi) return NS_ERR_ARG;
  const int D = c->P.dim;
  if (comp < 0 || comp >= D) return fail(c, NS_ERR_ARG, "box copy: component out of range");
  if (field == NS_FIELD_CART) {
    if (!put) return NS_ERR_ARG;
    for (int m = 0; m < 2 && D == 2; ++m)
      if (!c->CART[m]) {
        int r = alloc_field(c, &c->CART[m]);
        if (r != NS_OK) return r;
      }
    if (D == 3) {
      const int r = ensure_cart3(c);
      if (r != NS_OK) return r;
    }
    c->cart_pending = true;
  }
  bool face = false;
  double* dev = nullptr;
  if (D == 3) dev = field_ptr3d(c, field, comp, &face);
  else dev = (field == NS_FIELD_CART) ? c->CART[comp] : field_ptr(c, field, comp, &face);
  if (!dev) return fail(c, NS_ERR_ARG, "box copy: unknown field");
  int ext[3];
  for (int d = 0; d < 3; ++d) ext[d] = (d < D) ? c->N + ((face && comp == d) ? 1 : 0) : 1;
  for (int d = 0; d < 3; ++d)
    if (lo[d] < 0 || hi[d] >= ext[d] || hi[d] < lo[d]) return fail(c, NS_ERR_ARG, "box copy: index box outside the field");
  const long long wcells = hi[0] - lo[0] + 1, hrows = hi[1] - lo[1] + 1, nplanes = hi[2] - lo[2] + 1;
  if (jstride < wcells) return fail(c, NS_ERR_ARG, "box copy: jstride smaller than the box width");
  if (nplanes > 1 && kstride < jstride * hrows) return fail(c, NS_ERR_ARG, "box copy: kstride smaller than a box plane");
  const size_t w = (size_t)wcells * sizeof(double);
  const long P = c->pitch;
  const long plane = (long)P * (c->N + 1);  // 3D: (i, j, k) at (k (N + 1) + j) P + i
  const cudaMemcpyKind kind = where_device ? cudaMemcpyDeviceToDevice : (put ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
  for (long long k = 0; k < nplanes; ++k) {
    double* d = dev + (D == 3 ? (long)(lo[2] + k) * plane : 0) + (long)lo[1] * P + lo[0];
    double* h = data + k * kstride;
    cudaError_t e = put ? cudaMemcpy2DAsync(d, P * sizeof(double), h, (size_t)jstride * sizeof(double), w, (size_t)hrows, kind, c->st)
                        : cudaMemcpy2DAsync(h, (size_t)jstride * sizeof(double), d, P * sizeof(double), w, (size_t)hrows, kind, c->st);
    int r = cuda_check(c, e, "box copy");
    if (r != NS_OK) return r;
  }
  return NS_OK;
}

int ns_put_box(ns_ctx* c, int field, int comp, const double* data, const int lo[3], const int hi[3], long long jstride,
               long long kstride, int where_device) {
  int r = box_copy(c, field, comp, const_cast<double*>(data), lo, hi, jstride, kstride, where_device, true);
  if (r == NS_OK && !where_device) r = ns_sync(c);  // the caller may reuse its buffer on return
  return r;
}

int ns_get_box(ns_ctx* c, int field, int comp, double* data, const int lo[3], const int hi[3], long long jstride,
               long long kstride, int where_device) {
  int r = box_copy(c, field, comp, data, lo, hi, jstride, kstride, where_device, false);
  if (r == NS_OK) r = ns_sync(c);
  return r;
}

// the copies and resets of ns_set_state, enqueued without waiting (2D)
static int set_state_async(ns_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time,
                           bool keep_warm = false) {
  const int N = c->N;
  for (int m = 0; m < 2; ++m) {
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {N - 1 + (m == 0), N - 1 + (m == 1), 0};
    const long long js = N + (m == 0);
    int r = box_copy(c, NS_FIELD_VEL, m, const_cast<double*>(u[m]), lo, hi, js, 0, 0, true);
    if (r == NS_OK) r = box_copy(c, NS_FIELD_VEL_PREV, m, const_cast<double*>(u_prev[m]), lo, hi, js, 0, 0, true);
    if (r != NS_OK) return r;
  }
  const int lo[3] = {0, 0, 0}, hi[3] = {N - 1, N - 1, 0};
  int r = box_copy(c, NS_FIELD_PRESSURE, 0, const_cast<double*>(p), lo, hi, N, 0, 0, true);
  if (r != NS_OK) return r;
  for (int m = 0; m < 2; ++m) CK(cudaMemsetAsync(c->PHI[m], 0, c->fbytes, c->st), "memset phi");
  c->time = time;
  c->in_step = false;
  c->cart_pending = false;
  if (!keep_warm) c->pf_warm = -1;  // no previous phi for a warm start
  return NS_OK;
}

int ns_set_state(ns_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time) {
  if (!c || !u || !u_prev || !p) return NS_ERR_ARG;
  if (c->P.dim == 3) return set_state3d(c, u, u_prev, p, time);
  const int r = set_state_async(c, u, u_prev, p, time);
  return r != NS_OK ? r : ns_sync(c);
}

// the copies of ns_get_state, enqueued without waiting (2D)
static int get_state_async(ns_ctx* c, double* const* u, double* const* u_prev, double* p, double* phi) {
  const int N = c->N;
  for (int m = 0; m < 2; ++m) {
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {N - 1 + (m == 0), N - 1 + (m == 1), 0};
    const long long js = N + (m == 0);
    if (u && u[m]) { int r = box_copy(c, NS_FIELD_VEL, m, u[m], lo, hi, js, 0, 0, false); if (r) return r; }
    if (u_prev && u_prev[m]) { int r = box_copy(c, NS_FIELD_VEL_PREV, m, u_prev[m], lo, hi, js, 0, 0, false); if (r) return r; }
  }
  const int lo[3] = {0, 0, 0}, hi[3] = {N - 1, N - 1, 0};
  if (p) { int r = box_copy(c, NS_FIELD_PRESSURE, 0, p, lo, hi, N, 0, 0, false); if (r) return r; }
  if (phi) { int r = box_copy(c, NS_FIELD_PHI, 0, phi, lo, hi, N, 0, 0, false); if (r) return r; }
  return NS_OK;
}

int ns_get_state(ns_ctx* c, double* const* u, double* const* u_prev, double* p, double* phi) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return get_state3d(c, u, u_prev, p, phi);
  const int r = get_state_async(c, u, u_prev, p, phi);
  return r != NS_OK ? r : ns_sync(c);
}

int ns_init_fields(ns_ctx* c, int init_case) {
  if (!c || (init_case != NS_INIT_CAVITY && init_case != NS_INIT_TGV)) return NS_ERR_ARG;
  if (c->P.dim == 3) {
    // hybrid_grid_init of the AMREX_SPACEDIM = 3 build (fn_init.cpp:61-229,
    // kn_init.H:8-37): the cavity from rest, or the Taylor-Green case that
    // the source edit selects. Its z factors are commented out, so it is the
    // 2D vortex in every z plane: u = sin x cos y, v = -cos x sin y, w = 0,
    // u^{n-1} decayed by exp(-2 nu (t - dt)) with nu = 1 (1/Re with
    // fix_quirks), p = (cos 2x + cos 2y) / 4, and the cell velocity set
    // analytically (w = 0) for the first stage.
    const size_t N = c->N, nf = (N + 1) * N * N, nc = N * N * N;
    const double* lo = c->P.prob_lo;
    const double dx = c->g.dx[0], dy = c->g.dx[1], dt = c->dt, t0 = 0.0;
    const double nu_decay = c->P.fix_quirks ? 1.0 / c->P.ren : 1.0;
    const bool tgv = init_case == NS_INIT_TGV;
    const double decay = std::exp(-2.0 * nu_decay * (t0 - dt));
    std::vector<double> u(nf, 0.0), v(nf, 0.0), w(nf, 0.0), up(nf, 0.0), vp(nf, 0.0);
    std::vector<double> p(nc, 0.0), cu(nc, 0.0), cv(nc, 0.0), cw(nc, 0.0);
    for (size_t k = 0; k < N && tgv; ++k) {
      for (size_t j = 0; j < N; ++j)
        for (size_t i = 0; i <= N; ++i) {  // x faces (i, j + 1/2)
          const double x = lo[0] + (i + 0.0) * dx, y = lo[1] + (j + 0.5) * dy;
          u[(k * N + j) * (N + 1) + i] = std::sin(x) * std::cos(y);
          up[(k * N + j) * (N + 1) + i] = std::sin(x) * std::cos(y) * decay;
        }
      for (size_t j = 0; j <= N; ++j)
        for (size_t i = 0; i < N; ++i) {  // y faces (i + 1/2, j)
          const double x = lo[0] + (i + 0.5) * dx, y = lo[1] + (j + 0.0) * dy;
          v[(k * (N + 1) + j) * N + i] = -std::cos(x) * std::sin(y);
          vp[(k * (N + 1) + j) * N + i] = -std::cos(x) * std::sin(y) * decay;
        }
      for (size_t j = 0; j < N; ++j)
        for (size_t i = 0; i < N; ++i) {
          const double x = lo[0] + (i + 0.5) * dx, y = lo[1] + (j + 0.5) * dy;
          const size_t id = (k * N + j) * N + i;
          cu[id] = std::sin(x) * std::cos(y);
          cv[id] = -std::cos(x) * std::sin(y);
          p[id] = 0.25 * (std::cos(2.0 * x) + std::cos(2.0 * y));
        }
    }
    const double* u3[3] = {u.data(), v.data(), w.data()};
    const double* up3[3] = {up.data(), vp.data(), w.data()};
    int r = ns_set_state(c, u3, up3, p.data(), 0.0);
    if (r != NS_OK) return r;
    c->step = 0;
    if (!tgv) return NS_OK;
    const int l0[3] = {0, 0, 0}, h0[3] = {(int)N - 1, (int)N - 1, (int)N - 1};
    const double* cc[3] = {cu.data(), cv.data(), cw.data()};
    for (int m = 0; m < 3 && r == NS_OK; ++m)
      r = ns_put_box(c, NS_FIELD_CART, m, cc[m], l0, h0, (long long)N, (long long)(N * N), 0);
    return r;
  }
  // hybrid_grid_init (fn_init.cpp:61-229, kn_init.H:8-37), evaluated on the
  // host with the C library's sin/cos/exp and uploaded.
  const int N = c->N;
  const double* lo = c->P.prob_lo;
  const double dx = c->g.dx[0], dy = c->g.dx[1], dt = c->dt, t0 = 0.0;
  const double nu_decay = c->P.fix_quirks ? 1.0 / c->P.ren : 1.0;  // the reference hard-codes nu = 1
  std::vector<double> u((size_t)(N + 1) * N), v((size_t)N * (N + 1)), up(u.size()), vp(v.size());
  std::vector<double> p((size_t)N * N, 0.0), cu((size_t)N * N, 0.0), cv((size_t)N * N, 0.0);
  const bool tgv = init_case == NS_INIT_TGV;
  for (int j = 0; j < N; ++j)
    for (int i = 0; i <= N; ++i) {
      const double x = lo[0] + (i + 0.0) * dx, y = lo[1] + (j + 0.5) * dy;
      u[(size_t)j * (N + 1) + i] = tgv ? std::sin(x) * std::cos(y) : 0.0;
      up[(size_t)j * (N + 1) + i] = tgv ? std::sin(x) * std::cos(y) * std::exp(-2.0 * nu_decay * (t0 - dt)) : 0.0;
    }
  for (int j = 0; j <= N; ++j)
    for (int i = 0; i < N; ++i) {
      const double x = lo[0] + (i + 0.5) * dx, y = lo[1] + (j + 0.0) * dy;
      v[(size_t)j * N + i] = tgv ? -std::cos(x) * std::sin(y) : 0.0;
      vp[(size_t)j * N + i] = tgv ? -std::cos(x) * std::sin(y) * std::exp(-2.0 * nu_decay * (t0 - dt)) : 0.0;
    }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      const double x = lo[0] + (i + 0.5) * dx, y = lo[1] + (j + 0.5) * dy;
      if (tgv) {
        cu[(size_t)j * N + i] = std::sin(x) * std::cos(y);
        cv[(size_t)j * N + i] = -std::cos(x) * std::sin(y);
        p[(size_t)j * N + i] = 0.25 * (std::cos(2.0 * x) + std::cos(2.0 * y));
      }
    }
  const double* uu[2] = {u.data(), v.data()};
  const double* uup[2] = {up.data(), vp.data()};
  int r = ns_set_state(c, uu, uup, p.data(), 0.0);
  if (r != NS_OK) return r;
  c->step = 0;
  // the reference sets velCart analytically at init (not by cont2cart)
  const int l0[3] = {0, 0, 0}, h0[3] = {N - 1, N - 1, 0};
  r = ns_put_box(c, NS_FIELD_CART, 0, cu.data(), l0, h0, N, 0, 0);
  if (r == NS_OK) r = ns_put_box(c, NS_FIELD_CART, 1, cv.data(), l0, h0, N, 0, 0);
  return r;
}

// ---- building blocks --------------------------------------------------------

int ns_step_begin(ns_ctx* c) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return step_begin3d(c);
  ProjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  for (int m = 0; m < 2; ++m) {
    a.u[m] = c->U[m];
    a.uprev[m] = c->UP[m];
    a.du[m] = c->DU[m];
    a.S[m] = c->S[m];
  }
  a.p = c->Pp;
  LAUNCH(NS_PROF_STEP_BEGIN, "step_begin",
         (c->P.precision == NS_PREC_FP64_EXACT) ? launch_step_begin_exact(a, c->st) : launch_step_begin_fast(a, c->st));
  // velContPrev <- velCont, velStar <- velCont: the old u^{n-1} buffer becomes
  // the target of the projection
  for (int m = 0; m < 2; ++m) std::swap(c->U[m], c->UP[m]);
  c->base = -1;
  c->cur = -1;
  c->time += c->dt;
  c->in_step = true;
  c->norm_ready = false;
  c->mix_pending = false;
  c->base_ff_valid = false;
  c->s_ff_valid = false;
  return NS_OK;
}

// convective_flux_calc_quick: its cell convective term is formed first, into
// CONV, and the stage reads it (stage2d.cuh)
static int launch_conv_alt(ns_ctx* c, StageArgs& a) {
  if (c->P.conv_scheme != NS_CONV_QUICK) return NS_OK;
  for (int m = 0; m < 2; ++m) a.conv[m] = c->CONV[m];
  LAUNCH(NS_PROF_OTHER, "convective_flux_calc_quick", launch_conv_quick_exact(a, c->st));
  return NS_OK;
}

static int launch_rk(ns_ctx* c, int sub, bool use_cart) {
  const int in = c->cur;
  const int outb = pick_out(c->base, in);
  StageArgs a = base_stage_args(c);
  for (int m = 0; m < 2; ++m) {
    a.us[m] = face_ptr(c, in, m);
    a.ub[m] = face_ptr(c, c->base, m);
    a.out[m] = c->B[outb][m];
    a.cart[m] = use_cart ? c->CART[m] : nullptr;
  }
  a.rk = c->rk[sub];
  a.do_norm = (sub == 3);
  int rc = launch_conv_alt(c, a);
  if (rc != NS_OK) return rc;
  const int mode = (c->P.precision == NS_PREC_FP64_EXACT) ? kExactRK : kFastRK;
  LAUNCH(mode == kExactRK ? NS_PROF_STAGE_EXACT : NS_PROF_STAGE_FAST, "rk stage",
         (mode == kExactRK) ? launch_stage_exact(mode, a, c->st) : launch_stage_fast(mode, a, c->st));
  c->cur = outb;
  return NS_OK;
}

int ns_rk_stage(ns_ctx* c, int sub) {
  if (!c || sub < 0 || sub > 3) return NS_ERR_ARG;
  if (!c->in_step) return fail(c, NS_ERR_STATE, "ns_rk_stage before ns_step_begin");
  if (c->P.dim == 3) return rk_stage3d(c, sub);
  const bool use_cart = c->cart_pending;
  int r = launch_rk(c, sub, use_cart);
  if (r == NS_OK && use_cart) c->cart_pending = false;
  if (r == NS_OK && sub == 3) c->norm_ready = true;
  return r;
}

int ns_pseudo_norm(ns_ctx* c, double* norm) {
  if (!c) return NS_ERR_ARG;
  if (!c->norm_ready) return fail(c, NS_ERR_STATE, "ns_pseudo_norm needs stage 3 first");
  if (c->P.dim == 3) return pseudo_norm3d(c, norm);
  int r = sync_red(c, kRedNorm, 1);
  if (r != NS_OK) return r;
  if (norm) *norm = c->red_h[kRedNorm];
  c->base = c->cur;  // velCont <- velStar (main.cpp:1023-1026)
  c->norm_ready = false;
  return NS_OK;
}

int ns_explicit_predictor(ns_ctx* c, double* norm) {
  if (!c) return NS_ERR_ARG;
  if (!c->in_step) return fail(c, NS_ERR_STATE, "explicit predictor before ns_step_begin");
  if (c->P.dim == 3) return explicit_predictor3d(c, norm);
  const int in = c->cur;
  const int outb = pick_out(c->base, in);
  StageArgs a = base_stage_args(c);
  for (int m = 0; m < 2; ++m) {
    a.us[m] = face_ptr(c, in, m);
    a.ub[m] = face_ptr(c, c->base, m);
    a.out[m] = c->B[outb][m];
    a.cart[m] = c->cart_pending ? c->CART[m] : nullptr;
  }
  a.do_norm = 1;
  int rc = launch_conv_alt(c, a);
  if (rc != NS_OK) return rc;
  LAUNCH(NS_PROF_EXPLICIT, "explicit stage", launch_stage_exact(kExplicit, a, c->st));
  c->cart_pending = false;
  c->cur = outb;
  int r = sync_red(c, kRedNorm, 1);
  if (r != NS_OK) return r;
  if (norm) *norm = c->red_h[kRedNorm];
  c->base = c->cur;
  return NS_OK;
}

static int poisson_rhs_async(ns_ctx* c) {
  ProjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  for (int m = 0; m < 2; ++m) a.u[m] = face_ptr(c, c->cur, m);
  a.f = c->F;
  a.part = c->part;
  a.counter = c->counter;
  a.red_out = c->red + kRedDivBefore;  // {max|div|, sum}
  LAUNCH(NS_PROF_POISSON_RHS, "poisson rhs",
         (c->P.precision == NS_PREC_FP64_EXACT) ? launch_poisson_rhs_exact(a, c->st) : launch_poisson_rhs_fast(a, c->st));
  return NS_OK;
}

int ns_poisson_rhs(ns_ctx* c, double* divmax, double* sum) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return poisson_rhs3d(c, divmax, sum);
  int r = poisson_rhs_async(c);
  if (r == NS_OK) r = sync_red(c, kRedDivBefore, 2);
  if (r != NS_OK) return r;
  if (divmax) *divmax = c->red_h[kRedDivBefore];
  if (sum) *sum = c->red_h[kRedSum];
  // max|f| = (1.5/dt) max|div u*| (the same rounding), the zero-guess
  // residual of a warm-started mixed solve
  c->rhs_fmax = c->g.c15 * c->red_h[kRedDivBefore];
  c->rhs_fmax_valid = true;
  return NS_OK;
}

}  // extern "C"

template <typename T>
static int vcycle(ns_ctx* c, MGLevels<T>& M, int x0_zero) {
  // each smoother launch reads x[l] and writes x2[l]; the swap after it makes
  // the result x[l] again. Two launches per level: the buffers are back in
  // place when the cycle ends.
  for (int l = 0; l < c->lb; ++l) {
    LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg smooth", launch_mg_smooth<T>(M, l, 0, (l > 0) ? 1 : x0_zero, c->st));
    std::swap(M.x[l], M.x2[l]);
    LAUNCH(l == 0 ? NS_PROF_MG_RESTRICT0 : NS_PROF_MG_RESTRICT, "mg restrict", launch_mg_restrict<T>(M, l, c->st));
  }
  LAUNCH(NS_PROF_MG_BOTTOM, "mg bottom", launch_mg_bottom<T>(M, c->lb, (c->lb > 0) ? 1 : x0_zero, c->st));
  for (int l = c->lb - 1; l >= 0; --l) {
    LAUNCH(l == 0 ? NS_PROF_MG_SMOOTH0 : NS_PROF_MG_SMOOTH, "mg prolong+smooth", launch_mg_smooth<T>(M, l, 1, 0, c->st));
    std::swap(M.x[l], M.x2[l]);
  }
  return NS_OK;
}

// One V-cycle, replayed from a CUDA graph captured on first use: the ~22
// launches of a cycle become one graph launch. The smoother's buffer swaps
// leave every level's pointers as they were, so the captured arguments stay
// valid; the graph is rebuilt when the level-0 buffers change (the FP64
// hierarchy's level 0 is the caller's phi). If the stream cannot be captured
// (the legacy default stream), the cycle runs as plain launches.
template <typename T>
static int vcycle_graph(ns_ctx* c, MGLevels<T>& M, int x0_zero) {
  ns_ctx::VGraph& G = c->vg[sizeof(T) == 8 ? 1 : 0][x0_zero ? 1 : 0];
  if (G.unusable) return vcycle<T>(c, M, x0_zero);
  const void* key[4] = {M.x[0], M.x2[0], M.f[0], M.fmean};
  if (G.exec && std::memcmp(key, G.key, sizeof(key)) != 0) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  if (!G.exec) {
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      G.unusable = true;
      return vcycle<T>(c, M, x0_zero);
    }
    const long long l0 = c->launches;
    const bool prof = c->prof;
    c->prof = false;  // no event nodes inside the graph
    const int r = vcycle<T>(c, M, x0_zero);
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
  c->launches += G.nlaunch - 1;  // the kernels of the graph, as the library's launch count
  return NS_OK;
}

// mean of f (singular problem, AMReX makes the RHS solvable) written to red[kRedMean]
__global__ void k_set_mean(double* red, double inv_n) { red[kRedMean] = red[kRedSum] * inv_n; }

// ---- GMRES option (GMRES_Poisson.cpp:56-131) -----------------------------------
// Restarted GMRES on L phi = f - mean(f) with one FP64 V-cycle as the right
// preconditioner (a fixed linear map: the correction is M^-1 (V y), one more
// V-cycle per restart, so only the basis V is stored). Classical Gram-Schmidt
// with one re-orthogonalisation pass, Givens rotations on the host. The
// iteration stops on the same max-norm residual test as the V-cycle solver.
static int gmres_alloc(ns_ctx* c, int m) {
  if ((int)c->gm_v.size() >= m + 1) return NS_OK;
  for (int k = (int)c->gm_v.size(); k < m + 1; ++k) {
    double* v = nullptr;
    if (alloc_field(c, &v) != NS_OK) return NS_ERR_NOMEM;
    c->gm_v.push_back(v);
  }
  if (!c->gm_w) {
    if (alloc_field(c, &c->gm_w) != NS_OK || alloc_field(c, &c->gm_z) != NS_OK || alloc_field(c, &c->gm_b) != NS_OK)
      return NS_ERR_NOMEM;
    if (cudaMalloc(&c->gm_part, (size_t)kGmMaxV * kGmBlocks * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->gm_dev, 2 * kGmMaxV * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&c->gm_host, 2 * kGmMaxV * sizeof(double)) != cudaSuccess)
      return fail(c, NS_ERR_NOMEM, "cudaMalloc (GMRES) failed");
  }
  return NS_OK;
}

static int gmres_precond(ns_ctx* c, const double* in, double* out) {
  double* x0 = c->M64.x[0];
  double* f0 = c->M64.f[0];
  const double* fm = c->M64.fmean;
  c->M64.x[0] = out;
  c->M64.f[0] = const_cast<double*>(in);
  c->M64.fmean = nullptr;
  const int r = vcycle<double>(c, c->M64, 1);
  c->M64.x[0] = x0;
  c->M64.f[0] = f0;
  c->M64.fmean = fm;
  return r;
}

// the cells of the context's fields for the GMRES vector kernels
static GmGrid gm_grid(const ns_ctx* c) {
  GmGrid G;
  G.n = c->N;
  G.P = c->pitch;
  G.nz = c->P.dim == 3 ? c->N : 1;
  G.PL = (long)c->pitch * (c->N + 1);
  return G;
}

// out[k] = (w, V[k]) for k < nv, read back to c->gm_host
static int gmres_dots(ns_ctx* c, const std::vector<double*>& V, int nv, const double* w) {
  GmVecs vv;
  std::memset(&vv, 0, sizeof(vv));
  for (int k = 0; k < nv; ++k) vv.v[k] = V[k];
  LAUNCH(NS_PROF_OTHER, "gmres dots", launch_gm_mdot(gm_grid(c), nv, vv, w, c->gm_part, c->counter, c->gm_dev, c->st));
  CK(cudaMemcpyAsync(c->gm_host, c->gm_dev, nv * sizeof(double), cudaMemcpyDeviceToHost, c->st), "readback");
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

// w += s * sum_k coef[k] V[k] (coef from the host)
static int gmres_update(ns_ctx* c, const std::vector<double*>& V, int nv, const double* coef, double s, double* w) {
  GmVecs vv;
  std::memset(&vv, 0, sizeof(vv));
  for (int k = 0; k < nv; ++k) vv.v[k] = V[k];
  CK(cudaMemcpyAsync(c->gm_dev + kGmMaxV, coef, nv * sizeof(double), cudaMemcpyHostToDevice, c->st), "coefficients");
  LAUNCH(NS_PROF_OTHER, "gmres update", launch_gm_maxpy(gm_grid(c), nv, vv, c->gm_dev + kGmMaxV, s, w, c->st));
  // the next host write of the coefficients must wait for this kernel
  CK(cudaStreamSynchronize(c->st), "stream sync");
  return NS_OK;
}

// Restarted GMRES(m) with one FP64 V-cycle as right preconditioner on
// L phi = f - mean f from phi = 0, stopped on the multigrid's max-norm test.
// 2D and 3D: the operator, the preconditioner and the residual test are the
// context's own; the Krylov vectors are whole fields.
int nsh::poisson_gmres(ns_ctx* c, double tol_rel, double div_tol_res, int maxc, int* cycles, double* rnorm0_out,
                       double* rn_out) {
  const int m = std::max(2, std::min(c->P.gmres_restart, kGmMaxV - 1));
  int r = gmres_alloc(c, m);
  if (r != NS_OK) return r;
  const bool d3 = c->P.dim == 3;
  const GmGrid G = gm_grid(c);
  const int N = c->N;
  const long P = c->pitch;
  const int px = c->g.periodic[0], py = c->g.periodic[1], pz = c->g.periodic[2];
  double ih[3] = {c->M64.invh2[0][0], c->M64.invh2[0][1], 0.0};
  double* x = c->PHI[0];
  const double* F = c->F;
  if (d3) {
    gm3_fields(c, &x, &F, ih);
  } else {
    c->phi_cur = 0;
    c->M64.x[0] = c->PHI[0];
  }
  std::vector<double*>& V = c->gm_v;
  auto apply = [&](const double* in, double* out) -> int {
    if (d3) LAUNCH(NS_PROF_OTHER, "gmres apply", launch_gm_lap3(G, px, py, pz, ih[0], ih[1], ih[2], in, out, c->st));
    else LAUNCH(NS_PROF_OTHER, "gmres apply", launch_gm_lap(N, P, px, py, ih[0], ih[1], in, out, c->st));
    return NS_OK;
  };
  auto precond = [&](const double* in, double* out) -> int {
    return d3 ? gm3_precond(c, in, out) : gmres_precond(c, in, out);
  };
  auto resnorm = [&]() -> int {
    if (d3) r = gm3_resnorm(c);
    else {
      LAUNCH(NS_PROF_MG_RESNORM, "resnorm", launch_mg_resnorm<double>(c->M64, c->part, c->counter, c->red + kRedRes, c->st));
      r = NS_OK;
    }
    return r != NS_OK ? r : sync_red(c, kRedRes, 1);
  };
  // b = f - mean(f); x = 0 (poisson.cpp:63)
  LAUNCH(NS_PROF_OTHER, "gmres rhs", launch_gm_axpby(G, 1.0, F, 0.0, nullptr, c->red + kRedMean, -1.0, c->gm_b, c->st));
  CK(cudaMemsetAsync(x, 0, c->fbytes, c->st), "memset phi");
  r = resnorm();
  if (r != NS_OK) return r;
  const double rnorm0 = c->red_h[kRedRes];
  double rn = rnorm0;
  *rnorm0_out = rnorm0;
  const double tol = tol_rel * rnorm0;
  auto done = [&](double v) { return v <= tol && (div_tol_res <= 0 || v <= div_tol_res); };
  int its = 0;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  auto h = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
  while (!done(rn) && rnorm0 > 0 && its < maxc) {
    // r0 = b - L x into V[0]; beta = |r0|
    r = apply(x, c->gm_w);
    if (r != NS_OK) return r;
    LAUNCH(NS_PROF_OTHER, "gmres r0", launch_gm_axpby(G, 1.0, c->gm_b, -1.0, c->gm_w, nullptr, 0.0, V[0], c->st));
    r = gmres_dots(c, V, 1, V[0]);
    if (r != NS_OK) return r;
    const double beta = std::sqrt(c->gm_host[0]);
    if (!(beta > 0)) break;
    LAUNCH(NS_PROF_OTHER, "gmres scale", launch_gm_axpby(G, 1.0 / beta, V[0], 0.0, nullptr, nullptr, 0.0, V[0], c->st));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (int j = 0; j < m && its < maxc; ++j) {
      ++its;
      r = precond(V[j], c->gm_z);
      if (r == NS_OK) r = apply(c->gm_z, c->gm_w);
      if (r != NS_OK) return r;
      for (int i = 0; i <= j; ++i) h(i, j) = 0.0;
      for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, twice
        r = gmres_dots(c, V, j + 1, c->gm_w);
        if (r == NS_OK) r = gmres_update(c, V, j + 1, c->gm_host, -1.0, c->gm_w);
        if (r != NS_OK) return r;
        for (int i = 0; i <= j; ++i) h(i, j) += c->gm_host[i];
      }
      std::vector<double*> wv(1, c->gm_w);
      r = gmres_dots(c, wv, 1, c->gm_w);
      if (r != NS_OK) return r;
      const double hn = std::sqrt(c->gm_host[0]);
      // Givens rotations of column j
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * h(i, j) + sn[i] * h(i + 1, j);
        h(i + 1, j) = -sn[i] * h(i, j) + cs[i] * h(i + 1, j);
        h(i, j) = t;
      }
      const double den = std::hypot(h(j, j), hn);
      cs[j] = den > 0 ? h(j, j) / den : 1.0;
      sn[j] = den > 0 ? hn / den : 0.0;
      h(j, j) = den;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      k = j + 1;
      if (hn > 0 && j + 1 < m)
        LAUNCH(NS_PROF_OTHER, "gmres scale",
               launch_gm_axpby(G, 1.0 / hn, c->gm_w, 0.0, nullptr, nullptr, 0.0, V[j + 1], c->st));
      // the 2-norm estimate |g[j+1]| against the max-norm target (|r|_inf <= |r|_2)
      if (std::fabs(g[j + 1]) <= 0.5 * tol || hn == 0) break;
    }
    // y = H^-1 g; x += M^-1 (V y)
    for (int i = k - 1; i >= 0; --i) {
      double t = g[i];
      for (int l = i + 1; l < k; ++l) t -= h(i, l) * y[l];
      y[i] = h(i, i) != 0 ? t / h(i, i) : 0.0;
    }
    CK(cudaMemsetAsync(c->gm_w, 0, c->fbytes, c->st), "memset");
    r = gmres_update(c, V, k, y.data(), 1.0, c->gm_w);
    if (r == NS_OK) r = precond(c->gm_w, c->gm_z);
    if (r == NS_OK) LAUNCH(NS_PROF_OTHER, "gmres x", launch_gm_axpby(G, 1.0, x, 1.0, c->gm_z, nullptr, 0.0, x, c->st));
    if (r != NS_OK) return r;
    // the true max-norm residual of the multigrid test
    r = resnorm();
    if (r != NS_OK) return r;
    rn = c->red_h[kRedRes];
  }
  *cycles = its;
  *rn_out = rn;
  return done(rn) || rnorm0 == 0 ? NS_OK : NS_ERR_MG_STALL;
}

extern "C" {

static int alloc_mixed(ns_ctx* c);
static void split_const(double x, float* out);

int ns_poisson_solve(ns_ctx* c, int precision, int* cycles, double* res) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return poisson_solve3d(c, precision, cycles, res);
  const double nn = (double)c->N * (double)c->N;
  LAUNCH(NS_PROF_OTHER, "set mean", (k_set_mean<<<1, 1, 0, c->st>>>(c->red, 1.0 / nn), cudaGetLastError()));
  const int maxc = std::max(1, c->P.poisson_max_cycles);
  const double div_tol_res = c->P.poisson_tol_div > 0 ? c->P.poisson_tol_div * 1.5 / c->dt : 0.0;
  double rnorm0 = 0.0, rn = 0.0;
  int ncyc = 0;
  int status = NS_OK;
  if (c->P.poisson_solver == 1) {
    status = nsh::poisson_gmres(c, c->P.poisson_tol_rel, div_tol_res, maxc, &ncyc, &rnorm0, &rn);
    if (status != NS_OK && status != NS_ERR_MG_STALL) return status;
  } else if (precision == NS_PREC_MIXED) {
    // FP32 V-cycles inside an FP64 defect correction
    DCArgs d;
    std::memset(&d, 0, sizeof(d));
    d.n = c->N;
    d.pitch = c->pitch;
    d.periodic[0] = c->g.periodic[0];
    d.periodic[1] = c->g.periodic[1];
    d.invh2[0] = c->M64.invh2[0][0];
    d.invh2[1] = c->M64.invh2[0][1];
    d.f = c->F;
    d.fmean = c->red + kRedMean;
    d.part = c->part;
    d.counter = c->counter;
    d.red_out = c->red + kRedRes;
    d.e = c->M32.x[0];
    d.r32 = c->M32.f[0];
    // phi is carried in float-float (PFF) while the residual can still fall;
    // if it stalls above the tolerance the sweeps continue with the FP64
    // residual kernel.
    int r = alloc_mixed(c);
    if (r != NS_OK) return r;
    DCffArgs q;
    std::memset(&q, 0, sizeof(q));
    q.n = c->N;
    q.pitch = c->pitch;
    q.periodic[0] = c->g.periodic[0];
    q.periodic[1] = c->g.periodic[1];
    for (int d2 = 0; d2 < 2; ++d2) split_const(c->M64.invh2[0][d2], q.ih[d2]);
    q.e = c->M32.x[0];
    q.r32 = c->M32.f[0];
    q.f[0] = c->FFh;
    q.f[1] = c->FFl;
    q.part = c->part;
    q.counter = c->counter;
    q.red_out = c->red + kRedRes;
    const bool ff_start = c->P.dc_residual == 0;
    int pf = 0;
    int pc = 0;
    // warm start: the defect correction starts from the previous step's
    // float-float phi (a zero correction added to it), with the tolerance
    // relative to the zero-guess residual max|f - mean f|
    const bool warm = ff_start && c->P.poisson_warm_start && c->pf_warm >= 0 && c->rhs_fmax_valid && c->rhs_fmax > 0;
    if (ff_start) {
      LAUNCH(NS_PROF_OTHER, "rhs split", launch_rhs_ff(c->N, c->pitch, c->F, c->red + kRedMean, c->FFh, c->FFl, c->st));
      if (warm) {
        CK(cudaMemsetAsync(c->M32.x[0], 0, (size_t)c->pitch * (c->N + 1) * sizeof(float), c->st), "memset e");
        q.first = 0;
        q.phin[0] = c->PFh[c->pf_warm]; q.phin[1] = c->PFl[c->pf_warm];
        q.phout[0] = c->PFh[1 - c->pf_warm]; q.phout[1] = c->PFl[1 - c->pf_warm];
        pf = 1 - c->pf_warm;
      } else {
        q.first = 1;
        q.phin[0] = c->PFh[0]; q.phin[1] = c->PFl[0];
        q.phout[0] = c->PFh[0]; q.phout[1] = c->PFl[0];
      }
      LAUNCH(NS_PROF_DC_UPDATE, "dc update", launch_dc_update_ff(q, c->st));
    } else {
      // FP64 phi and residual from the first sweep: phi = 0, r = f - mean f
      d.first = 1;
      d.phi_in = c->PHI[0];
      d.phi_out = c->PHI[0];
      LAUNCH(NS_PROF_DC_UPDATE, "dc update", launch_dc_update(d, c->st));
    }
    r = sync_red(c, kRedRes, 1);
    if (r != NS_OK) return r;
    rn = c->red_h[kRedRes];
    rnorm0 = warm ? c->rhs_fmax : rn;
    c->rhs_fmax_valid = false;
    const double tol = std::max(c->P.poisson_tol_rel * rnorm0, 0.0);
    auto done = [&](double x) { return x <= tol && (div_tol_res <= 0 || x <= div_tol_res); };
    double best = rn;
    int stall = 0;
    bool ffmode = ff_start;
    while (!done(rn) && rnorm0 > 0) {
      if (ncyc >= maxc) { status = NS_ERR_MG_STALL; break; }
      int r2 = vcycle_graph<float>(c, c->M32, 1);
      if (r2 != NS_OK) return r2;
      if (ffmode) {
        q.first = 0;
        q.phin[0] = c->PFh[pf]; q.phin[1] = c->PFl[pf];
        q.phout[0] = c->PFh[1 - pf]; q.phout[1] = c->PFl[1 - pf];
        LAUNCH(NS_PROF_DC_UPDATE, "dc update", launch_dc_update_ff(q, c->st));
        pf = 1 - pf;
      } else {
        d.first = 0;
        d.phi_in = c->PHI[pc];
        d.phi_out = c->PHI[1 - pc];
        LAUNCH(NS_PROF_DC_UPDATE, "dc update", launch_dc_update(d, c->st));
        pc = 1 - pc;
      }
      ++ncyc;
      r2 = sync_red(c, kRedRes, 1);
      if (r2 != NS_OK) return r2;
      rn = c->red_h[kRedRes];
      if (rn < 0.5 * best) {
        best = rn;
        stall = 0;
      } else if (++stall >= (ffmode ? 2 : 6)) {
        if (!ffmode) { status = NS_ERR_MG_STALL; break; }
        // float-float floor reached: continue from the FP64 phi
        LAUNCH(NS_PROF_OTHER, "phi to fp64", launch_ff_to_double(c->N, c->pitch, c->PFh[pf], c->PFl[pf], c->PHI[0], c->st));
        ffmode = false;
        pc = 0;
        stall = 0;
        c->dc_fallbacks++;
      }
    }
    if (ffmode)
      LAUNCH(NS_PROF_OTHER, "phi to fp64", launch_ff_to_double(c->N, c->pitch, c->PFh[pf], c->PFl[pf], c->PHI[0], c->st));
    c->phi_cur = ffmode ? 0 : pc;
    c->pf_warm = (ffmode && status == NS_OK) ? pf : -1;
  } else {
    c->phi_cur = 0;
    c->M64.x[0] = c->PHI[0];
    // the step's solve starts from zero (poisson.cpp:63); the adjoint's solves
    // start from the previous step's solution with the tolerance relative to |f|
    const bool warm = c->phi_guess != nullptr;
    if (warm)
      CK(cudaMemcpyAsync(c->PHI[0], c->phi_guess, c->fbytes, cudaMemcpyDeviceToDevice, c->st), "phi guess");
    else
      CK(cudaMemsetAsync(c->PHI[0], 0, c->fbytes, c->st), "memset phi");
    LAUNCH(NS_PROF_MG_RESNORM, "resnorm", launch_mg_resnorm<double>(c->M64, c->part, c->counter, c->red + kRedRes, c->st));
    int r = sync_red(c, kRedRes, c->tol_from_f ? kRedF - kRedRes + 1 : 1);
    if (r != NS_OK) return r;
    rnorm0 = c->red_h[kRedRes];
    rn = rnorm0;
    if (c->tol_from_f) rnorm0 = std::max(rnorm0, c->red_h[kRedF]);
    const double tol = c->P.poisson_tol_rel * rnorm0;
    auto done = [&](double x) { return x <= tol && (div_tol_res <= 0 || x <= div_tol_res); };
    double best = rn;
    int stall = 0;
    while (!done(rn) && rnorm0 > 0) {
      if (ncyc >= maxc) { status = NS_ERR_MG_STALL; break; }
      int r2 = vcycle_graph<double>(c, c->M64, (ncyc == 0 && !warm) ? 1 : 0);
      if (r2 != NS_OK) return r2;
      ++ncyc;
      LAUNCH(NS_PROF_MG_RESNORM, "resnorm", launch_mg_resnorm<double>(c->M64, c->part, c->counter, c->red + kRedRes, c->st));
      r2 = sync_red(c, kRedRes, 1);
      if (r2 != NS_OK) return r2;
      rn = c->red_h[kRedRes];
      if (rn < 0.5 * best) { best = rn; stall = 0; } else if (++stall >= 6) { status = NS_ERR_MG_STALL; break; }
    }
  }
  if (cycles) *cycles = ncyc;
  if (res) *res = rnorm0 > 0 ? rn / rnorm0 : 0.0;
  if (status != NS_OK) c->err = "Poisson residual stalled before the tolerance";
  return status;
}

static int project_async(ns_ctx* c) {
  ProjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = c->g;
  for (int m = 0; m < 2; ++m) {
    a.u[m] = face_ptr(c, c->cur, m);
    a.uout[m] = c->U[m];
  }
  a.p = c->Pp;
  a.pw = c->Pp;
  a.phi = c->PHI[c->phi_cur];
  a.part = c->part;
  a.counter = c->counter;
  a.red_out = c->red + kRedDivAfter;
  LAUNCH(NS_PROF_PROJECT, "project",
         (c->P.precision == NS_PREC_FP64_EXACT) ? launch_project_exact(a, c->st) : launch_project_fast(a, c->st));
  return NS_OK;
}

int ns_project(ns_ctx* c, double* divmax) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return project3d(c, divmax);
  int r = project_async(c);
  if (r == NS_OK) r = sync_red(c, kRedDivAfter, 1);
  if (r != NS_OK) return r;
  if (divmax) *divmax = c->red_h[kRedDivAfter];
  c->in_step = false;
  return NS_OK;
}

static void split_const(double x, float* out) {
  out[0] = (float)x;
  out[1] = (float)(x - (double)out[0]);
}

// One pseudo-iteration of the mixed-precision predictor: the anchor stage
// evaluates G(u_base) in float-float arithmetic (after adding the pending
// increment of the previous iteration), then three FP32 increment stages; the
// fourth stage's increment e4 stays in E[0] and its norm is the
// pseudo-increment norm of Error_Computation.
// the anchor is evaluated exactly (float-float) on the first iteration, at
// most kAnchorEvery iterations after the last exact one, and once the
// pseudo-norm has fallen below kAnchorDrop times its value after the last
// exact one; the others update it by an FP32 increment evaluation. Each
// update rounds the stored G0 to FP32, an error relative to |G0| at that
// iteration; the errors add up until the next exact anchor and shift the
// converged u* by their sum over 1.5/dt, so the refresh on a falling norm
// keeps that sum within a small multiple of the final norm however few
// iterations the step takes.
// (4096^2 cavity: a cap of 16 gives 5 exact anchors a step, 32 gives 3 and
// 0.8% more steps/s.)
constexpr int kAnchorEvery = 32;
constexpr double kAnchorDrop = 1e-2;

static int mixed_iteration(ns_ctx* c, double* norm) {
  if (!c->s_ff_valid) {
    const double* S[2] = {c->S[0], c->S[1]};
    LAUNCH(NS_PROF_OTHER, "split S", launch_split_ff(c->g, S, c->SFh, c->SFl, c->st));
    c->s_ff_valid = true;
  }
  if (!c->base_ff_valid) {
    const double* B[2] = {face_ptr(c, c->base, 0), face_ptr(c, c->base, 1)};
    LAUNCH(NS_PROF_OTHER, "split base", launch_split_ff(c->g, B, c->BH[0], c->BL[0], c->st));
    c->mb = 0;
    c->base_ff_valid = true;
    c->mix_pending = false;
  }
  const bool exact = !c->mix_pending || c->mix_it - c->mix_last_exact >= kAnchorEvery ||
                     !(c->mix_norm >= kAnchorDrop * c->mix_norm_exact);
  if (exact) c->mix_last_exact = c->mix_it;
  ++c->mix_it;
  if (exact) {
    AnchorFFArgs a;
    std::memset(&a, 0, sizeof(a));
    a.g = c->g;
    const int mb = c->mb, nb = 1 - c->mb;
    for (int m = 0; m < 2; ++m) {
      a.bh[m] = c->BH[mb][m];
      a.bl[m] = c->BL[mb][m];
      a.e4[m] = c->mix_pending ? c->E[0][m] : nullptr;
      a.Sh[m] = c->SFh[m];
      a.Sl[m] = c->SFl[m];
      a.obh[m] = c->BH[nb][m];
      a.obl[m] = c->BL[nb][m];
      a.g0[m] = c->G0[m];
      split_const(c->g.inv_dx[m], a.inv_dx[m]);
      split_const(1.0 / (c->g.ren * c->g.dx2[m]), a.vcoef[m]);
    }
    split_const(c->g.c15, a.c15);
    LAUNCH(NS_PROF_ANCHOR, "anchor stage", launch_anchor_ff(a, c->st));
    c->mb = nb;
  } else {
    // incremental anchor: G0 + dG(u_b; e4) by the FP32 increment kernel with
    // rk = 1 (its rounding error is relative to e4); the same launch writes
    // u_b + e4 in float-float to the other base buffer. The exact float-float
    // anchor of the next kAnchorEvery-th iteration removes whatever these
    // updates accumulated
    const int mb = c->mb, nb = 1 - c->mb;
    IncArgs u;
    std::memset(&u, 0, sizeof(u));
    u.g = c->g;
    u.part = reinterpret_cast<float2*>(c->part);
    u.counter = c->counter;
    u.norm_out = c->red + kRedNorm;
    for (int m = 0; m < 2; ++m) {
      u.sh[m] = c->BH[mb][m];
      u.g0[m] = c->G0[m];
      u.ein[m] = c->E[0][m];
      u.eout[m] = c->G0b[m];
      u.bl[m] = c->BL[mb][m];
      u.obh[m] = c->BH[nb][m];
      u.obl[m] = c->BL[nb][m];
      u.inv_dx[m] = (float)c->g.inv_dx[m];
      u.vcoef[m] = (float)(1.0 / (c->g.ren * c->g.dx2[m]));
    }
    u.c15 = (float)c->g.c15;
    u.rk_prev = 1.f;
    u.rk = 1.f;
    u.do_norm = 0;
    LAUNCH(NS_PROF_INC, "anchor update", launch_inc_stage(u, c->st));
    for (int m = 0; m < 2; ++m) std::swap(c->G0[m], c->G0b[m]);
    c->mb = nb;
  }
  const int nb = c->mb;  // the base of this iteration's increment stages
  IncArgs ia;
  std::memset(&ia, 0, sizeof(ia));
  ia.g = c->g;
  ia.part = reinterpret_cast<float2*>(c->part);
  ia.counter = c->counter;
  ia.norm_out = c->red + kRedNorm;
  for (int m = 0; m < 2; ++m) {
    ia.sh[m] = c->BH[nb][m];  // the hi part is the FP32 copy of u_base
    ia.g0[m] = c->G0[m];
    ia.inv_dx[m] = (float)c->g.inv_dx[m];
    ia.vcoef[m] = (float)(1.0 / (c->g.ren * c->g.dx2[m]));
  }
  ia.c15 = (float)c->g.c15;
  for (int s = 1; s <= 3; ++s) {
    const int src = (s == 2) ? 0 : 1, dst = (s == 2) ? 1 : 0;
    for (int m = 0; m < 2; ++m) {
      ia.ein[m] = (s == 1) ? nullptr : c->E[src][m];
      ia.eout[m] = c->E[dst][m];
    }
    ia.rk_prev = (float)c->rk[s - 1];
    ia.rk = (float)c->rk[s];
    ia.do_norm = (s == 3);
    if (s == 3 && c->note_d != nullptr) {
      c->note_seq += 1.0;
      ia.note = c->note_d;
      ia.note_seq = c->note_seq;
    }
    LAUNCH(NS_PROF_INC, "increment stage", launch_inc_stage(ia, c->st));
  }
  c->mix_pending = true;
  if (!read_note(c, norm)) {  // no mapped note, or it did not arrive in time
    int r = sync_red(c, kRedNorm, 1);
    if (r != NS_OK) return r;
    *norm = c->red_h[kRedNorm];
  }
  c->mix_norm = *norm;
  if (exact) c->mix_norm_exact = *norm;
  return NS_OK;
}

// u* = u_base + e4 once the mixed iteration stops
static int mixed_finalize(ns_ctx* c) {
  if (!c->base_ff_valid) return NS_OK;
  const int outb = pick_out(c->base, c->base);
  const float* h[2] = {c->BH[c->mb][0], c->BH[c->mb][1]};
  const float* l[2] = {c->BL[c->mb][0], c->BL[c->mb][1]};
  const float* e[2] = {c->mix_pending ? c->E[0][0] : nullptr, c->mix_pending ? c->E[0][1] : nullptr};
  double* out[2] = {c->B[outb][0], c->B[outb][1]};
  LAUNCH(NS_PROF_OTHER, "add increment", launch_ff_add_inc(c->g, h, l, e, out, c->st));
  c->base = outb;
  c->cur = outb;
  c->mix_pending = false;
  c->base_ff_valid = false;
  return NS_OK;
}

static int alloc_mixed(ns_ctx* c) {
  if (c->G0[0]) return NS_OK;
  const size_t fb = (size_t)c->pitch * (c->N + 1) * sizeof(float);
  for (int m = 0; m < 2; ++m) {
    float** ps[13] = {&c->G0[m], &c->G0b[m], &c->E[0][m], &c->E[1][m], &c->BH[0][m], &c->BH[1][m], &c->BL[0][m],
                      &c->BL[1][m], &c->SFh[m], &c->SFl[m], &c->PFh[m], &c->PFl[m], m == 0 ? &c->FFh : &c->FFl};
    for (float** p : ps) {
      if (cudaMalloc(p, fb) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc (mixed) failed");
      CK(cudaMemsetAsync(*p, 0, fb, c->st), "memset");
    }
  }
  return NS_OK;
}

}  // extern "C"

int nsh::run_predictor(ns_ctx* c, ns_step_stats* sp) {
  ns_step_stats& s = *sp;
  const bool mixed = (c->P.precision == NS_PREC_MIXED) && c->P.pseudo_timestepping != 0;
  if (mixed) {
    int ra = alloc_mixed(c);
    if (ra != NS_OK) return ra;
  }
  c->mix_pending = false;
  c->mix_it = 0;
  c->mix_last_exact = 0;
  int r = ns_step_begin(c);
  if (r != NS_OK) return r;
  if (c->early_uprev) {
    // ns_step_host: the new u^{n-1} (UP, the step's input u^n) goes back to
    // the host on the side stream while the predictor runs
    CK(cudaEventRecord(c->side_ev[0], c->st), "event");
    CK(cudaStreamWaitEvent(c->side, c->side_ev[0], 0), "stream wait");
    const int N = c->N;
    for (int m = 0; m < 2; ++m) {
      const size_t w = (size_t)(N + (m == 0)) * sizeof(double), h = (size_t)(N + (m == 1));
      CK(cudaMemcpy2DAsync(c->early_uprev[m], w, c->UP[m], c->pitch * sizeof(double), w, h, cudaMemcpyDeviceToHost,
                           c->side),
         "u_prev copy");
    }
    CK(cudaEventRecord(c->side_ev[1], c->side), "event");
    c->early_uprev = nullptr;
  }
  int countIter = 0;
  double normError = 1.e9;
  while (normError > c->P.momentum_tolerance) {
    if (c->P.pseudo_timestepping == 0) {
      r = ns_explicit_predictor(c, &normError);
      if (r != NS_OK) return r;
      countIter = 1;
      break;
    }
    if (mixed && !c->cart_pending) {
      // the analytic first-stage cell velocity of an initial condition is
      // only consumed by the FP64 stages, so the first iteration after
      // ns_init_fields(TGV) runs in FP64
      r = mixed_iteration(c, &normError);
      if (r != NS_OK) return r;
    } else {
      for (int sub = 0; sub < 4; ++sub) {
        r = ns_rk_stage(c, sub);
        if (r != NS_OK) return r;
      }
      r = ns_pseudo_norm(c, &normError);
      if (r != NS_OK) return r;
    }
    countIter++;
    if (std::isnan(normError)) {
      c->in_step = false;
      return fail(c, NS_ERR_NONFINITE, "pseudo-increment norm is NaN (non-finite fields)");
    }
    if (countIter > c->P.iter_num) { s.status = NS_WARN_PSEUDO_MAXITER; break; }
    if (normError > 1.e2) { s.status = NS_WARN_PSEUDO_DIVERGED; break; }
  }
  s.pseudo_iters = countIter;
  s.norm_error = normError;
  return mixed_finalize(c);
}

extern "C" {

int ns_step(ns_ctx* c, ns_step_stats* stats) {
  if (!c) return NS_ERR_ARG;
  if (c->P.dim == 3) return step3d(c, stats);
  ns_step_stats s;
  std::memset(&s, 0, sizeof(s));
  if (c->ev_ok) cudaEventRecord(c->ev[0], c->st);
  int r = run_predictor(c, &s);
  if (r != NS_OK) return r;
  if (c->ev_ok) cudaEventRecord(c->ev[1], c->st);
  r = ns_poisson_rhs(c, &s.div_before, &s.rhs_sum);
  if (r != NS_OK) return r;
  if (!std::isfinite(s.div_before) || !std::isfinite(s.rhs_sum)) {
    c->in_step = false;
    return fail(c, NS_ERR_NONFINITE, "Poisson right-hand side is not finite");
  }
  const int prec = (c->P.precision == NS_PREC_MIXED) ? NS_PREC_MIXED : NS_PREC_FP64;
  const long long fb0 = c->dc_fallbacks;
  r = ns_poisson_solve(c, prec, &s.poisson_cycles, &s.poisson_res);
  s.poisson_fp64_fallback = (int)(c->dc_fallbacks - fb0);
  if (r != NS_OK && r != NS_ERR_MG_STALL) return r;
  const int mg_status = r;
  if (c->ev_ok) cudaEventRecord(c->ev[2], c->st);
  r = ns_project(c, &s.div_after);
  if (r != NS_OK) return r;
  c->step++;
  if (c->ev_ok) {
    cudaEventRecord(c->ev[3], c->st);
    cudaEventSynchronize(c->ev[3]);
    float a = 0, b = 0, d = 0;
    cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&d, c->ev[2], c->ev[3]);
    s.ms_predictor = a; s.ms_poisson = b; s.ms_project = d;
  }
  if (stats) *stats = s;
  if (mg_status != NS_OK) return mg_status;
  return s.status;
}

int ns_get_cell_velocity(ns_ctx* c, double* const* cart) {
  if (!c || !cart) return NS_ERR_ARG;
  if (c->in_step) return fail(c, NS_ERR_STATE, "cell velocity inside a step");
  const int D = c->P.dim;
  for (int d = 0; d < D; ++d)
    if (!cart[d]) return NS_ERR_ARG;
  if (!c->cell_tmp) {
    if (cudaMalloc(&c->cell_tmp, c->fbytes) != cudaSuccess) return fail(c, NS_ERR_NOMEM, "cudaMalloc failed");
  }
  const int N = c->N;
  const long plane = D == 3 ? (long)c->pitch * (N + 1) : 0;
  for (int d = 0; d < D; ++d) {
    bool face = false;
    const double* u = D == 3 ? field_ptr3d(c, NS_FIELD_VEL, d, &face) : c->U[d];
    LAUNCH(NS_PROF_OTHER, "cell velocity", launch_cell_velocity(u, c->cell_tmp, N, c->pitch, plane, d, D, c->st));
    // the dense host copy: N planes (3D) of N rows of N values
    for (int k = 0; k < (D == 3 ? N : 1); ++k)
      CK(cudaMemcpy2DAsync(cart[d] + (size_t)k * N * N, (size_t)N * sizeof(double), c->cell_tmp + k * plane,
                           (size_t)c->pitch * sizeof(double), (size_t)N * sizeof(double), (size_t)N,
                           cudaMemcpyDeviceToHost, c->st),
         "cell velocity copy");
  }
  return ns_sync(c);
}

int ns_checkpoint_get(ns_ctx* c, double* const* u, double* const* u_prev, double* p, double* time, long long* step) {
  if (!c || !u || !u_prev || !p) return NS_ERR_ARG;
  if (c->in_step) return fail(c, NS_ERR_STATE, "checkpoint inside a step");
  const int r = ns_get_state(c, u, u_prev, p, nullptr);
  if (r != NS_OK) return r;
  if (time) *time = c->time;
  if (step) *step = c->step;
  return NS_OK;
}

int ns_checkpoint_put(ns_ctx* c, const double* const* u, const double* const* u_prev, const double* p, double time,
                      long long step) {
  if (!c || step < 0) return NS_ERR_ARG;
  const int r = ns_set_state(c, u, u_prev, p, time);
  if (r != NS_OK) return r;
  c->step = step;
  return NS_OK;
}

long long ns_get_step(const ns_ctx* c) { return c ? c->step : -1; }

// The copies in and out are enqueued on the context's stream with the step
// between them: nothing waits for the upload (the step's kernels follow it in
// stream order), and one synchronisation ends the call. CUDA events around
// the two copy phases give ms_h2d and ms_d2h.
int ns_step_host(ns_ctx* c, double* const* u, double* const* u_prev, double* p, ns_step_stats* stats) {
  if (!c || !u || !u_prev || !p) return NS_ERR_ARG;
  const double t = c->time;
  const bool two_d = c->P.dim == 2;
  // 2D: the outgoing u_prev (the incoming u, which the step leaves in place)
  // is copied back on a side stream while the step runs
  bool overlap = false;
  if (two_d) {
    if (!c->side) {
      if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) c->side = nullptr;
      for (auto& e : c->side_ev)
        if (c->side && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) e = nullptr;
    }
    overlap = c->side && c->side_ev[0] && c->side_ev[1];
  }
  if (c->ev_ok) cudaEventRecord(c->ev[4], c->st);
  // a warm-started mixed solve keeps the previous step's phi as its initial
  // guess: it meets the same tolerance whatever state the host uploads
  int r = two_d ? set_state_async(c, u, u_prev, p, t, true) : ns_set_state(c, u, u_prev, p, t);
  if (r != NS_OK) return r;
  if (c->ev_ok) cudaEventRecord(c->ev[5], c->st);
  ns_step_stats s;
  std::memset(&s, 0, sizeof(s));
  c->early_uprev = overlap ? u_prev : nullptr;
  const int st = ns_step(c, &s);
  c->early_uprev = nullptr;
  if (overlap) {
    // the side copy was enqueued after step begin: wait for it on the host
    // (also on the error path, before the caller may reuse u_prev)
    const cudaError_t e = cudaEventSynchronize(c->side_ev[1]);
    if (st >= 0 && e != cudaSuccess) return cuda_check(c, e, "u_prev copy");
  }
  if (st < 0) {
    if (stats) *stats = s;
    return st;
  }
  if (c->ev_ok) cudaEventRecord(c->ev[6], c->st);
  r = two_d ? get_state_async(c, u, overlap ? nullptr : u_prev, p, nullptr) : ns_get_state(c, u, u_prev, p, nullptr);
  if (r != NS_OK) return r;
  if (c->ev_ok) cudaEventRecord(c->ev[7], c->st);
  r = ns_sync(c);
  if (r != NS_OK) return r;
  if (c->ev_ok) {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, c->ev[4], c->ev[5]);
    cudaEventElapsedTime(&b, c->ev[6], c->ev[7]);
    s.ms_h2d = a;
    s.ms_d2h = b;
  }
  if (stats) *stats = s;
  return st;
}

}  // extern "C"

extern "C" {

// The per-launch event pairs are resolved only here, in ns_profile_read and
// when nsh::kProfPending launches are pending, never at the per-iteration
// syncs of the step (the stream would idle while the host reads them). The
// pool is filled when profiling is switched on, outside any timed region.
int ns_profile_enable(ns_ctx* c, int on) {
  if (!c) return NS_ERR_ARG;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  prof_resolve(c);
  c->prof = on != 0;
  if (c->prof) {
    while (c->evpool.size() < (size_t)nsh::kProfPool) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e), "event create");
      c->evpool.push_back(e);
    }
  }
  return NS_OK;
}

int ns_profile_read(ns_ctx* c, double* ms, long long* counts, int nkinds, int reset) {
  if (!c || nkinds < 0) return NS_ERR_ARG;
  CK(cudaStreamSynchronize(c->st), "stream sync");
  prof_resolve(c);
  for (int k = 0; k < nkinds && k < NS_PROF_KINDS; ++k) {
    if (ms) ms[k] = c->pms[k];
    if (counts) counts[k] = c->pcnt[k];
  }
  if (reset)
    for (int k = 0; k < NS_PROF_KINDS; ++k) { c->pms[k] = 0.0; c->pcnt[k] = 0; }
  return NS_OK;
}

long long ns_launch_count(const ns_ctx* c) { return c ? c->launches : -1; }

int ns_bounds_check_read(ns_ctx* c, unsigned long long* status, int reset) {
  if (!c || !status) return NS_ERR_ARG;
#ifdef NS_BOUNDS_CHECK
  CK(cudaStreamSynchronize(c->st), "stream sync");
  unsigned long long h[3] = {0, 0, 0};
  CK(cudaMemcpy(h, c->check, sizeof(h), cudaMemcpyDeviceToHost), "status read");
  for (int k = 0; k < 3; ++k) status[k] = h[k];
  if (reset) CK(cudaMemset(c->check, 0, sizeof(h)), "status reset");
  return NS_OK;
#else
  status[0] = status[1] = status[2] = 0;
  return NS_ERR_UNSUPPORTED;
#endif
}

void* ns_host_alloc(unsigned long long bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) return nullptr;
  return p;
}

void ns_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

}  // extern "C"
