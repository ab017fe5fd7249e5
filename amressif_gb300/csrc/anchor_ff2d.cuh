// Anchor stage of the mixed-precision pseudo-iteration in float-float
// arithmetic (2D).
//
// Same stencil as k_stage2d (cont2cart + ghosts, QUICK half-node fluxes,
// viscous term, flux ghost rule, face RHS; main.cpp:931-1017) evaluated at
// u_base = base + e4 with ~48-bit float-float numbers on the FP32 pipes, so
// that G(u_base) = S - (1.5/dt) u_base + avg(-conv + visc) keeps FP64-class
// accuracy although its terms cancel to the pseudo-residual. The base itself
// is stored as two float arrays (hi, lo); hi doubles as the FP32 copy read by
// the increment stages.
#pragma once
#include "ff.cuh"
#include "ns_common.cuh"

namespace ns {

struct AnchorFFArgs {
  Geom g;
  const float* bh[2];   // base, hi part (faces)
  const float* bl[2];   // base, lo part
  const float* e4[2];   // pending increment (nullable)
  const float* Sh[2];   // step-constant source S, hi / lo
  const float* Sl[2];
  float* obh[2];        // new base hi / lo
  float* obl[2];
  float* g0[2];         // G(u_base) rounded to FP32
  // constants as float-float (hi, lo) pairs
  float inv_dx[2][2], vcoef[2][2], c15[2];
};

template <int TX, int TY>
struct AnchorSmem {
  static constexpr int CW = TX + 6, CH = TY + 6;
  static constexpr int FXW = TX + 3, FXH = TY + 2;
  static constexpr int FYW = TX + 2, FYH = TY + 3;
  static constexpr int TW = TX + 2, TH = TY + 2;
  ff c[2][CH][CW];
  ff fx[2][FXH][FXW];
  ff fy[2][FYH][FYW];
  ff t[2][TH][TW];
};

__device__ __forceinline__ ff anchor_u(const AnchorFFArgs& A, int m, long id) {
  ff u = ff_make(A.bh[m][id], A.bl[m][id]);
  if (A.e4[m] != nullptr) u = ff_add_f(u, A.e4[m][id]);
  return u;
}

// QUICK flux (fn_flux_calc.cpp:66-76): u>0 -> u*Q_L, u<0 -> u*Q_R, where
// ud = ucon+|ucon| and up = ucon-|ucon| are exactly u or 0.
__device__ __forceinline__ ff quick_flux_ff(ff u, ff a, ff b, ff c, ff e) {
  if (u.hi > 0.f) {
    const ff q = (ff_scale2(ff_make(-e.hi, -e.lo) - ff_scale2(c, 2.f) + 3.f * b, 0.125f)) + c;
    return u * q;
  } else if (u.hi < 0.f) {
    const ff q = (ff_scale2(ff_make(-a.hi, -a.lo) - ff_scale2(b, 2.f) + 3.f * c, 0.125f)) + b;
    return u * q;
  }
  return ff_make(0.f, 0.f);
}

__device__ __forceinline__ ff cart_ghost_ff(const CartBC& b, int m, ff q) {
  const int r = b.rule[m];
  if (r == kInlet) return ff_from_double(b.add[m]) - q;
  return r == kNeg ? -q : q;
}

template <int TX, int TY>
__global__ void __launch_bounds__(256) k_anchor_ff2d(AnchorFFArgs A) {
  using SM = AnchorSmem<TX, TY>;
  __shared__ SM sm;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool perx = g.periodic[0], pery = g.periodic[1];

  for (int t = tid; t < SM::CW * SM::CH; t += NT) {
    const int lx = t % SM::CW, ly = t / SM::CW;
    const int a = x0 - 3 + lx, b = y0 - 3 + ly;
    const bool inx = (a >= 0 && a < N), iny = (b >= 0 && b < N);
    ff cu = ff_make(0.f, 0.f), cv = cu;
    if ((inx || perx) && (iny || pery)) {
      const long id = (long)wrapi(b, N) * P + wrapi(a, N);
      cu = ff_scale2(anchor_u(A, 0, id) + anchor_u(A, 0, id + 1), 0.5f);
      cv = ff_scale2(anchor_u(A, 1, id) + anchor_u(A, 1, id + P), 0.5f);
    }
    sm.c[0][ly][lx] = cu;
    sm.c[1][ly][lx] = cv;
  }
  __syncthreads();
  if (!perx) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int a = x0 - 3 + lx, b = y0 - 3 + ly;
      if (!(b >= 0 && b < N) && !pery) continue;
      if (a >= -3 && a < 0) {
        const int ml = (-a - 1) - (x0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost_ff(g.bc[0], m, sm.c[m][ly][ml]);
      } else if (a >= N && a < N + 3) {
        const int ml = (2 * N - 1 - a) - (x0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost_ff(g.bc[1], m, sm.c[m][ly][ml]);
      }
    }
    __syncthreads();
  }
  if (!pery) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int b = y0 - 3 + ly;
      if (b >= -3 && b < 0) {
        const int ml = (-b - 1) - (y0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost_ff(g.bc[2], m, sm.c[m][ml][lx]);
      } else if (b >= N && b < N + 3) {
        const int ml = (2 * N - 1 - b) - (y0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost_ff(g.bc[3], m, sm.c[m][ml][lx]);
      }
    }
    __syncthreads();
  }
  const bool wx = (g.flux_ghost[0] == kWrap), wy = (g.flux_ghost[1] == kWrap);

  for (int t = tid; t < SM::FXW * SM::FXH; t += NT) {
    const int fx = t % SM::FXW, fyy = t / SM::FXW;
    const int a = x0 - 1 + fx, b = y0 - 1 + fyy;
    const bool rowin = (b >= 0 && b < N);
    const bool facein = (a >= 0 && a <= N);
    const bool need_u = (fyy >= 1 && fyy <= TY) && rowin && (facein || wx);
    const bool need_v = (fx >= 1 && fx <= TX + 1) && (rowin || wy) && facein;
    if (!need_u && !need_v) continue;
    const int aa = facein ? a : wrapi(a, N);
    const ff ucf = anchor_u(A, 0, (long)wrapi(b, N) * P + aa);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      sm.fx[m][fyy][fx] = quick_flux_ff(ucf, sm.c[m][ly][lx + 1], sm.c[m][ly][lx], sm.c[m][ly][lx - 1], sm.c[m][ly][lx - 2]);
    }
  }
  for (int t = tid; t < SM::FYW * SM::FYH; t += NT) {
    const int fx = t % SM::FYW, fyy = t / SM::FYW;
    const int a = x0 - 1 + fx, b = y0 - 1 + fyy;
    const bool colin = (a >= 0 && a < N);
    const bool facein = (b >= 0 && b <= N);
    const bool need_u = (fyy >= 1 && fyy <= TY + 1) && (colin || wx) && facein;
    const bool need_v = (fx >= 1 && fx <= TX) && colin && (facein || wy);
    if (!need_u && !need_v) continue;
    const int bb = facein ? b : wrapi(b, N);
    const ff vcf = anchor_u(A, 1, (long)bb * P + wrapi(a, N));
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      sm.fy[m][fyy][fx] = quick_flux_ff(vcf, sm.c[m][ly + 1][lx], sm.c[m][ly][lx], sm.c[m][ly - 1][lx], sm.c[m][ly - 2][lx]);
    }
  }
  __syncthreads();

  const ff idx_ = ff_make(A.inv_dx[0][0], A.inv_dx[0][1]), idy_ = ff_make(A.inv_dx[1][0], A.inv_dx[1][1]);
  const ff vx = ff_make(A.vcoef[0][0], A.vcoef[0][1]), vy = ff_make(A.vcoef[1][0], A.vcoef[1][1]);
  for (int t = tid; t < SM::TW * SM::TH; t += NT) {
    const int tx = t % SM::TW, ty = t / SM::TW;
    const int a = x0 - 1 + tx, b = y0 - 1 + ty;
    const bool need_u = (ty >= 1 && ty <= TY) && (b < N) && ((a >= 0 && a < N) || wx);
    const bool need_v = (tx >= 1 && tx <= TX) && (a < N) && ((b >= 0 && b < N) || wy);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      const ff conv = (sm.fx[m][ty][tx + 1] - sm.fx[m][ty][tx]) * idx_ + (sm.fy[m][ty + 1][tx] - sm.fy[m][ty][tx]) * idy_;
      const ff c2 = ff_scale2(sm.c[m][ly][lx], 2.f);
      const ff visc = (sm.c[m][ly][lx + 1] - c2 + sm.c[m][ly][lx - 1]) * vx + (sm.c[m][ly + 1][lx] - c2 + sm.c[m][ly - 1][lx]) * vy;
      sm.t[m][ty][tx] = visc - conv;
    }
  }
  __syncthreads();
  if (tid < 2 * (TY + TX)) {
    if (tid < TY) {
      const int ty = tid + 1;
      if (x0 == 0 && !wx) sm.t[0][ty][0] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][1] : ff_make(0.f, 0.f);
    } else if (tid < 2 * TY) {
      const int ty = tid - TY + 1;
      const int tx = N - (x0 - 1);
      if (tx >= 1 && tx < SM::TW && !wx)
        sm.t[0][ty][tx] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][tx - 1] : ff_make(0.f, 0.f);
    } else if (tid < 2 * TY + TX) {
      const int tx = tid - 2 * TY + 1;
      if (y0 == 0 && !wy) sm.t[1][0][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][1][tx] : ff_make(0.f, 0.f);
    } else {
      const int tx = tid - 2 * TY - TX + 1;
      const int ty = N - (y0 - 1);
      if (ty >= 1 && ty < SM::TH && !wy)
        sm.t[1][ty][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][ty - 1][tx] : ff_make(0.f, 0.f);
    }
  }
  __syncthreads();

  const ff c15 = ff_make(A.c15[0], A.c15[1]);
  const int nfx = (x0 + TX >= N) ? (N - x0 + 1) : TX;
  const int nfy = (y0 + TY >= N) ? (N - y0 + 1) : TY;
  const int ncx = min(TX, N - x0), ncy = min(TY, N - y0);
  for (int t = tid; t < nfx * ncy + ncx * nfy; t += NT) {
    int m, a, b;
    if (t < nfx * ncy) { m = 0; a = x0 + t % nfx; b = y0 + t / nfx; }
    else { const int q = t - nfx * ncy; m = 1; a = x0 + q % ncx; b = y0 + q / ncx; }
    const long id = (long)b * P + a;
    const int tx = a - (x0 - 1), ty = b - (y0 - 1);
    const ff tm = (m == 0) ? sm.t[0][ty][tx - 1] : sm.t[1][ty - 1][tx];
    const ff tc = sm.t[m][ty][tx];
    const ff u = anchor_u(A, m, id);
    const ff G = (ff_make(A.Sh[m][id], A.Sl[m][id]) - c15 * u) + ff_scale2(tm + tc, 0.5f);
    A.obh[m][id] = u.hi;
    A.obl[m][id] = u.lo;
    A.g0[m][id] = G.hi + G.lo;
  }
}

// FP64 field -> float-float (hi, lo) arrays, integer split (no FP64 pipe)
static __global__ void __launch_bounds__(256) k_split_ff2d(Geom g, const double* x0, const double* x1, float* h0, float* l0,
                                                           float* h1, float* l1) {
  const int N = g.N;
  const long P = g.pitch;
  const long nu = (long)(N + 1) * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * nu; t += (long)gridDim.x * blockDim.x) {
    const int m = (t < nu) ? 0 : 1;
    const long q = (m == 0) ? t : t - nu;
    const int a = (m == 0) ? (int)(q % (N + 1)) : (int)(q % N);
    const int b = (m == 0) ? (int)(q / (N + 1)) : (int)(q / N);
    const long id = (long)b * P + a;
    const ff v = ff_from_double(m == 0 ? x0[id] : x1[id]);
    if (m == 0) { h0[id] = v.hi; l0[id] = v.lo; }
    else { h1[id] = v.hi; l1[id] = v.lo; }
  }
}

// u* = (hi + lo) + e (FP64) once the mixed iteration stops
static __global__ void __launch_bounds__(256) k_ff_add_inc2d(Geom g, const float* h0, const float* l0, const float* h1,
                                                             const float* l1, const float* e0, const float* e1, double* o0,
                                                             double* o1) {
  const int N = g.N;
  const long P = g.pitch;
  const long nu = (long)(N + 1) * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * nu; t += (long)gridDim.x * blockDim.x) {
    const int m = (t < nu) ? 0 : 1;
    const long q = (m == 0) ? t : t - nu;
    const int a = (m == 0) ? (int)(q % (N + 1)) : (int)(q % N);
    const int b = (m == 0) ? (int)(q / (N + 1)) : (int)(q / N);
    const long id = (long)b * P + a;
    if (m == 0) o0[id] = ((double)h0[id] + (double)l0[id]) + (e0 ? (double)e0[id] : 0.0);
    else o1[id] = ((double)h1[id] + (double)l1[id]) + (e1 ? (double)e1[id] : 0.0);
  }
}

}  // namespace ns
