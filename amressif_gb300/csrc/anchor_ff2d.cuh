// Anchor stage of the mixed-precision pseudo-iteration in float-float
// arithmetic (2D).
//
// Same stencil as k_stage2d (cont2cart + ghosts, QUICK half-node fluxes,
// viscous term, flux ghost rule, face RHS; main.cpp:931-1017) evaluated at
// u_base = base + e4 with ~48-bit float-float numbers on the FP32 pipes, so
// that G(u_base) = S - (1.5/dt) u_base + avg(-conv + visc) keeps FP64-class
// accuracy although its terms cancel to the pseudo-residual. The base itself
// is stored as two float arrays (hi, lo); hi doubles as the FP32 copy read by
// the increment stages. Thread mapping as in k_inc_stage2d (flattened rectangles).
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
  static constexpr int UW = TX + 7, UH = TY + 6;
  static constexpr int VW = TX + 6, VH = TY + 7;
  static constexpr int CW = TX + 6, CH = TY + 6;
  static constexpr int FXW = TX + 3, FXH = TY + 2;
  static constexpr int FYW = TX + 2, FYH = TY + 3;
  static constexpr int TW = TX + 2, TH = TY + 2;
  union {
    struct {
      ff u[UH][UW];
      ff v[VH][VW];
    } f;
    ff t[2][TH][TW];  // totals reuse the face tiles once the fluxes exist
  };
  ff c[2][CH][CW];
  ff fx[2][FXH][FXW];
  ff fy[2][FYH][FYW];
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
    const ff q = (ff_scale2(-e - ff_scale2(c, 2.f) + 3.f * b, 0.125f)) + c;
    return u * q;
  } else if (u.hi < 0.f) {
    const ff q = (ff_scale2(-a - ff_scale2(b, 2.f) + 3.f * c, 0.125f)) + b;
    return u * q;
  }
  return ff_make(0.f, 0.f);
}

__device__ __forceinline__ ff cart_ghost_ff(const CartBC& b, int m, ff q) {
  const int r = b.rule[m];
  if (r == kInlet) return ff_from_double(b.add[m]) - q;
  return r == kNeg ? -q : q;
}

template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_anchor_ff2d(AnchorFFArgs A) {
  using SM = AnchorSmem<TX, TY>;
  extern __shared__ __align__(16) unsigned char anchor_smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(anchor_smem_raw);
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const bool perx = g.periodic[0], pery = g.periodic[1];
  const ff zero = ff_make(0.f, 0.f);

  // ---- 0. face tiles of u_base = base + e4 ----------------------------------
  NS_RECT_LOOP(SM::UW, SM::UH, NT, r, c) {
    int b = y0 - 3 + r;
    if (b < 0 || b >= N) b = pery ? wrapi(b, N) : -1;
    int a = x0 - 3 + c;
    if (a < 0 || a > N) a = perx ? wrapi(a, N) : -1;
    sm.f.u[r][c] = (b >= 0 && a >= 0) ? anchor_u(A, 0, (long)b * P + a) : zero;
  }
  NS_RECT_LOOP(SM::VW, SM::VH, NT, r, c) {
    int b = y0 - 3 + r;
    if (b < 0 || b > N) b = pery ? wrapi(b, N) : -1;
    int a = x0 - 3 + c;
    if (a < 0 || a >= N) a = perx ? wrapi(a, N) : -1;
    sm.f.v[r][c] = (b >= 0 && a >= 0) ? anchor_u(A, 1, (long)b * P + a) : zero;
  }
  __syncthreads();

  // ---- 1. cell-centred velocity + wall / lid ghosts ---------------------------
  NS_RECT_LOOP(SM::CW, SM::CH, NT, r, c) {
      sm.c[0][r][c] = ff_scale2(sm.f.u[r][c] + sm.f.u[r][c + 1], 0.5f);
      sm.c[1][r][c] = ff_scale2(sm.f.v[r][c] + sm.f.v[r + 1][c], 0.5f);
    }
  __syncthreads();
  const bool lox = !perx && x0 == 0, hix = !perx && x0 + TX + 3 > N;
  const bool loy = !pery && y0 == 0, hiy = !pery && y0 + TY + 3 > N;
  if (lox || hix) {
    for (int q = threadIdx.x; q < 6 * SM::CH; q += NT) {
      const int r = q / 6, k = q - 6 * (q / 6);
      const int b = y0 - 3 + r;
      if (!pery && (b < 0 || b >= N)) continue;
      int c, cm, side;
      if (k < 3) { if (!lox) continue; c = k; cm = 5 - k; side = 0; }
      else {
        if (!hix) continue;
        const int a = N + (k - 3);
        c = a - (x0 - 3);
        if (c >= SM::CW) continue;
        cm = (2 * N - 1 - a) - (x0 - 3);
        side = 1;
      }
      for (int m = 0; m < 2; ++m) sm.c[m][r][c] = cart_ghost_ff(g.bc[side], m, sm.c[m][r][cm]);
    }
    __syncthreads();
  }
  if (loy || hiy) {
    for (int q = threadIdx.x; q < 6 * SM::CW; q += NT) {
      const int k = q / SM::CW, c = q - k * SM::CW;
      int r, rm, side;
      if (k < 3) { if (!loy) continue; r = k; rm = 5 - k; side = 2; }
      else {
        if (!hiy) continue;
        const int b = N + (k - 3);
        r = b - (y0 - 3);
        if (r >= SM::CH) continue;
        rm = (2 * N - 1 - b) - (y0 - 3);
        side = 3;
      }
      for (int m = 0; m < 2; ++m) {
        if (side == 3 && m == 0 && g.lid_u != nullptr && g.bc[3].rule[0] == kInlet) {
          int a = x0 - 3 + c;
          a = a < 0 ? 0 : (a >= N ? N - 1 : a);
          sm.c[m][r][c] = ff_from_double(2 * g.lid_u[a]) - sm.c[m][rm][c];
        } else {
          sm.c[m][r][c] = cart_ghost_ff(g.bc[side], m, sm.c[m][rm][c]);
        }
      }
    }
    __syncthreads();
  }

  // ---- 2. QUICK half-node fluxes -------------------------------------------------
  NS_RECT_LOOP(SM::FXW, SM::FXH, NT, fr, fc) {
      const ff u = sm.f.u[fr + 2][fc + 2];
#pragma unroll
      for (int m = 0; m < 2; ++m)
        sm.fx[m][fr][fc] = quick_flux_ff(u, sm.c[m][fr + 2][fc + 3], sm.c[m][fr + 2][fc + 2], sm.c[m][fr + 2][fc + 1],
                                         sm.c[m][fr + 2][fc]);
    }
  NS_RECT_LOOP(SM::FYW, SM::FYH, NT, fr, fc) {
      const ff v = sm.f.v[fr + 2][fc + 2];
#pragma unroll
      for (int m = 0; m < 2; ++m)
        sm.fy[m][fr][fc] = quick_flux_ff(v, sm.c[m][fr + 3][fc + 2], sm.c[m][fr + 2][fc + 2], sm.c[m][fr + 1][fc + 2],
                                         sm.c[m][fr][fc + 2]);
    }
  __syncthreads();

  // ---- 3. total = -conv + visc (the face tiles are dead: t reuses them) ------------
  const ff idx_ = ff_make(A.inv_dx[0][0], A.inv_dx[0][1]), idy_ = ff_make(A.inv_dx[1][0], A.inv_dx[1][1]);
  const ff vx = ff_make(A.vcoef[0][0], A.vcoef[0][1]), vy = ff_make(A.vcoef[1][0], A.vcoef[1][1]);
  NS_RECT_LOOP(SM::TW, SM::TH, NT, tr, tc) {
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const ff conv = (sm.fx[m][tr][tc + 1] - sm.fx[m][tr][tc]) * idx_ + (sm.fy[m][tr + 1][tc] - sm.fy[m][tr][tc]) * idy_;
        const ff c2 = ff_scale2(sm.c[m][tr + 2][tc + 2], 2.f);
        const ff visc = (sm.c[m][tr + 2][tc + 3] - c2 + sm.c[m][tr + 2][tc + 1]) * vx +
                        (sm.c[m][tr + 3][tc + 2] - c2 + sm.c[m][tr + 1][tc + 2]) * vy;
        sm.t[m][tr][tc] = visc - conv;
      }
    }
  __syncthreads();
  const bool wrapx = g.flux_ghost[0] == kWrap, wrapy = g.flux_ghost[1] == kWrap;
  if ((x0 == 0 || x0 + TX >= N) && !wrapx) {
    for (int tr = threadIdx.x; tr < SM::TH; tr += NT) {
      if (x0 == 0) sm.t[0][tr][0] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][tr][1] : zero;
      const int tc = N - (x0 - 1);
      if (x0 + TX >= N && tc < SM::TW) sm.t[0][tr][tc] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][tr][tc - 1] : zero;
    }
  }
  if ((y0 == 0 || y0 + TY >= N) && !wrapy) {
    for (int tc = threadIdx.x; tc < SM::TW; tc += NT) {
      if (y0 == 0) sm.t[1][0][tc] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][1][tc] : zero;
      const int tr = N - (y0 - 1);
      if (y0 + TY >= N && tr < SM::TH) sm.t[1][tr][tc] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][tr - 1][tc] : zero;
    }
  }
  __syncthreads();

  // ---- 4. G(u_base) at the faces of the tile -----------------------------------------
  const ff c15 = ff_make(A.c15[0], A.c15[1]);
  auto face = [&](int m, int a, int b) {
    const int tc = a - (x0 - 1), tr = b - (y0 - 1);
    const long id = (long)b * P + a;
    const ff tm = (m == 0) ? sm.t[0][tr][tc - 1] : sm.t[1][tr - 1][tc];
    const ff tc_ = sm.t[m][tr][tc];
    const ff u = anchor_u(A, m, id);
    const ff G = (ff_make(A.Sh[m][id], A.Sl[m][id]) - c15 * u) + ff_scale2(tm + tc_, 0.5f);
    A.obh[m][id] = u.hi;
    A.obl[m][id] = u.lo;
    A.g0[m][id] = G.hi + G.lo;
  };
  NS_RECT_LOOP(TX, TY, NT, k, l) {
    const int a = x0 + l, b = y0 + k;
    if (a < N && b < N) { face(0, a, b); face(1, a, b); }
  }
  if (x0 + TX >= N && N > x0)
    for (int k = threadIdx.x; k < TY; k += NT)
      if (y0 + k < N) face(0, N, y0 + k);
  if (y0 + TY >= N && N > y0)
    for (int k = threadIdx.x; k < TX; k += NT)
      if (x0 + k < N) face(1, x0 + k, N);
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
