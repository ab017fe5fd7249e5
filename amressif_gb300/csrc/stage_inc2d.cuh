// FP32 increment stages of the mixed-precision pseudo-time iteration (2D).
//
// The reference's RK pseudo-iteration (main.cpp:929-1026) evaluates, from a
// base u_b, the stages u*_{s+1} = u_b + rk[s] G(u*_s) with G the BDF2 residual
// of the QUICK + viscous momentum equation. Writing u*_s = u_b + e_s,
//   G(u_b + e_s) = G(u_b) + dG(u_b; e_s),
//   dG = -(1.5/dt) e_s + avg(-[conv(u_b+e_s) - conv(u_b)] + visc(e_s)).
// G(u_b) is evaluated once per iteration in FP64 (the anchor stage). dG only
// involves the small increment e_s: it is evaluated here in FP32 from an FP32
// copy of u_b, with the QUICK flux difference expanded so that no term
// subtracts two nearly equal FP32 numbers:
//   dF = dud * Q_L(phi) + ud' * Q_L(eps) + dup * Q_R(phi) + up' * Q_R(eps),
// with phi = cart(u_b), eps = cart(e_s) and the upwind switch differences
// dud, dup taken from the signs of u_b and u_b + e_s. Its rounding error is
// relative to the increment, so the iteration has the FP64 fixed point and the
// FP64 iterates up to terms proportional to the final increment.
#pragma once
#include "ns_common.cuh"

namespace ns {

struct IncArgs {
  Geom g;
  const float* sh[2];   // FP32 copy of u_base (faces)
  const float* g0[2];   // G(u_base) (faces)
  const float* ein[2];  // e_s (faces); nullptr => e_s = rk_prev * g0
  float rk_prev;
  float* eout[2];       // e_{s+1} = rk * (G0 + dG)
  float rk;
  float inv_dx[2];      // 1/dx, 1/dy
  float vcoef[2];       // 1/(ren dx^2), 1/(ren dy^2)
  float c15;            // 1.5/dt
  int do_norm;
  double* part;
  unsigned* counter;
  double* norm_out;
};

template <int TX, int TY>
struct IncSmem {
  static constexpr int CW = TX + 6, CH = TY + 6;
  static constexpr int FXW = TX + 3, FXH = TY + 2;
  static constexpr int FYW = TX + 2, FYH = TY + 3;
  static constexpr int TW = TX + 2, TH = TY + 2;
  float cp[2][CH][CW];   // cart(u_base)
  float ce[2][CH][CW];   // cart(e_s)
  float fx[2][FXH][FXW];
  float fy[2][FYH][FYW];
  float t[2][TH][TW];
};

__device__ __forceinline__ float inc_e(const IncArgs& A, int m, long id) {
  return A.ein[m] != nullptr ? A.ein[m][id] : A.rk_prev * A.g0[m][id];
}

// QUICK flux difference F(ub + e, phi + eps) - F(ub, phi) (fn_flux_calc.cpp:66-76)
// a, b, c, e: phi at i+1, i, i-1, i-2; pa..pe the same for eps.
__device__ __forceinline__ float quick_dflux(float ub, float eb, float a, float b, float c, float e, float pa, float pb_,
                                             float pc, float pe) {
  const float un = ub + eb;
  const bool sb = ub > 0.f, sn = un > 0.f;
  float dud, dup;
  if (sb && sn) { dud = eb; dup = 0.f; }
  else if (!sb && !sn) { dud = 0.f; dup = eb; }
  else if (sb) { dud = -ub; dup = un; }
  else { dud = un; dup = -ub; }
  const float udn = sn ? un : 0.f, upn = sn ? 0.f : un;
  const float qr_phi = 0.125f * (-a - 2.f * b + 3.f * c) + b;
  const float ql_phi = 0.125f * (-e - 2.f * c + 3.f * b) + c;
  const float qr_eps = 0.125f * (-pa - 2.f * pb_ + 3.f * pc) + pb_;
  const float ql_eps = 0.125f * (-pe - 2.f * pc + 3.f * pb_) + pc;
  return dud * ql_phi + udn * ql_eps + dup * qr_phi + upn * qr_eps;
}

template <int TX, int TY>
__global__ void __launch_bounds__(256) k_inc_stage2d(IncArgs A) {
  using SM = IncSmem<TX, TY>;
  __shared__ SM sm;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool perx = g.periodic[0], pery = g.periodic[1];

  // ---- cell-centred u_base and increment -------------------------------------
  for (int t = tid; t < SM::CW * SM::CH; t += NT) {
    const int lx = t % SM::CW, ly = t / SM::CW;
    const int a = x0 - 3 + lx, b = y0 - 3 + ly;
    const bool inx = (a >= 0 && a < N), iny = (b >= 0 && b < N);
    float pu = 0.f, pv = 0.f, eu = 0.f, ev = 0.f;
    if ((inx || perx) && (iny || pery)) {
      const int aa = wrapi(a, N), bb = wrapi(b, N);
      const long id = (long)bb * P + aa;
      pu = 0.5f * (A.sh[0][id] + A.sh[0][id + 1]);
      pv = 0.5f * (A.sh[1][id] + A.sh[1][id + P]);
      eu = 0.5f * (inc_e(A, 0, id) + inc_e(A, 0, id + 1));
      ev = 0.5f * (inc_e(A, 1, id) + inc_e(A, 1, id + P));
    }
    sm.cp[0][ly][lx] = pu;
    sm.cp[1][ly][lx] = pv;
    sm.ce[0][ly][lx] = eu;
    sm.ce[1][ly][lx] = ev;
  }
  __syncthreads();
  if (!perx) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int a = x0 - 3 + lx, b = y0 - 3 + ly;
      if (!(b >= 0 && b < N) && !pery) continue;
      int side = -1, ml = 0;
      if (a >= -3 && a < 0) { side = 0; ml = (-a - 1) - (x0 - 3); }
      else if (a >= N && a < N + 3) { side = 1; ml = (2 * N - 1 - a) - (x0 - 3); }
      if (side < 0) continue;
      for (int m = 0; m < 2; ++m) {
        sm.cp[m][ly][lx] = cart_ghost_f(g.bc[side], m, sm.cp[m][ly][ml], false);
        sm.ce[m][ly][lx] = cart_ghost_f(g.bc[side], m, sm.ce[m][ly][ml], true);
      }
    }
    __syncthreads();
  }
  if (!pery) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int b = y0 - 3 + ly;
      int side = -1, ml = 0;
      if (b >= -3 && b < 0) { side = 2; ml = (-b - 1) - (y0 - 3); }
      else if (b >= N && b < N + 3) { side = 3; ml = (2 * N - 1 - b) - (y0 - 3); }
      if (side < 0) continue;
      for (int m = 0; m < 2; ++m) {
        sm.cp[m][ly][lx] = cart_ghost_f(g.bc[side], m, sm.cp[m][ml][lx], false);
        sm.ce[m][ly][lx] = cart_ghost_f(g.bc[side], m, sm.ce[m][ml][lx], true);
      }
    }
    __syncthreads();
  }
  const bool wx = (g.flux_ghost[0] == kWrap), wy = (g.flux_ghost[1] == kWrap);

  // ---- flux differences -------------------------------------------------------
  for (int t = tid; t < SM::FXW * SM::FXH; t += NT) {
    const int fx = t % SM::FXW, fyy = t / SM::FXW;
    const int a = x0 - 1 + fx, b = y0 - 1 + fyy;
    const bool rowin = (b >= 0 && b < N);
    const bool facein = (a >= 0 && a <= N);
    const bool need_u = (fyy >= 1 && fyy <= TY) && rowin && (facein || wx);
    const bool need_v = (fx >= 1 && fx <= TX + 1) && (rowin || wy) && facein;
    if (!need_u && !need_v) continue;
    const int aa = facein ? a : wrapi(a, N);
    const long id = (long)wrapi(b, N) * P + aa;
    const float ub = A.sh[0][id], eb = inc_e(A, 0, id);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      sm.fx[m][fyy][fx] = quick_dflux(ub, eb, sm.cp[m][ly][lx + 1], sm.cp[m][ly][lx], sm.cp[m][ly][lx - 1], sm.cp[m][ly][lx - 2],
                                      sm.ce[m][ly][lx + 1], sm.ce[m][ly][lx], sm.ce[m][ly][lx - 1], sm.ce[m][ly][lx - 2]);
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
    const long id = (long)bb * P + wrapi(a, N);
    const float vb = A.sh[1][id], eb = inc_e(A, 1, id);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      sm.fy[m][fyy][fx] = quick_dflux(vb, eb, sm.cp[m][ly + 1][lx], sm.cp[m][ly][lx], sm.cp[m][ly - 1][lx], sm.cp[m][ly - 2][lx],
                                      sm.ce[m][ly + 1][lx], sm.ce[m][ly][lx], sm.ce[m][ly - 1][lx], sm.ce[m][ly - 2][lx]);
    }
  }
  __syncthreads();

  // ---- total-flux difference at cells ----------------------------------------
  const float idx_ = A.inv_dx[0], idy_ = A.inv_dx[1];
  const float vx = A.vcoef[0], vy = A.vcoef[1];
  for (int t = tid; t < SM::TW * SM::TH; t += NT) {
    const int tx = t % SM::TW, ty = t / SM::TW;
    const int a = x0 - 1 + tx, b = y0 - 1 + ty;
    const bool need_u = (ty >= 1 && ty <= TY) && (b < N) && ((a >= 0 && a < N) || wx);
    const bool need_v = (tx >= 1 && tx <= TX) && (a < N) && ((b >= 0 && b < N) || wy);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      const float conv = (sm.fx[m][ty][tx + 1] - sm.fx[m][ty][tx]) * idx_ + (sm.fy[m][ty + 1][tx] - sm.fy[m][ty][tx]) * idy_;
      const float ce = sm.ce[m][ly][lx];
      const float visc = (sm.ce[m][ly][lx + 1] - 2.f * ce + sm.ce[m][ly][lx - 1]) * vx +
                         (sm.ce[m][ly + 1][lx] - 2.f * ce + sm.ce[m][ly - 1][lx]) * vy;
      sm.t[m][ty][tx] = visc - conv;
    }
  }
  __syncthreads();
  if (tid < 2 * (TY + TX)) {
    if (tid < TY) {
      const int ty = tid + 1;
      if (x0 == 0 && !wx) sm.t[0][ty][0] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][1] : 0.f;
    } else if (tid < 2 * TY) {
      const int ty = tid - TY + 1;
      const int tx = N - (x0 - 1);
      if (tx >= 1 && tx < SM::TW && !wx) sm.t[0][ty][tx] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][tx - 1] : 0.f;
    } else if (tid < 2 * TY + TX) {
      const int tx = tid - 2 * TY + 1;
      if (y0 == 0 && !wy) sm.t[1][0][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][1][tx] : 0.f;
    } else {
      const int tx = tid - 2 * TY - TX + 1;
      const int ty = N - (y0 - 1);
      if (ty >= 1 && ty < SM::TH && !wy) sm.t[1][ty][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][ty - 1][tx] : 0.f;
    }
  }
  __syncthreads();

  // ---- face update --------------------------------------------------------------
  const float c15 = A.c15, rk = A.rk;
  double nrm[2] = {0.0, 0.0};
  const int nfx = (x0 + TX >= N) ? (N - x0 + 1) : TX;
  const int nfy = (y0 + TY >= N) ? (N - y0 + 1) : TY;
  const int ncx = min(TX, N - x0), ncy = min(TY, N - y0);
  for (int t = tid; t < nfx * ncy + ncx * nfy; t += NT) {
    int m, a, b;
    if (t < nfx * ncy) { m = 0; a = x0 + t % nfx; b = y0 + t / nfx; }
    else { const int q = t - nfx * ncy; m = 1; a = x0 + q % ncx; b = y0 + q / ncx; }
    const long id = (long)b * P + a;
    const int tx = a - (x0 - 1), ty = b - (y0 - 1);
    const float tm = (m == 0) ? sm.t[0][ty][tx - 1] : sm.t[1][ty - 1][tx];
    const float tc = sm.t[m][ty][tx];
    const float dG = 0.5f * (tm + tc) - c15 * inc_e(A, m, id);
    const float e = rk * (A.g0[m][id] + dG);
    A.eout[m][id] = e;
    if (A.do_norm) {
      const int face = (m == 0) ? a : b;
      const double w = (face == 0 || face == N) ? 0.5 : 1.0;
      nrm[m] += (double)e * (double)e * w;
    }
  }
  if (A.do_norm) {
    if (grid_reduce_last<2>(nrm, A.part, A.counter, 0u) && threadIdx.x == 0) {
      const double npts = (double)N * (double)N;
      *A.norm_out = fmax(sqrt(nrm[0]) / sqrt(npts), sqrt(nrm[1]) / sqrt(npts));
    }
  }
}

}  // namespace ns
