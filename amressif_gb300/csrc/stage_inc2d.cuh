// FP32 increment stages of the mixed-precision pseudo-time iteration (2D).
//
// The reference's RK pseudo-iteration (main.cpp:929-1026) evaluates, from a
// base u_b, the stages u*_{s+1} = u_b + rk[s] G(u*_s) with G the BDF2 residual
// of the QUICK + viscous momentum equation. Writing u*_s = u_b + e_s,
//   G(u_b + e_s) = G(u_b) + dG(u_b; e_s),
//   dG = -(1.5/dt) e_s + avg(-[conv(u_b+e_s) - conv(u_b)] + visc(e_s)).
// G(u_b) is evaluated once per iteration in float-float arithmetic (the anchor
// stage). dG only involves the small increment e_s: it is evaluated here in
// FP32 from the FP32 part of u_b, with the QUICK flux difference expanded so
// that no term subtracts two nearly equal FP32 numbers:
//   dF = dud * Q_L(phi) + ud' * Q_L(eps) + dup * Q_R(phi) + up' * Q_R(eps),
// with phi = cart(u_b), eps = cart(e_s) and the upwind switch differences
// dud, dup taken from the signs of u_b and u_b + e_s. Its rounding error is
// relative to the increment, so the iteration keeps the FP64 fixed point and
// follows the FP64 iterates up to terms proportional to the final increment.
//
// Tile: TX x TY cells per block of NT threads; every phase walks a fixed
// rectangle of shared memory with a flattened thread index (compile-time
// widths), so no lane idles on the halo columns.
#pragma once
#include "ns_common.cuh"

namespace ns {

struct IncArgs {
  Geom g;
  const float* sh[2];   // FP32 part of u_base (faces)
  const float* g0[2];   // G(u_base) (faces)
  const float* ein[2];  // e_s (faces); nullptr => e_s = rk_prev * g0
  float rk_prev;
  float* eout[2];       // e_{s+1} = rk * (G0 + dG)
  float rk;
  float inv_dx[2];      // 1/dx, 1/dy
  float vcoef[2];       // 1/(ren dx^2), 1/(ren dy^2)
  float c15;            // 1.5/dt
  int do_norm;
  float2* part;         // float-float block partials of the norm
  unsigned* counter;
  double* norm_out;
};

template <int TX, int TY>
struct IncSmem {
  // face tiles, origin (x0-3, y0-3)
  static constexpr int UW = TX + 7, UH = TY + 6;
  static constexpr int VW = TX + 6, VH = TY + 7;
  static constexpr int CW = TX + 6, CH = TY + 6;   // cells, origin (x0-3, y0-3)
  static constexpr int FXW = TX + 3, FXH = TY + 2; // x-face fluxes, origin (x0-1, y0-1)
  static constexpr int FYW = TX + 2, FYH = TY + 3; // y-face fluxes, origin (x0-1, y0-1)
  static constexpr int TW = TX + 2, TH = TY + 2;   // totals, origin (x0-1, y0-1)
  float ub[UH][UW], ue[UH][UW];
  float vb[VH][VW], ve[VH][VW];
  union {
    float cp[2][CH][CW];   // cart(u_base), dead once the fluxes exist
    float t[2][TH][TW];
  };
  float ce[2][CH][CW];     // cart(e_s)
  float fx[2][FXH][FXW];
  float fy[2][FYH][FYW];
};

// QUICK flux difference F(ub + e, phi + eps) - F(ub, phi) (fn_flux_calc.cpp:66-76)
// a, b, c, e: phi at i+1, i, i-1, i-2; pa..pe the same for eps. Branch-free.
__device__ __forceinline__ float quick_dflux(float ub, float eb, float a, float b, float c, float e, float pa, float pb_,
                                             float pc, float pe) {
  const float un = ub + eb;
  const bool sb = ub > 0.f, sn = un > 0.f;
  const float dud = sn ? (sb ? eb : un) : (sb ? -ub : 0.f);
  const float dup = sn ? (sb ? 0.f : -ub) : (sb ? un : eb);
  const float udn = sn ? un : 0.f, upn = sn ? 0.f : un;
  const float qr_phi = fmaf(0.125f, (-a - 2.f * b) + 3.f * c, b);
  const float ql_phi = fmaf(0.125f, (-e - 2.f * c) + 3.f * b, c);
  const float qr_eps = fmaf(0.125f, (-pa - 2.f * pb_) + 3.f * pc, pb_);
  const float ql_eps = fmaf(0.125f, (-pe - 2.f * pc) + 3.f * pb_, pc);
  return fmaf(dud, ql_phi, fmaf(udn, ql_eps, fmaf(dup, qr_phi, upn * qr_eps)));
}

template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_inc_stage2d(IncArgs A) {
  using SM = IncSmem<TX, TY>;
  extern __shared__ __align__(16) unsigned char inc_smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(inc_smem_raw);
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const bool perx = g.periodic[0], pery = g.periodic[1];
  const float* __restrict__ shu = A.sh[0];
  const float* __restrict__ shv = A.sh[1];
  const bool e_from_g0 = (A.ein[0] == nullptr);
  const float* __restrict__ eu_src = e_from_g0 ? A.g0[0] : A.ein[0];
  const float* __restrict__ ev_src = e_from_g0 ? A.g0[1] : A.ein[1];
  const float escale = e_from_g0 ? A.rk_prev : 1.f;

  // ---- 0. face tiles -------------------------------------------------------
  NS_RECT_LOOP(SM::UW, SM::UH, NT, r, c) {
    int b = y0 - 3 + r;
    if (b < 0 || b >= N) b = pery ? wrapi(b, N) : -1;
    int a = x0 - 3 + c;  // face index in [0, N]
    if (a < 0 || a > N) a = perx ? wrapi(a, N) : -1;
    float vb = 0.f, ve = 0.f;
    if (b >= 0 && a >= 0) {
      const long id = (long)b * P + a;
      vb = shu[id];
      ve = escale * eu_src[id];
    }
    sm.ub[r][c] = vb;
    sm.ue[r][c] = ve;
  }
  NS_RECT_LOOP(SM::VW, SM::VH, NT, r, c) {
    int b = y0 - 3 + r;  // face row in [0, N]
    if (b < 0 || b > N) b = pery ? wrapi(b, N) : -1;
    int a = x0 - 3 + c;
    if (a < 0 || a >= N) a = perx ? wrapi(a, N) : -1;
    float vb = 0.f, ve = 0.f;
    if (b >= 0 && a >= 0) {
      const long id = (long)b * P + a;
      vb = shv[id];
      ve = escale * ev_src[id];
    }
    sm.vb[r][c] = vb;
    sm.ve[r][c] = ve;
  }
  __syncthreads();

  // ---- 1. cell-centred values (cont2cart) ---------------------------------
  NS_RECT_LOOP(SM::CW, SM::CH, NT, r, c) {
    sm.cp[0][r][c] = 0.5f * (sm.ub[r][c] + sm.ub[r][c + 1]);
    sm.cp[1][r][c] = 0.5f * (sm.vb[r][c] + sm.vb[r + 1][c]);
    sm.ce[0][r][c] = 0.5f * (sm.ue[r][c] + sm.ue[r][c + 1]);
    sm.ce[1][r][c] = 0.5f * (sm.ve[r][c] + sm.ve[r + 1][c]);
  }
  __syncthreads();
  // wall / lid ghosts (utilities.cpp:62-349): x sides first, then y sides
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
      for (int m = 0; m < 2; ++m) {
        sm.cp[m][r][c] = cart_ghost_f(g.bc[side], m, sm.cp[m][r][cm], false);
        sm.ce[m][r][c] = cart_ghost_f(g.bc[side], m, sm.ce[m][r][cm], true);
      }
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
        sm.cp[m][r][c] = cart_ghost_f(g.bc[side], m, sm.cp[m][rm][c], false);
        sm.ce[m][r][c] = cart_ghost_f(g.bc[side], m, sm.ce[m][rm][c], true);
      }
    }
    __syncthreads();
  }

  // ---- 2. flux differences at x faces and y faces ----------------------------
  NS_RECT_LOOP(SM::FXW, SM::FXH, NT, fr, fc) {
    const float ub = sm.ub[fr + 2][fc + 2], eb = sm.ue[fr + 2][fc + 2];
#pragma unroll
    for (int m = 0; m < 2; ++m)
      sm.fx[m][fr][fc] = quick_dflux(ub, eb, sm.cp[m][fr + 2][fc + 3], sm.cp[m][fr + 2][fc + 2], sm.cp[m][fr + 2][fc + 1],
                                     sm.cp[m][fr + 2][fc], sm.ce[m][fr + 2][fc + 3], sm.ce[m][fr + 2][fc + 2],
                                     sm.ce[m][fr + 2][fc + 1], sm.ce[m][fr + 2][fc]);
  }
  NS_RECT_LOOP(SM::FYW, SM::FYH, NT, fr, fc) {
    const float vb = sm.vb[fr + 2][fc + 2], eb = sm.ve[fr + 2][fc + 2];
#pragma unroll
    for (int m = 0; m < 2; ++m)
      sm.fy[m][fr][fc] = quick_dflux(vb, eb, sm.cp[m][fr + 3][fc + 2], sm.cp[m][fr + 2][fc + 2], sm.cp[m][fr + 1][fc + 2],
                                     sm.cp[m][fr][fc + 2], sm.ce[m][fr + 3][fc + 2], sm.ce[m][fr + 2][fc + 2],
                                     sm.ce[m][fr + 1][fc + 2], sm.ce[m][fr][fc + 2]);
  }
  __syncthreads();

  // ---- 3. total-flux differences at cells (t reuses the cp storage) -------------
  const float idx_ = A.inv_dx[0], idy_ = A.inv_dx[1], vx = A.vcoef[0], vy = A.vcoef[1];
  NS_RECT_LOOP(SM::TW, SM::TH, NT, tr, tc) {
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const float conv = (sm.fx[m][tr][tc + 1] - sm.fx[m][tr][tc]) * idx_ + (sm.fy[m][tr + 1][tc] - sm.fy[m][tr][tc]) * idy_;
      const float ce = sm.ce[m][tr + 2][tc + 2];
      const float visc = (sm.ce[m][tr + 2][tc + 3] - 2.f * ce + sm.ce[m][tr + 2][tc + 1]) * vx +
                         (sm.ce[m][tr + 3][tc + 2] - 2.f * ce + sm.ce[m][tr + 1][tc + 2]) * vy;
      sm.t[m][tr][tc] = visc - conv;
    }
  }
  __syncthreads();
  // normal-component ghosts of the total flux (main.cpp:945-1014)
  const bool wrapx = g.flux_ghost[0] == kWrap, wrapy = g.flux_ghost[1] == kWrap;
  if ((x0 == 0 || x0 + TX >= N) && !wrapx) {
    for (int tr = threadIdx.x; tr < SM::TH; tr += NT) {
      if (x0 == 0) sm.t[0][tr][0] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][tr][1] : 0.f;
      const int tc = N - (x0 - 1);
      if (x0 + TX >= N && tc < SM::TW) sm.t[0][tr][tc] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][tr][tc - 1] : 0.f;
    }
  }
  if ((y0 == 0 || y0 + TY >= N) && !wrapy) {
    for (int tc = threadIdx.x; tc < SM::TW; tc += NT) {
      if (y0 == 0) sm.t[1][0][tc] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][1][tc] : 0.f;
      const int tr = N - (y0 - 1);
      if (y0 + TY >= N && tr < SM::TH) sm.t[1][tr][tc] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][tr - 1][tc] : 0.f;
    }
  }
  __syncthreads();

  // ---- 4. face update -----------------------------------------------------------
  const float c15 = A.c15, rk = A.rk;
  float n0 = 0.f, n1 = 0.f;
  auto face_u = [&](int a, int b) {
    const int tc = a - (x0 - 1), tr = b - (y0 - 1);
    const long id = (long)b * P + a;
    const float dG = 0.5f * (sm.t[0][tr][tc - 1] + sm.t[0][tr][tc]) - c15 * sm.ue[tr + 2][tc + 2];
    const float e = rk * (A.g0[0][id] + dG);
    A.eout[0][id] = e;
    const float w = (a == 0 || a == N) ? 0.5f : 1.f;
    n0 = fmaf(w * e, e, n0);
  };
  auto face_v = [&](int a, int b) {
    const int tc = a - (x0 - 1), tr = b - (y0 - 1);
    const long id = (long)b * P + a;
    const float dG = 0.5f * (sm.t[1][tr - 1][tc] + sm.t[1][tr][tc]) - c15 * sm.ve[tr + 2][tc + 2];
    const float e = rk * (A.g0[1][id] + dG);
    A.eout[1][id] = e;
    const float w = (b == 0 || b == N) ? 0.5f : 1.f;
    n1 = fmaf(w * e, e, n1);
  };
  NS_RECT_LOOP(TX, TY, NT, k, l) {
    const int a = x0 + l, b = y0 + k;
    if (a < N && b < N) { face_u(a, b); face_v(a, b); }
  }
  if (x0 + TX >= N && N > x0) {  // last face column a = N
    for (int k = threadIdx.x; k < TY; k += NT)
      if (y0 + k < N) face_u(N, y0 + k);
  }
  if (y0 + TY >= N && N > y0) {  // last face row b = N
    for (int k = threadIdx.x; k < TX; k += NT)
      if (x0 + k < N) face_v(x0 + k, N);
  }
  if (A.do_norm) {
    float v[2] = {n0, n1};
    double out[2];
    if (grid_reduce_last_f<2, NT>(v, A.part, A.counter, 0u, out) && threadIdx.x == 0) {
      const double npts = (double)N * (double)N;
      *A.norm_out = fmax(sqrt(out[0]) / sqrt(npts), sqrt(out[1]) / sqrt(npts));
    }
  }
}

}  // namespace ns
