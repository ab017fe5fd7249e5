// Mixed-precision 3D predictor (NS_PREC_MIXED): each pseudo-iteration
// evaluates the BDF2 residual G at u_b, u_b + e1, u_b + e2, u_b + e3
// (main.cpp:945-1014). The anchor G0 = G(u_b) is computed in FP64 by the
// cart / flux / total passes of ns3d.cuh and k3_anchor_face below, which
// rounds G0 and u_b to FP32. The three other stages evaluate only the
// increment dG(u_b; e) = G(u_b + e) - G0 in FP32:
//   dF = (un+ - ub+) Q+(phi_b) + (un- - ub-) Q-(phi_b) + un Q_sign(un)(phi_e)
// for the QUICK flux F = u+ Q+(phi) + u- Q-(phi) (fn_flux_calc.cpp:66-76),
// with un = ub + e and the positive-part difference un+ - ub+ taken from the
// signs (e, -ub or max(un, 0)), so no term subtracts nearly equal FP32
// numbers; the viscous term, the ghost rules (homogeneous for the increment)
// and the flux-ghost rule of the faces are linear. Every FP32 rounding error
// is proportional to the increment, so the fixed point is the FP64 one. The
// last stage writes u_b + e4 in FP64 and the pseudo-norm of e4 (the
// Error_Computation norm, utilities.cpp:421-493).
#pragma once
#include "ns3d.cuh"

namespace ns {

struct Inc3 {
  Geom g;
  const float* ub[3];      // FP32 copy of u_b (faces)
  const float* g0[3];      // G(u_b) rounded to FP32 (faces)
  const float* ein[3];     // stage input increment; nullptr: rk_prev * g0
  float* eout[3];          // stage output increment (not written by the last stage)
  float* phb[3];           // ghosted FP32 cell velocity of u_b, (N+4)^3
  float* phe[3];           // ghosted cell velocity of the increment
  float* dfl[3][3];        // flux increments dfl[d][m] at the faces along d
  float* dt[3];            // cell total increments
  const double* base64[3]; // u_b (last stage)
  double* out64[3];        // u_b + e4 (last stage)
  float rk_prev, rk, c15;
  float inv_dx[3], vcoef[3];  // 1/dx, 1/(Re dx^2)
  int first, last;
  double* part;
  unsigned* counter;
  double* norm_out;
};

struct Anc3 {
  float* g0[3];
  float* ub[3];
};

#ifndef NS_3D_ARGS_ONLY

__device__ __forceinline__ float inc_e(const Inc3& A, int m, long id) {
  return A.ein[m] ? A.ein[m][id] : A.rk_prev * A.g0[m][id];
}

// G0 = S - (1.5/dt) u_b + avg(t) (FP64, as k3_face with u = u_b), rounded to
// FP32 together with u_b
__global__ void __launch_bounds__(256) k3_anchor_face(Arg3 A, Anc3 O) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const int lim[3] = {N + (m == 0), N + (m == 1), N + (m == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    const int c[3] = {i, j, k};
    const int a = c[m];
    const long id = id3(g, i, j, k);
    const long st = fstride[m];
    const long base = id - (long)a * st;
    const double tl = t_along(A, m, a - 1, base, st), tr = t_along(A, m, a, base, st);
    const double u = A.u[m][id];
    const double G = (A.S[m][id] - g.c15 * u) + 0.5 * (tl + tr);
    O.g0[m][id] = (float)G;
    O.ub[m][id] = (float)u;
  }
}

// ghosted cell velocity of the increment (homogeneous ghosts) and, in the
// first stage, of u_b; cells with more than one index outside [0, N) are 0
__global__ void __launch_bounds__(256) k3i_cart(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(2, 2, 2)
  if (i > N + 1 || j > N + 1 || k > N + 1) return;
  const int c[3] = {i, j, k};
  int out_d = -1, nout = 0;
  for (int d = 0; d < 3; ++d)
    if (c[d] < 0 || c[d] >= N) { out_d = d; ++nout; }
  int cm[3] = {i, j, k};
  int side = 0;
  if (nout == 1) {
    const int d = out_d;
    side = c[d] < 0 ? 0 : 1;
    cm[d] = g.periodic[d] ? wrapi(c[d], N) : (c[d] < 0 ? -c[d] - 1 : 2 * N - 1 - c[d]);
  }
  const bool mirror = nout == 1 && !g.periodic[out_d];
  const long gi = gid3(N, i, j, k);
  for (int m = 0; m < 3; ++m) {
    float ve = 0.f, vb = 0.f;
    if (nout <= 1) {
      const long a = id3(g, cm[0], cm[1], cm[2]);
      const long b = a + (m == 0 ? 1 : (m == 1 ? g.pitch : g.plane));
      ve = 0.5f * (inc_e(A, m, a) + inc_e(A, m, b));
      if (A.first) vb = 0.5f * (A.ub[m][a] + A.ub[m][b]);
      if (mirror) {
        const CartBC& bc = g.bc[2 * out_d + side];
        ve = cart_ghost_f(bc, m, ve, true);
        if (A.first) vb = cart_ghost_f(bc, m, vb, false);
      }
    }
    A.phe[m][gi] = ve;
    if (A.first) A.phb[m][gi] = vb;
  }
}

// QUICK interpolants: u > 0 from cells -2, -1, 0; u <= 0 from cells -1, 0, +1
__device__ __forceinline__ float q3p(float x2, float x1, float x0) { return -0.125f * x2 + 0.75f * x1 + 0.375f * x0; }
__device__ __forceinline__ float q3m(float x1, float x0, float xa) { return 0.375f * x1 + 0.75f * x0 - 0.125f * xa; }

// flux increments of the three components at every face along the three
// directions, each face once (the faces of k3_flux)
__global__ void __launch_bounds__(256) k3i_flux(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  if (i > N || j > N || k > N) return;
  const long G1[3] = {1, N + 4, (long)(N + 4) * (N + 4)};
  const long gc = gid3(N, i, j, k);
  const long fc = id3(g, i, j, k);
  const int c[3] = {i, j, k};
  for (int d = 0; d < 3; ++d) {
    bool ok = true;
    for (int e = 0; e < 3; ++e)
      if (e != d && c[e] >= N) ok = false;
    if (!ok) continue;
    const long s = G1[d];
    const float ub = A.ub[d][fc];
    const float e = inc_e(A, d, fc);
    const float un = ub + e;
    const float dpos = ub > 0.f ? (un > 0.f ? e : -ub) : fmaxf(un, 0.f);  // un+ - ub+
    const float dneg = e - dpos;                                            // un- - ub-
    const bool pos = un > 0.f;
    for (int m = 0; m < 3; ++m) {
      const float* pb = A.phb[m];
      const float* pe = A.phe[m];
      const float b2 = pb[gc - 2 * s], b1 = pb[gc - s], b0 = pb[gc], ba = pb[gc + s];
      const float e1 = pe[gc - s], e0 = pe[gc];
      const float qe = pos ? q3p(pe[gc - 2 * s], e1, e0) : q3m(e1, e0, pe[gc + s]);
      A.dfl[d][m][fc] = dpos * q3p(b2, b1, b0) + dneg * q3m(b1, b0, ba) + un * qe;
    }
  }
}

// dt_m = nu lap(phi_e,m) - div dF_m at the cells
__global__ void __launch_bounds__(256) k3i_total(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  if (i >= N || j >= N || k >= N) return;
  const long G1[3] = {1, N + 4, (long)(N + 4) * (N + 4)};
  const long gc = gid3(N, i, j, k);
  const long fc = id3(g, i, j, k);
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const float* ph = A.phe[m];
    const float p0 = ph[gc];
    float conv = 0.f, visc = 0.f;
    for (int d = 0; d < 3; ++d) {
      const long s = G1[d];
      const float* F = A.dfl[d][m];
      conv += (F[fc + fstride[d]] - F[fc]) * A.inv_dx[d];
      visc += (ph[gc + s] - 2.f * p0 + ph[gc - s]) * A.vcoef[d];
    }
    A.dt[m][fc] = visc - conv;
  }
}

__device__ __forceinline__ float t_along_inc(const Inc3& A, int m, int a, long base, long st) {
  const int N = A.g.N;
  if (a >= 0 && a < N) return A.dt[m][base + a * st];
  const int fg = A.g.flux_ghost[m];
  if (fg == kWrap) return A.dt[m][base + (long)wrapi(a, N) * st];
  if (fg == kZero) return 0.f;
  const int am = a < 0 ? 0 : N - 1;
  return -A.dt[m][base + (long)am * st];
}

// e_out = rk (G0 - (1.5/dt) e_in + avg(dt)); the last stage writes
// u_b + e_out in FP64 and the pseudo-norm of e_out
__global__ void __launch_bounds__(256) k3i_face(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  double nrm[3] = {0.0, 0.0, 0.0};
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const int lim[3] = {N + (m == 0), N + (m == 1), N + (m == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    const int c[3] = {i, j, k};
    const int a = c[m];
    const long id = id3(g, i, j, k);
    const long st = fstride[m];
    const long base = id - (long)a * st;
    const float tl = t_along_inc(A, m, a - 1, base, st), tr = t_along_inc(A, m, a, base, st);
    const float G = (A.g0[m][id] - A.c15 * inc_e(A, m, id)) + 0.5f * (tl + tr);
    const float eo = A.rk * G;
    if (A.last) {
      A.out64[m][id] = A.base64[m][id] + (double)eo;
      const float w = (a == 0 || a == N) ? 0.5f : 1.f;
      nrm[m] = (double)(eo * eo * w);
    } else {
      A.eout[m][id] = eo;
    }
  }
  if (A.last && grid_reduce_last<3>(nrm, A.part, A.counter, 0u) && threadIdx.x == 0) {
    const double npts = (double)N * N * N;
    double e = 0.0;
    for (int m = 0; m < 3; ++m) e = fmax(e, sqrt(nrm[m]) / sqrt(npts));
    *A.norm_out = e;
  }
}

#endif  // NS_3D_ARGS_ONLY

}  // namespace ns
