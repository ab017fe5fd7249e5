// Tangent-linear and adjoint operators of one 3D step, periodic boxes in the
// physical mode (flux ghosts wrapped, p / phi ghosts wrapped), FP64.
//
// In a periodic direction face N is the image of face 0 (the step updates
// both identically), so the degrees of freedom are the faces 0 .. N-1 of
// every component and every index wraps: the operators below are
// translation-invariant and need no ghost cells. With the QUICK switches
// frozen at u* the predictor Jacobian J = dA/du - (1.5/dt) I acts as
//   jvp: dphi_m = cell average of v_m; dF_{d,m}(f) = v_d(f) Q_{d,m}(f) +
//        u_d(f) Q(dphi_m); dt_m = nu lap dphi_m - div_d dF_{d,m};
//        (J v)_m(f) = avg(dt_m)(f) - (1.5/dt) v_m(f),
//   vjp: the transposed passes (tbar, flux adjoints and the advecting-velocity
//        adjoint, cell-velocity adjoint, face average),
// where Q_{d,m} is the base QUICK interpolant at the face (fn_flux_calc.cpp:66-76).
#pragma once
#include "ns3d.cuh"

namespace ns {

struct A3Args {
  Geom g;
  const double* us[3];  // base u* (faces)
  double* phb[3];       // base cell velocity
  double* q[3][3];      // base QUICK interpolant of component m at the faces along d
  const double* v[3];   // tangent direction / adjoint input
  double* dph[3];       // cell velocity tangent / adjoint
  double* fl[3][3];     // face flux tangents / adjoints
  double* ct[3];        // cell totals (tangent) / tbar (adjoint)
  double* uadv[3];      // advecting-velocity adjoint
  double* out[3];
};

struct Bcg3 {
  Geom g;
  double* x[3];
  double* r[3];
  double* rh[3];
  double* p[3];
  double* v[3];
  double* s[3];
  double* t[3];
  const double* b[3];
  double* sc;
  double* part;
  unsigned* counter;
};

#ifndef NS_ADJ3_ARGS_ONLY

// wrapped index of (i, j, k) shifted by o along d
__device__ __forceinline__ long wid(const Geom& g, int i, int j, int k, int d, int o) {
  const int N = g.N;
  int c[3] = {i, j, k};
  c[d] = wrapi(c[d] + o, N);
  return id3(g, c[0], c[1], c[2]);
}

#define NS3A_IJK                                                 \
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);           \
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);            \
  const int k = blockIdx.z;                                      \
  const int N = A.g.N;                                           \
  if (i >= N || j >= N || k >= N) return;                        \
  const long id = id3(A.g, i, j, k);

__device__ __forceinline__ double qleft3(double e, double c, double b) { return -0.125 * e + 0.75 * c + 0.375 * b; }
__device__ __forceinline__ double qright3(double c, double b, double a) { return 0.375 * c + 0.75 * b - 0.125 * a; }

// QUICK interpolant at face f along d of a cell field x, switch from u
__device__ __forceinline__ double quick_at(const Geom& g, const double* x, int i, int j, int k, int d, double u) {
  if (u > 0) return qleft3(x[wid(g, i, j, k, d, -2)], x[wid(g, i, j, k, d, -1)], x[id3(g, i, j, k)]);
  return qright3(x[wid(g, i, j, k, d, -1)], x[id3(g, i, j, k)], x[wid(g, i, j, k, d, 1)]);
}

__global__ void __launch_bounds__(256) k3a_base_cells(A3Args A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.phb[m][id] = 0.5 * (A.us[m][id] + A.us[m][wid(A.g, i, j, k, m, 1)]);
}

__global__ void __launch_bounds__(256) k3a_base_q(A3Args A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    const double u = A.us[d][id];
    for (int m = 0; m < 3; ++m) A.q[d][m][id] = quick_at(A.g, A.phb[m], i, j, k, d, u);
  }
}

// ---- tangent ------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3a_jv_cells(A3Args A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.dph[m][id] = 0.5 * (A.v[m][id] + A.v[m][wid(A.g, i, j, k, m, 1)]);
}

__global__ void __launch_bounds__(256) k3a_jv_flux(A3Args A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    const double u = A.us[d][id], du = A.v[d][id];
    for (int m = 0; m < 3; ++m) A.fl[d][m][id] = du * A.q[d][m][id] + u * quick_at(A.g, A.dph[m], i, j, k, d, u);
  }
}

__global__ void __launch_bounds__(256) k3a_jv_total(A3Args A) {
  NS3A_IJK
  const Geom& g = A.g;
  for (int m = 0; m < 3; ++m) {
    const double* x = A.dph[m];
    const double c = x[id];
    double visc = 0.0, conv = 0.0;
    for (int d = 0; d < 3; ++d) {
      visc += (x[wid(g, i, j, k, d, 1)] - 2.0 * c + x[wid(g, i, j, k, d, -1)]) * g.inv_dx2[d];
      conv += (A.fl[d][m][wid(g, i, j, k, d, 1)] - A.fl[d][m][id]) * g.inv_dx[d];
    }
    A.ct[m][id] = visc * g.inv_ren - conv;
  }
}

__global__ void __launch_bounds__(256) k3a_jv_faces(A3Args A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m)
    A.out[m][id] = 0.5 * (A.ct[m][wid(A.g, i, j, k, m, -1)] + A.ct[m][id]) - A.g.c15 * A.v[m][id];
}

// ---- adjoint ------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k3a_vj_tbar(A3Args A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.ct[m][id] = 0.5 * (A.v[m][id] + A.v[m][wid(A.g, i, j, k, m, 1)]);
}

__global__ void __launch_bounds__(256) k3a_vj_flux(A3Args A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    double ua = 0.0;
    for (int m = 0; m < 3; ++m) {
      const double fb = (A.ct[m][id] - A.ct[m][wid(A.g, i, j, k, d, -1)]) * A.g.inv_dx[d];
      A.fl[d][m][id] = fb;
      ua += fb * A.q[d][m][id];
    }
    A.uadv[d][id] = ua;
  }
}

// weight of cell offset o (cell - face) in the face's QUICK interpolant
__device__ __forceinline__ double quick_w3(bool pos, int o) {
  if (pos) return o == -2 ? -0.125 : (o == -1 ? 0.75 : (o == 0 ? 0.375 : 0.0));
  return o == -1 ? 0.375 : (o == 0 ? 0.75 : (o == 1 ? -0.125 : 0.0));
}

__global__ void __launch_bounds__(256) k3a_vj_cells(A3Args A) {
  NS3A_IJK
  const Geom& g = A.g;
  for (int m = 0; m < 3; ++m) {
    const double* tb = A.ct[m];
    const double c = tb[id];
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
      s += (tb[wid(g, i, j, k, d, 1)] - 2.0 * c + tb[wid(g, i, j, k, d, -1)]) * g.inv_dx2[d] * g.inv_ren;
      for (int f = -1; f <= 2; ++f) {  // faces (along d) whose stencil holds this cell
        const long fid = wid(g, i, j, k, d, f);
        const double u = A.us[d][fid];
        s += A.fl[d][m][fid] * u * quick_w3(u > 0, -f);
      }
    }
    A.dph[m][id] = s;
  }
}

__global__ void __launch_bounds__(256) k3a_vj_faces(A3Args A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m)
    A.out[m][id] = A.uadv[m][id] + 0.5 * (A.dph[m][wid(A.g, i, j, k, m, -1)] + A.dph[m][id]) - A.g.c15 * A.v[m][id];
}

// ---- projection pieces (wrapped) --------------------------------------------------------
// f = D u + coef * pb; sum f into sum_out, max |f| into max_out (nullable)
__global__ void __launch_bounds__(256) k3a_div(Geom g, const double* u0, const double* u1, const double* u2,
                                               const double* pb, double coef, double* f, double* part, unsigned* counter,
                                               double* sum_out, double* max_out) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  const int N = g.N;
  double v[2] = {0.0, 0.0};
  if (i < N && j < N && k < N) {
    const long id = id3(g, i, j, k);
    double r = (u0[wid(g, i, j, k, 0, 1)] - u0[id]) * g.inv_dx[0] + (u1[wid(g, i, j, k, 1, 1)] - u1[id]) * g.inv_dx[1] +
               (u2[wid(g, i, j, k, 2, 1)] - u2[id]) * g.inv_dx[2];
    if (pb) r += coef * pb[id];
    f[id] = r;
    v[0] = r;
    v[1] = fabs(r);
  }
  if (grid_reduce_last<2>(v, part, counter, 2u) && threadIdx.x == 0) {
    sum_out[0] = v[0];
    if (max_out) max_out[0] = v[1];
  }
}

// out = in - coef grad psi
__global__ void __launch_bounds__(256) k3a_gradsub(A3Args A, const double* psi, double coef) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d)
    A.out[d][id] = A.v[d][id] - coef * (psi[id] - psi[wid(A.g, i, j, k, d, -1)]) * A.g.inv_dx[d];
}

// out = a x + b y (y nullable); faces of three components
__global__ void __launch_bounds__(256) k3a_lincomb(Geom g, double a, const double* x0, const double* x1, const double* x2,
                                                   double b, const double* y0, const double* y1, const double* y2, double* o0,
                                                   double* o1, double* o2) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= g.N || j >= g.N || k >= g.N) return;
  const long id = id3(g, i, j, k);
  o0[id] = a * x0[id] + (y0 ? b * y0[id] : 0.0);
  o1[id] = a * x1[id] + (y1 ? b * y1[id] : 0.0);
  o2[id] = a * x2[id] + (y2 ? b * y2[id] : 0.0);
}

// cells: out = a x + b y (y nullable)
__global__ void __launch_bounds__(256) k3a_cells(Geom g, double a, const double* x, double b, const double* y, double* o) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= g.N || j >= g.N || k >= g.N) return;
  const long id = id3(g, i, j, k);
  o[id] = a * x[id] + (y ? b * y[id] : 0.0);
}

// b = -(-G dp + (2/dt) du - (0.5/dt) du_prev)
__global__ void __launch_bounds__(256) k3a_tlm_rhs(A3Args A, const double* dp, const double* dup0, const double* dup1,
                                                   const double* dup2) {
  NS3A_IJK
  const double c2 = A.g.c15 + A.g.c05;
  const double* dup[3] = {dup0, dup1, dup2};
  for (int d = 0; d < 3; ++d) {
    const double gp = (dp[id] - dp[wid(A.g, i, j, k, d, -1)]) * A.g.inv_dx[d];
    A.out[d][id] = -(-gp + c2 * A.v[d][id] - A.g.c05 * dup[d][id]);
  }
}

// ---- BiCGStab over the three face fields ---------------------------------------------------
#define BCG3_PROLOGUE                                                                                          \
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z; \
  const bool in = i < A.g.N && j < A.g.N && k < A.g.N;                                                         \
  const long id = in ? id3(A.g, i, j, k) : 0;

__global__ void __launch_bounds__(256) k3b_init(Bcg3 A) {
  BCG3_PROLOGUE
  double red[2] = {0.0, 0.0};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const double bb = A.b[m][id], r = bb - A.v[m][id];
      A.r[m][id] = r;
      A.rh[m][id] = r;
      A.p[m][id] = r;
      red[0] += r * r;
      red[1] += bb * bb;
    }
  if (grid_reduce_last<2>(red, A.part, A.counter, 0u) && threadIdx.x == 0) {
    double* sc = A.sc;
    sc[kBcRho] = red[0];
    sc[kBcAlpha] = 1.0;
    sc[kBcOmega] = 1.0;
    sc[kBcBeta] = 0.0;
    sc[kBcRR] = red[0];
    sc[kBcRR0] = red[0];
    sc[kBcBB] = red[1];
    sc[kBcBreak] = 0.0;
  }
}

__global__ void __launch_bounds__(256) k3b_alpha(Bcg3 A) {
  BCG3_PROLOGUE
  double red[1] = {0.0};
  if (in)
    for (int m = 0; m < 3; ++m) red[0] += A.rh[m][id] * A.v[m][id];
  if (grid_reduce_last<1>(red, A.part, A.counter, 0u) && threadIdx.x == 0) {
    double* sc = A.sc;
    if (red[0] != 0.0 && isfinite(red[0])) sc[kBcAlpha] = sc[kBcRho] / red[0];
    else { sc[kBcAlpha] = 0.0; sc[kBcBreak] = 1.0; }
  }
}

__global__ void __launch_bounds__(256) k3b_s(Bcg3 A) {
  BCG3_PROLOGUE
  if (!in) return;
  const double al = A.sc[kBcAlpha];
  for (int m = 0; m < 3; ++m) A.s[m][id] = A.r[m][id] - al * A.v[m][id];
}

__global__ void __launch_bounds__(256) k3b_omega(Bcg3 A) {
  BCG3_PROLOGUE
  double red[2] = {0.0, 0.0};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const double t = A.t[m][id];
      red[0] += t * A.s[m][id];
      red[1] += t * t;
    }
  if (grid_reduce_last<2>(red, A.part, A.counter, 0u) && threadIdx.x == 0) {
    double* sc = A.sc;
    sc[kBcOmega] = red[1] > 0.0 ? red[0] / red[1] : 0.0;
    if (sc[kBcOmega] == 0.0) sc[kBcBreak] = 2.0;
  }
}

__global__ void __launch_bounds__(256) k3b_xr(Bcg3 A) {
  BCG3_PROLOGUE
  const double al = A.sc[kBcAlpha], om = A.sc[kBcOmega];
  double red[2] = {0.0, 0.0};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const double s = A.s[m][id];
      A.x[m][id] += al * A.p[m][id] + om * s;
      const double r = s - om * A.t[m][id];
      A.r[m][id] = r;
      red[0] += A.rh[m][id] * r;
      red[1] += r * r;
    }
  if (grid_reduce_last<2>(red, A.part, A.counter, 0u) && threadIdx.x == 0) {
    double* sc = A.sc;
    const double rho = sc[kBcRho];
    sc[kBcBeta] = (rho != 0.0 && om != 0.0) ? (red[0] / rho) * (al / om) : 0.0;
    if (rho == 0.0) sc[kBcBreak] = 3.0;
    sc[kBcRho] = red[0];
    sc[kBcRR] = red[1];
  }
}

__global__ void __launch_bounds__(256) k3b_p(Bcg3 A) {
  BCG3_PROLOGUE
  if (!in) return;
  const double be = A.sc[kBcBeta], om = A.sc[kBcOmega];
  for (int m = 0; m < 3; ++m) A.p[m][id] = A.r[m][id] + be * (A.p[m][id] - om * A.v[m][id]);
}
#undef BCG3_PROLOGUE

// ---- enstrophy: E = 1/2 sum over the edges of |curl u|^2 dV ----------------------------------
// omega_x at the x edge (i+1/2, j, k) = dw/dy - dv/dz, and cyclically
__global__ void __launch_bounds__(256) k3a_vort(A3Args A) {
  NS3A_IJK
  const Geom& g = A.g;
  const double* u = A.v[0];
  const double* v = A.v[1];
  const double* w = A.v[2];
  A.out[0][id] = (w[id] - w[wid(g, i, j, k, 1, -1)]) * g.inv_dx[1] - (v[id] - v[wid(g, i, j, k, 2, -1)]) * g.inv_dx[2];
  A.out[1][id] = (u[id] - u[wid(g, i, j, k, 2, -1)]) * g.inv_dx[2] - (w[id] - w[wid(g, i, j, k, 0, -1)]) * g.inv_dx[0];
  A.out[2][id] = (v[id] - v[wid(g, i, j, k, 0, -1)]) * g.inv_dx[0] - (u[id] - u[wid(g, i, j, k, 1, -1)]) * g.inv_dx[1];
}

__global__ void __launch_bounds__(256) k3a_enstrophy(Geom g, const double* o0, const double* o1, const double* o2,
                                                     double* part, unsigned* counter, double* red_out) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  double v[1] = {0.0};
  if (i < g.N && j < g.N && k < g.N) {
    const long id = id3(g, i, j, k);
    v[0] = 0.5 * (o0[id] * o0[id] + o1[id] * o1[id] + o2[id] * o2[id]) * g.dx[0] * g.dx[1] * g.dx[2];
  }
  if (grid_reduce_last<1>(v, part, counter, 0u) && threadIdx.x == 0) red_out[0] = v[0];
}

// dE/du from the edge vorticity in A.v: the transpose of k3a_vort, times dV
__global__ void __launch_bounds__(256) k3a_enstrophy_grad(A3Args A) {
  NS3A_IJK
  const Geom& g = A.g;
  const double* ox = A.v[0];
  const double* oy = A.v[1];
  const double* oz = A.v[2];
  const double dv = g.dx[0] * g.dx[1] * g.dx[2];
  A.out[0][id] = dv * ((oy[id] - oy[wid(g, i, j, k, 2, 1)]) * g.inv_dx[2] + (oz[wid(g, i, j, k, 1, 1)] - oz[id]) * g.inv_dx[1]);
  A.out[1][id] = dv * ((ox[wid(g, i, j, k, 2, 1)] - ox[id]) * g.inv_dx[2] + (oz[id] - oz[wid(g, i, j, k, 0, 1)]) * g.inv_dx[0]);
  A.out[2][id] = dv * ((ox[id] - ox[wid(g, i, j, k, 1, 1)]) * g.inv_dx[1] + (oy[wid(g, i, j, k, 0, 1)] - oy[id]) * g.inv_dx[0]);
}

#endif  // NS_ADJ3_ARGS_ONLY

}  // namespace ns
