// Tangent-linear and adjoint operators of one 3D step, periodic boxes in the
// physical mode (flux ghosts wrapped, p / phi ghosts wrapped). The operators
// are FP64; in the mixed-precision mode the linear solves refine an FP64
// residual with inner FP32 BiCGStab solves (the operator kernels are
// templates on the element type).
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

// operands of the predictor Jacobian in element type T (double: the FP64
// operator; float: the inner solves of the mixed-precision refinement)
template <typename T>
struct A3T {
  Geom g;
  const T* us[3];  // base u* (faces)
  T* phb[3];       // base cell velocity
  T* q[3][3];      // base QUICK interpolant of component m at the faces along d
  const T* v[3];   // tangent direction / adjoint input
  T* dph[3];       // cell velocity tangent / adjoint
  T* fl[3][3];     // face flux tangents / adjoints
  T* ct[3];        // cell totals (tangent) / tbar (adjoint)
  T* uadv[3];      // advecting-velocity adjoint
  T* out[3];
  T ix[3], vc[3], c15;  // 1/dx, 1/(Re dx^2), 1.5/dt in T
};
using A3Args = A3T<double>;

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

// mixed-precision refinement of a Jacobian solve op(J) x = b: the FP64
// residual r = b - op(J) x (op in FP64) rounded to FP32, an inner FP32
// BiCGStab for op(J) d = r, x += d
struct Ref3 {
  Geom g;
  const double* b[3];
  const double* v[3];  // op(J) x
  float* r32[3];
  double* x[3];
  const float* d[3];
  double* sc;          // sc[kRfRR] = max |r|, sc[kRfBB] = max |b|
  double* part;
  unsigned* counter;
};
enum RefScalar { kRfRR = kBcN, kRfBB = kBcN + 1, kRfN = kBcN + 2 };

struct Bcg3f {
  Geom g;
  float* x[3];
  float* r[3];
  float* rh[3];
  float* p[3];
  float* v[3];
  float* s[3];
  float* t[3];
  const float* b[3];
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

template <typename T>
__device__ __forceinline__ T qleft3(T e, T c, T b) { return (T)-0.125 * e + (T)0.75 * c + (T)0.375 * b; }
template <typename T>
__device__ __forceinline__ T qright3(T c, T b, T a) { return (T)0.375 * c + (T)0.75 * b - (T)0.125 * a; }

// QUICK interpolant at face f along d of a cell field x, switch from u
template <typename T>
__device__ __forceinline__ T quick_at(const Geom& g, const T* x, int i, int j, int k, int d, T u) {
  if (u > (T)0) return qleft3(x[wid(g, i, j, k, d, -2)], x[wid(g, i, j, k, d, -1)], x[id3(g, i, j, k)]);
  return qright3(x[wid(g, i, j, k, d, -1)], x[id3(g, i, j, k)], x[wid(g, i, j, k, d, 1)]);
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_base_cells(A3T<T> A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.phb[m][id] = (T)0.5 * (A.us[m][id] + A.us[m][wid(A.g, i, j, k, m, 1)]);
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_base_q(A3T<T> A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    const T u = A.us[d][id];
    for (int m = 0; m < 3; ++m) A.q[d][m][id] = quick_at(A.g, (const T*)A.phb[m], i, j, k, d, u);
  }
}

// ---- tangent ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k3a_jv_cells(A3T<T> A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.dph[m][id] = (T)0.5 * (A.v[m][id] + A.v[m][wid(A.g, i, j, k, m, 1)]);
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_jv_flux(A3T<T> A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    const T u = A.us[d][id], du = A.v[d][id];
    for (int m = 0; m < 3; ++m) A.fl[d][m][id] = du * A.q[d][m][id] + u * quick_at(A.g, (const T*)A.dph[m], i, j, k, d, u);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_jv_total(A3T<T> A) {
  NS3A_IJK
  const Geom& g = A.g;
  for (int m = 0; m < 3; ++m) {
    const T* x = A.dph[m];
    const T c = x[id];
    T visc = (T)0, conv = (T)0;
    for (int d = 0; d < 3; ++d) {
      visc += (x[wid(g, i, j, k, d, 1)] - (T)2 * c + x[wid(g, i, j, k, d, -1)]) * A.vc[d];
      conv += (A.fl[d][m][wid(g, i, j, k, d, 1)] - A.fl[d][m][id]) * A.ix[d];
    }
    A.ct[m][id] = visc - conv;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_jv_faces(A3T<T> A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m)
    A.out[m][id] = (T)0.5 * (A.ct[m][wid(A.g, i, j, k, m, -1)] + A.ct[m][id]) - A.c15 * A.v[m][id];
}

// ---- adjoint ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k3a_vj_tbar(A3T<T> A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m) A.ct[m][id] = (T)0.5 * (A.v[m][id] + A.v[m][wid(A.g, i, j, k, m, 1)]);
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_vj_flux(A3T<T> A) {
  NS3A_IJK
  for (int d = 0; d < 3; ++d) {
    T ua = (T)0;
    for (int m = 0; m < 3; ++m) {
      const T fb = (A.ct[m][id] - A.ct[m][wid(A.g, i, j, k, d, -1)]) * A.ix[d];
      A.fl[d][m][id] = fb;
      ua += fb * A.q[d][m][id];
    }
    A.uadv[d][id] = ua;
  }
}

// weight of cell offset o (cell - face) in the face's QUICK interpolant
template <typename T>
__device__ __forceinline__ T quick_w3(bool pos, int o) {
  if (pos) return o == -2 ? (T)-0.125 : (o == -1 ? (T)0.75 : (o == 0 ? (T)0.375 : (T)0));
  return o == -1 ? (T)0.375 : (o == 0 ? (T)0.75 : (o == 1 ? (T)-0.125 : (T)0));
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_vj_cells(A3T<T> A) {
  NS3A_IJK
  const Geom& g = A.g;
  for (int m = 0; m < 3; ++m) {
    const T* tb = A.ct[m];
    const T c = tb[id];
    T s = (T)0;
    for (int d = 0; d < 3; ++d) {
      s += (tb[wid(g, i, j, k, d, 1)] - (T)2 * c + tb[wid(g, i, j, k, d, -1)]) * A.vc[d];
      for (int f = -1; f <= 2; ++f) {  // faces (along d) whose stencil holds this cell
        const long fid = wid(g, i, j, k, d, f);
        const T u = A.us[d][fid];
        s += A.fl[d][m][fid] * u * quick_w3<T>(u > (T)0, -f);
      }
    }
    A.dph[m][id] = s;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k3a_vj_faces(A3T<T> A) {
  NS3A_IJK
  for (int m = 0; m < 3; ++m)
    A.out[m][id] = A.uadv[m][id] + (T)0.5 * (A.dph[m][wid(A.g, i, j, k, m, -1)] + A.dph[m][id]) - A.c15 * A.v[m][id];
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

// ---- mixed-precision refinement -------------------------------------------------------------
#define REF3_PROLOGUE                                                                                          \
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z; \
  const bool in = i < A.g.N && j < A.g.N && k < A.g.N;                                                         \
  const long id = in ? id3(A.g, i, j, k) : 0;

__global__ void __launch_bounds__(256) k3r_to_f32(Geom g, const double* x0, const double* x1, const double* x2, float* y0,
                                                  float* y1, float* y2) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= g.N || j >= g.N || k >= g.N) return;
  const long id = id3(g, i, j, k);
  y0[id] = (float)x0[id];
  y1[id] = (float)x1[id];
  y2[id] = (float)x2[id];
}

// max |b - op(J) x| and max |b| (max norms: no squares to underflow in FP32)
__global__ void __launch_bounds__(256) k3r_resmax(Ref3 A) {
  REF3_PROLOGUE
  float red[2] = {0.f, 0.f};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const double b = A.b[m][id];
      red[0] = fmaxf(red[0], (float)fabs(b - A.v[m][id]));
      red[1] = fmaxf(red[1], (float)fabs(b));
    }
  double out[2];
  if (grid_reduce_last_f<2, 256>(red, reinterpret_cast<float2*>(A.part), A.counter, 3u, out) && threadIdx.x == 0) {
    A.sc[kRfRR] = out[0];
    A.sc[kRfBB] = out[1];
  }
}

// r32 = (b - op(J) x) / max |r|: the right-hand side of the inner solve, O(1)
__global__ void __launch_bounds__(256) k3r_scaled(Ref3 A, double inv) {
  REF3_PROLOGUE
  if (!in) return;
  for (int m = 0; m < 3; ++m) A.r32[m][id] = (float)((A.b[m][id] - A.v[m][id]) * inv);
}

// x += max |r| d
__global__ void __launch_bounds__(256) k3r_update(Ref3 A, double scale) {
  REF3_PROLOGUE
  if (!in) return;
  for (int m = 0; m < 3; ++m) A.x[m][id] += scale * (double)A.d[m][id];
}
#undef REF3_PROLOGUE

// ---- BiCGStab in FP32 (the inner solves), from x = 0 ------------------------------------------
#define BCGF_PROLOGUE                                                                                          \
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z; \
  const bool in = i < A.g.N && j < A.g.N && k < A.g.N;                                                         \
  const long id = in ? id3(A.g, i, j, k) : 0;

__global__ void __launch_bounds__(256) k3c_init(Bcg3f A) {
  BCGF_PROLOGUE
  float red[1] = {0.f};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const float r = A.b[m][id];
      A.x[m][id] = 0.f;
      A.r[m][id] = r;
      A.rh[m][id] = r;
      A.p[m][id] = r;
      red[0] += r * r;
    }
  double out[1];
  if (grid_reduce_last_f<1, 256>(red, reinterpret_cast<float2*>(A.part), A.counter, 0u, out) && threadIdx.x == 0) {
    double* sc = A.sc;
    sc[kBcRho] = out[0];
    sc[kBcAlpha] = 1.0;
    sc[kBcOmega] = 1.0;
    sc[kBcBeta] = 0.0;
    sc[kBcRR] = out[0];
    sc[kBcRR0] = out[0];
    sc[kBcBB] = out[0];
    sc[kBcBreak] = 0.0;
  }
}

__global__ void __launch_bounds__(256) k3c_alpha(Bcg3f A) {
  BCGF_PROLOGUE
  float red[1] = {0.f};
  if (in)
    for (int m = 0; m < 3; ++m) red[0] += A.rh[m][id] * A.v[m][id];
  double out[1];
  if (grid_reduce_last_f<1, 256>(red, reinterpret_cast<float2*>(A.part), A.counter, 0u, out) && threadIdx.x == 0) {
    double* sc = A.sc;
    if (out[0] != 0.0 && isfinite(out[0])) sc[kBcAlpha] = sc[kBcRho] / out[0];
    else { sc[kBcAlpha] = 0.0; sc[kBcBreak] = 1.0; }
  }
}

__global__ void __launch_bounds__(256) k3c_s(Bcg3f A) {
  BCGF_PROLOGUE
  if (!in) return;
  const float al = (float)A.sc[kBcAlpha];
  for (int m = 0; m < 3; ++m) A.s[m][id] = A.r[m][id] - al * A.v[m][id];
}

__global__ void __launch_bounds__(256) k3c_omega(Bcg3f A) {
  BCGF_PROLOGUE
  float red[2] = {0.f, 0.f};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const float t = A.t[m][id];
      red[0] += t * A.s[m][id];
      red[1] += t * t;
    }
  double out[2];
  if (grid_reduce_last_f<2, 256>(red, reinterpret_cast<float2*>(A.part), A.counter, 0u, out) && threadIdx.x == 0) {
    double* sc = A.sc;
    sc[kBcOmega] = out[1] > 0.0 ? out[0] / out[1] : 0.0;
    if (sc[kBcOmega] == 0.0) sc[kBcBreak] = 2.0;
  }
}

__global__ void __launch_bounds__(256) k3c_xr(Bcg3f A) {
  BCGF_PROLOGUE
  const float al = (float)A.sc[kBcAlpha], om = (float)A.sc[kBcOmega];
  float red[2] = {0.f, 0.f};
  if (in)
    for (int m = 0; m < 3; ++m) {
      const float s = A.s[m][id];
      A.x[m][id] += al * A.p[m][id] + om * s;
      const float r = s - om * A.t[m][id];
      A.r[m][id] = r;
      red[0] += A.rh[m][id] * r;
      red[1] += r * r;
    }
  double out[2];
  if (grid_reduce_last_f<2, 256>(red, reinterpret_cast<float2*>(A.part), A.counter, 0u, out) && threadIdx.x == 0) {
    double* sc = A.sc;
    const double rho = sc[kBcRho], al64 = sc[kBcAlpha], om64 = sc[kBcOmega];
    sc[kBcBeta] = (rho != 0.0 && om64 != 0.0) ? (out[0] / rho) * (al64 / om64) : 0.0;
    if (rho == 0.0) sc[kBcBreak] = 3.0;
    sc[kBcRho] = out[0];
    sc[kBcRR] = out[1];
  }
}

__global__ void __launch_bounds__(256) k3c_p(Bcg3f A) {
  BCGF_PROLOGUE
  if (!in) return;
  const float be = (float)A.sc[kBcBeta], om = (float)A.sc[kBcOmega];
  for (int m = 0; m < 3; ++m) A.p[m][id] = A.r[m][id] + be * (A.p[m][id] - om * A.v[m][id]);
}
#undef BCGF_PROLOGUE

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
