// Tangent-linear and adjoint operators of one time step (2D, FP64).
//
// The predictor's converged state u* solves G(u*) = 0 with
//   G(u) = -grad p^n + A(u; lid) - (1.5/dt)(u - u^n) + (0.5/dt)(u^n - u^{n-1}),
// A = face average of (-conv_QUICK + visc) (main.cpp:931-1017). With the
// upwind switches frozen at u*, the Jacobian J = dA/du - (1.5/dt) I acts on
// interior faces (boundary-face velocities are fixed by Q4 and carry no
// tangent). This file holds:
//   jvp:  (J v + dA/dlid dlid) by four gather passes (cell velocity tangent,
//         face flux tangent, cell total tangent, face average),
//   vjp:  J^T w (and the lid adjoint) by the transposed passes.
// The wall / lid cavity is supported (every ghost rule of utilities.cpp:62-349
// except periodic wrap). Ghosted cell arrays hold cells [-2, N+1]^2 with row
// stride N+4.
#pragma once
#include "ns_common.cuh"

namespace ns {

struct AdjArgs {
  Geom g;
  const double* us[2];   // base state u* (faces)
  double* phi[2];        // ghosted cell velocity of u* (filled by k_adj_cart)
  // tangent
  const double* v[2];    // direction (faces)
  const double* dlid;    // lid tangent per column (nullable)
  double* dphi[2];       // ghosted tangent cell velocity
  double* dF[4];         // face flux tangents: x faces comp 0/1, y faces comp 0/1
  double* dt_[2];        // cell total tangent
  double* out[2];        // J v (faces)
  // adjoint
  const double* w[2];    // adjoint input (faces)
  double* tbar[2];       // cell total adjoint
  double* Fbar[4];       // face flux adjoints (x faces comp 0/1, y faces comp 0/1)
  double* uadv[2];       // advecting-velocity adjoint (faces)
  double* phibar[2];     // ghosted cell velocity adjoint
  double* lidbar;        // per-column lid adjoint (nullable)
};

// ---- BiCGStab on the interior faces (device-resident scalars) -----------------------
// The linearised predictor J x = b (tangent) or J^T x = b (adjoint) is solved by
// BiCGStab instead of the pseudo-time iteration: J = dA/du - (1.5/dt) I is the
// Jacobian of the converged predictor, and the solution is the same; the
// Krylov solve needs several times fewer operator applications.
enum BcgScalar { kBcRho = 0, kBcAlpha = 1, kBcOmega = 2, kBcBeta = 3, kBcRR = 4, kBcBB = 5, kBcBreak = 6, kBcRR0 = 7, kBcN = 8 };

struct BcgArgs {
  Geom g;
  double* x[2];
  double* r[2];
  double* rh[2];  // shadow residual
  double* p[2];
  double* v[2];   // A p
  double* s[2];
  double* t[2];   // A s
  const double* b[2];
  double* sc;     // kBcN device scalars
  double* part;
  unsigned* counter;
};

__host__ __device__ __forceinline__ long gidx(int i, int j, int N) { return (long)(i + 2) + (long)(j + 2) * (N + 4); }

#ifndef NS_ADJOINT_ARGS_ONLY
// sign of the ghost rule for comp m on side s (kNeg/kInlet: -1, kPos: +1)
__device__ __forceinline__ double ghost_sign(const Geom& g, int side, int m) { return g.bc[side].rule[m] == kPos ? 1.0 : -1.0; }

// ghosted cell velocity from faces (cont2cart + wall/lid ghosts); tangent
// version when homogeneous (ghost = s*q, lid part 2*dlid)
__device__ __forceinline__ double cell_vel(const Geom& g, const double* u0, const double* u1, int m, int i, int j) {
  const long P = g.pitch;
  return (m == 0) ? 0.5 * (u0[(long)j * P + i] + u0[(long)j * P + i + 1]) : 0.5 * (u1[(long)j * P + i] + u1[(long)(j + 1) * P + i]);
}

__global__ void k_adj_cart(Geom g, const double* s0, const double* s1, double* d0, double* d1, const double* lid,
                           int homogeneous) {
  const int N = g.N;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 2;
  const int j = (int)blockIdx.y - 2;
  if (i > N + 1 || j > N + 1) return;
  for (int m = 0; m < 2; ++m) {
    double val = 0.0;
    const bool inx = i >= 0 && i < N, iny = j >= 0 && j < N;
    if (inx && iny) {
      val = cell_vel(g, s0, s1, m, i, j);
    } else if (iny && !inx) {  // x ghosts
      const int side = i < 0 ? 0 : 1;
      const int mi = i < 0 ? -i - 1 : 2 * N - 1 - i;
      const double q = cell_vel(g, s0, s1, m, mi, j);
      const CartBC& b = g.bc[side];
      val = (b.rule[m] == kInlet) ? (homogeneous ? -q : b.add[m] - q) : (b.rule[m] == kNeg ? -q : q);
    } else if (inx && !iny) {  // y ghosts
      const int side = j < 0 ? 2 : 3;
      const int mj = j < 0 ? -j - 1 : 2 * N - 1 - j;
      const double q = cell_vel(g, s0, s1, m, i, mj);
      const CartBC& b = g.bc[side];
      if (b.rule[m] == kInlet) {
        double add = b.add[m];
        if (side == 3 && m == 0 && lid != nullptr) add = 2 * lid[i];
        else if (homogeneous) add = 0.0;
        val = add - q;
      } else {
        val = (b.rule[m] == kNeg ? -q : q);
      }
    }
    (m == 0 ? d0 : d1)[gidx(i, j, N)] = val;
  }
}

// QUICK interpolations at a face: left (u>0) and right (u<=0) biased
__device__ __forceinline__ double qleft(double e, double c, double b) { return -0.125 * e + 0.75 * c + 0.375 * b; }
__device__ __forceinline__ double qright(double c, double b, double a) { return 0.375 * c + 0.75 * b - 0.125 * a; }

// ---- tangent -------------------------------------------------------------------
// pass 2: face flux tangents at interior faces
__global__ void k_jvp_flux(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  // x face (i, j): i in [1, N-1], j in [0, N)
  if (j < N && i >= 1 && i <= N - 1) {
    const long id = (long)j * P + i;
    const double u = A.us[0][id], du = A.v[0][id];
    for (int m = 0; m < 2; ++m) {
      const double* ph = A.phi[m];
      const double* dph = A.dphi[m];
      double r;
      if (u > 0) r = du * qleft(ph[gidx(i - 2, j, N)], ph[gidx(i - 1, j, N)], ph[gidx(i, j, N)]) +
                     u * qleft(dph[gidx(i - 2, j, N)], dph[gidx(i - 1, j, N)], dph[gidx(i, j, N)]);
      else r = du * qright(ph[gidx(i - 1, j, N)], ph[gidx(i, j, N)], ph[gidx(i + 1, j, N)]) +
               u * qright(dph[gidx(i - 1, j, N)], dph[gidx(i, j, N)], dph[gidx(i + 1, j, N)]);
      A.dF[m][id] = r;
    }
  }
  // y face (i, j): i in [0, N), j in [1, N-1]
  if (i < N && j >= 1 && j <= N - 1) {
    const long id = (long)j * P + i;
    const double v = A.us[1][id], dv = A.v[1][id];
    for (int m = 0; m < 2; ++m) {
      const double* ph = A.phi[m];
      const double* dph = A.dphi[m];
      double r;
      if (v > 0) r = dv * qleft(ph[gidx(i, j - 2, N)], ph[gidx(i, j - 1, N)], ph[gidx(i, j, N)]) +
                     v * qleft(dph[gidx(i, j - 2, N)], dph[gidx(i, j - 1, N)], dph[gidx(i, j, N)]);
      else r = dv * qright(ph[gidx(i, j - 1, N)], ph[gidx(i, j, N)], ph[gidx(i, j + 1, N)]) +
               v * qright(dph[gidx(i, j - 1, N)], dph[gidx(i, j, N)], dph[gidx(i, j + 1, N)]);
      A.dF[2 + m][id] = r;
    }
  }
}

// pass 3: cell total tangent dt = -dconv + dvisc (boundary-face fluxes are 0)
__global__ void k_jvp_total(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= N || j >= N) return;
  const double vx = g.inv_ren * g.inv_dx2[0], vy = g.inv_ren * g.inv_dx2[1];
  for (int m = 0; m < 2; ++m) {
    const double fxl = (i >= 1) ? A.dF[m][(long)j * P + i] : 0.0;
    const double fxr = (i + 1 <= N - 1) ? A.dF[m][(long)j * P + i + 1] : 0.0;
    const double fyl = (j >= 1) ? A.dF[2 + m][(long)j * P + i] : 0.0;
    const double fyr = (j + 1 <= N - 1) ? A.dF[2 + m][(long)(j + 1) * P + i] : 0.0;
    const double conv = (fxr - fxl) * g.inv_dx[0] + (fyr - fyl) * g.inv_dx[1];
    const double* d = A.dphi[m];
    const double c = d[gidx(i, j, N)];
    const double visc = (d[gidx(i + 1, j, N)] - 2 * c + d[gidx(i - 1, j, N)]) * vx + (d[gidx(i, j + 1, N)] - 2 * c + d[gidx(i, j - 1, N)]) * vy;
    A.dt_[m][(long)j * P + i] = visc - conv;
  }
}

// pass 4: J v at interior faces (boundary faces: 0)
__global__ void k_jvp_faces(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    A.out[0][id] = (i >= 1 && i <= N - 1) ? 0.5 * (A.dt_[0][id - 1] + A.dt_[0][id]) - g.c15 * A.v[0][id] : 0.0;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    A.out[1][id] = (j >= 1 && j <= N - 1) ? 0.5 * (A.dt_[1][id - P] + A.dt_[1][id]) - g.c15 * A.v[1][id] : 0.0;
  }
}

// ---- adjoint -------------------------------------------------------------------
// pass 1: cell total adjoint from the face adjoint (interior faces only: the
// odd flux reflection makes R = 0 at boundary faces, main.cpp:945-1014)
__global__ void k_vjp_tbar(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= N || j >= N) return;
  const long id = (long)j * P + i;
  const double wl = (i >= 1) ? A.w[0][id] : 0.0, wr = (i + 1 <= N - 1) ? A.w[0][id + 1] : 0.0;
  const double ws = (j >= 1) ? A.w[1][id] : 0.0, wn = (j + 1 <= N - 1) ? A.w[1][id + P] : 0.0;
  A.tbar[0][id] = 0.5 * (wl + wr);
  A.tbar[1][id] = 0.5 * (ws + wn);
}

// pass 2: face flux adjoints and the advecting-velocity adjoint
__global__ void k_vjp_flux(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    double ua = 0.0;
    if (i >= 1 && i <= N - 1) {
      const double u = A.us[0][id];
      for (int m = 0; m < 2; ++m) {
        const double fb = (A.tbar[m][id] - A.tbar[m][id - 1]) * g.inv_dx[0];  // conv_bar = -tbar
        A.Fbar[m][id] = fb;
        const double* ph = A.phi[m];
        const double q = (u > 0) ? qleft(ph[gidx(i - 2, j, N)], ph[gidx(i - 1, j, N)], ph[gidx(i, j, N)])
                                 : qright(ph[gidx(i - 1, j, N)], ph[gidx(i, j, N)], ph[gidx(i + 1, j, N)]);
        ua += fb * q;
      }
    } else {
      A.Fbar[0][id] = 0.0;
      A.Fbar[1][id] = 0.0;
    }
    A.uadv[0][id] = ua;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    double va = 0.0;
    if (j >= 1 && j <= N - 1) {
      const double v = A.us[1][id];
      for (int m = 0; m < 2; ++m) {
        const double fb = (A.tbar[m][id] - A.tbar[m][id - P]) * g.inv_dx[1];
        A.Fbar[2 + m][id] = fb;
        const double* ph = A.phi[m];
        const double q = (v > 0) ? qleft(ph[gidx(i, j - 2, N)], ph[gidx(i, j - 1, N)], ph[gidx(i, j, N)])
                                 : qright(ph[gidx(i, j - 1, N)], ph[gidx(i, j, N)], ph[gidx(i, j + 1, N)]);
        va += fb * q;
      }
    } else {
      A.Fbar[2][id] = 0.0;
      A.Fbar[3][id] = 0.0;
    }
    A.uadv[1][id] = va;
  }
}

// QUICK weight of cell offset k (cell - face index) in the face value:
// u>0: cells i-2, i-1, i -> -1/8, 3/4, 3/8; u<=0: cells i-1, i, i+1 -> 3/8, 3/4, -1/8
__device__ __forceinline__ double quick_w(bool pos, int k) {
  if (pos) return k == -2 ? -0.125 : (k == -1 ? 0.75 : (k == 0 ? 0.375 : 0.0));
  return k == -1 ? 0.375 : (k == 0 ? 0.75 : (k == 1 ? -0.125 : 0.0));
}

// pass 3: ghosted cell velocity adjoint (viscous + QUICK transport)
__global__ void k_vjp_phibar(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 2;
  const int j = (int)blockIdx.y - 2;
  if (i > N + 1 || j > N + 1) return;
  const double vx = g.inv_ren * g.inv_dx2[0], vy = g.inv_ren * g.inv_dx2[1];
  auto tb = [&](int m, int a, int b) -> double {
    return (a >= 0 && a < N && b >= 0 && b < N) ? A.tbar[m][(long)b * P + a] : 0.0;
  };
  for (int m = 0; m < 2; ++m) {
    double s = (tb(m, i - 1, j) + tb(m, i + 1, j) - 2 * tb(m, i, j)) * vx + (tb(m, i, j - 1) + tb(m, i, j + 1) - 2 * tb(m, i, j)) * vy;
    if (j >= 0 && j < N) {
      for (int f = i - 1; f <= i + 2; ++f) {  // x faces whose stencil holds cell i
        if (f < 1 || f > N - 1) continue;
        const long id = (long)j * P + f;
        const double u = A.us[0][id];
        s += A.Fbar[m][id] * u * quick_w(u > 0, i - f);
      }
    }
    if (i >= 0 && i < N) {
      for (int f = j - 1; f <= j + 2; ++f) {  // y faces whose stencil holds cell j
        if (f < 1 || f > N - 1) continue;
        const long id = (long)f * P + i;
        const double v = A.us[1][id];
        s += A.Fbar[2 + m][id] * v * quick_w(v > 0, j - f);
      }
    }
    A.phibar[m][gidx(i, j, N)] = s;
  }
}

// cell velocity adjoint of an interior cell after folding its ghost images
__device__ __forceinline__ double phibar_folded(const AdjArgs& A, int m, int i, int j) {
  const Geom& g = A.g;
  const int N = g.N;
  const double* pb = A.phibar[m];
  double s = pb[gidx(i, j, N)];
  if (i <= 1) s += ghost_sign(g, 0, m) * pb[gidx(-i - 1, j, N)];
  if (i >= N - 2) s += ghost_sign(g, 1, m) * pb[gidx(2 * N - 1 - i, j, N)];
  if (j <= 1) s += ghost_sign(g, 2, m) * pb[gidx(i, -j - 1, N)];
  if (j >= N - 2) s += ghost_sign(g, 3, m) * pb[gidx(i, 2 * N - 1 - j, N)];
  return s;
}

// pass 4: J^T w at interior faces, and the lid adjoint per column
__global__ void k_vjp_faces(AdjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    A.out[0][id] = (i >= 1 && i <= N - 1)
                       ? A.uadv[0][id] + 0.5 * (phibar_folded(A, 0, i - 1, j) + phibar_folded(A, 0, i, j)) - g.c15 * A.w[0][id]
                       : 0.0;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    A.out[1][id] = (j >= 1 && j <= N - 1)
                       ? A.uadv[1][id] + 0.5 * (phibar_folded(A, 1, i, j - 1) + phibar_folded(A, 1, i, j)) - g.c15 * A.w[1][id]
                       : 0.0;
  }
  if (A.lidbar != nullptr && j == 0 && i < N)  // ghost = 2 lid - q on rows N, N+1
    A.lidbar[i] = 2.0 * (A.phibar[0][gidx(i, N, N)] + A.phibar[0][gidx(i, N + 1, N)]);
}

// ---- projection pieces ------------------------------------------------------------
// f = D u + coef * pb over interior faces (boundary faces carry no tangent or
// adjoint), with sum f reduced into sum_out and max |f| into max_out (nullable)
__global__ void __launch_bounds__(256) k_adj_div(Geom g, const double* u0, const double* u1, const double* pb, double coef,
                                                 double* f, double* part, unsigned* counter, double* sum_out,
                                                 double* max_out) {
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  double v[2] = {0.0, 0.0};
  if (i < N && j < N) {
    const long id = (long)j * P + i;
    const double ul = (i >= 1) ? u0[id] : 0.0, ur = (i + 1 <= N - 1) ? u0[id + 1] : 0.0;
    const double vs = (j >= 1) ? u1[id] : 0.0, vn = (j + 1 <= N - 1) ? u1[id + P] : 0.0;
    double r = (ur - ul) * g.inv_dx[0] + (vn - vs) * g.inv_dx[1];
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

// out = in - coef * grad(psi) on interior faces (mirror ghosts: zero gradient
// on boundary faces), boundary faces of out set to bnd
__global__ void k_adj_gradsub(Geom g, const double* in0, const double* in1, const double* psi, double coef, double* o0,
                              double* o1) {
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    o0[id] = (i >= 1 && i <= N - 1) ? in0[id] - coef * (psi[id] - psi[id - 1]) * g.inv_dx[0] : 0.0;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    o1[id] = (j >= 1 && j <= N - 1) ? in1[id] - coef * (psi[id] - psi[id - P]) * g.inv_dx[1] : 0.0;
  }
}

// out = a * x + b * y on interior faces (y nullable), 0 on boundary faces
__global__ void k_adj_lincomb(Geom g, double a, const double* x0, const double* x1, double b, const double* y0,
                              const double* y1, double* o0, double* o1) {
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    o0[id] = (i >= 1 && i <= N - 1) ? a * x0[id] + (y0 ? b * y0[id] : 0.0) : 0.0;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    o1[id] = (j >= 1 && j <= N - 1) ? a * x1[id] + (y1 ? b * y1[id] : 0.0) : 0.0;
  }
}

// cells: out = a * x + b * y (y nullable)
__global__ void k_adj_cells(Geom g, double a, const double* x, double b, const double* y, double* o) {
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i < N && j < N) {
    const long id = (long)j * P + i;
    o[id] = a * x[id] + (y ? b * y[id] : 0.0);
  }
}

// ---- right-hand side of the linearised predictor ----------------------------------
// b = -(dA/dlid dlid - G dp + (2/dt) du - (0.5/dt) du_prev) on interior faces: the
// derivative of the source S = -grad p + (0.5/dt)(u - u_prev) + (1.5/dt) u and of
// the lid ghost (jl = jvp(v = 0, dlid), nullable)
__global__ void k_tlm_rhs(Geom g, const double* jl0, const double* jl1, const double* dp, const double* du0, const double* du1,
                          const double* dup0, const double* dup1, double* o0, double* o1) {
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  const double c2 = g.c15 + g.c05;
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    double r = 0.0;
    if (i >= 1 && i <= N - 1)
      r = -((jl0 ? jl0[id] : 0.0) - (dp[id] - dp[id - 1]) * g.inv_dx[0] + c2 * du0[id] - g.c05 * dup0[id]);
    o0[id] = r;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    double r = 0.0;
    if (j >= 1 && j <= N - 1)
      r = -((jl1 ? jl1[id] : 0.0) - (dp[id] - dp[id - P]) * g.inv_dx[1] + c2 * du1[id] - g.c05 * dup1[id]);
    o1[id] = r;
  }
}

// interior-face test of component m at (i, j)
__device__ __forceinline__ bool bcg_face(int N, int m, int i, int j) {
  return (m == 0) ? (j < N && i >= 1 && i <= N - 1) : (i < N && j >= 1 && j <= N - 1);
}

#define BCG_PROLOGUE                                                                    \
  const int N = A.g.N;                                                                  \
  const long P = A.g.pitch;                                                             \
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5); \
  const long id = (long)j * P + i;

// r = b - v (v = A x0), rh = r, p = r; rr = (r, r), bb = (b, b)
__global__ void __launch_bounds__(256) k_bcg_init(BcgArgs A) {
  BCG_PROLOGUE
  double red[2] = {0.0, 0.0};
  for (int m = 0; m < 2; ++m) {
    if (!bcg_face(N, m, i, j)) continue;
    const double bb = A.b[m][id];
    const double r = bb - A.v[m][id];
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

// alpha = rho / (rh, v)
__global__ void __launch_bounds__(256) k_bcg_alpha(BcgArgs A) {
  BCG_PROLOGUE
  double red[1] = {0.0};
  for (int m = 0; m < 2; ++m)
    if (bcg_face(N, m, i, j)) red[0] += A.rh[m][id] * A.v[m][id];
  if (grid_reduce_last<1>(red, A.part, A.counter, 0u) && threadIdx.x == 0) {
    double* sc = A.sc;
    if (red[0] != 0.0 && isfinite(red[0])) {
      sc[kBcAlpha] = sc[kBcRho] / red[0];
    } else {
      sc[kBcAlpha] = 0.0;
      sc[kBcBreak] = 1.0;
    }
  }
}

// s = r - alpha v
__global__ void __launch_bounds__(256) k_bcg_s(BcgArgs A) {
  BCG_PROLOGUE
  const double al = A.sc[kBcAlpha];
  for (int m = 0; m < 2; ++m)
    if (bcg_face(N, m, i, j)) A.s[m][id] = A.r[m][id] - al * A.v[m][id];
}

// omega = (t, s) / (t, t)
__global__ void __launch_bounds__(256) k_bcg_omega(BcgArgs A) {
  BCG_PROLOGUE
  double red[2] = {0.0, 0.0};
  for (int m = 0; m < 2; ++m)
    if (bcg_face(N, m, i, j)) {
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

// x += alpha p + omega s; r = s - omega t; beta = (rho'/rho)(alpha/omega)
__global__ void __launch_bounds__(256) k_bcg_xr(BcgArgs A) {
  BCG_PROLOGUE
  const double al = A.sc[kBcAlpha], om = A.sc[kBcOmega];
  double red[2] = {0.0, 0.0};
  for (int m = 0; m < 2; ++m)
    if (bcg_face(N, m, i, j)) {
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

// p = r + beta (p - omega v)
__global__ void __launch_bounds__(256) k_bcg_p(BcgArgs A) {
  BCG_PROLOGUE
  const double be = A.sc[kBcBeta], om = A.sc[kBcOmega];
  for (int m = 0; m < 2; ++m)
    if (bcg_face(N, m, i, j)) A.p[m][id] = A.r[m][id] + be * (A.p[m][id] - om * A.v[m][id]);
}

#undef BCG_PROLOGUE

// ---- objective: kinetic energy of the lower-left quarter --------------------------
// J = 1/2 sum_{i < N/2, j < N/2} (phi_u^2 + phi_v^2) dx dy with the cell-centred
// velocity phi of cont2cart (utilities.cpp:661 evaluates the same cell average)
__global__ void __launch_bounds__(256) k_adj_objective(Geom g, const double* u0, const double* u1, double* part,
                                                       unsigned* counter, double* red_out) {
  const int N = g.N, H = N / 2;
  const long P = g.pitch;
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  double v[1] = {0.0};
  if (i < H && j < H) {
    const long id = (long)j * P + i;
    const double a = 0.5 * (u0[id] + u0[id + 1]), b = 0.5 * (u1[id] + u1[id + P]);
    v[0] = 0.5 * (a * a + b * b) * g.dx[0] * g.dx[1];
  }
  if (grid_reduce_last<1>(v, part, counter, 0u) && threadIdx.x == 0) red_out[0] = v[0];
}

// dJ/du on the faces (boundary faces carry no adjoint)
__global__ void k_adj_objective_grad(Geom g, const double* u0, const double* u1, double* o0, double* o1) {
  const int N = g.N, H = N / 2;
  const long P = g.pitch;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  const double w = 0.5 * g.dx[0] * g.dx[1];
  if (j < N && i <= N) {
    const long id = (long)j * P + i;
    double r = 0.0;
    if (j < H && i >= 1 && i <= N - 1) {
      if (i - 1 < H) r += 0.5 * (u0[id - 1] + u0[id]) * w;
      if (i < H) r += 0.5 * (u0[id] + u0[id + 1]) * w;
    }
    o0[id] = r;
  }
  if (i < N && j <= N) {
    const long id = (long)j * P + i;
    double r = 0.0;
    if (i < H && j >= 1 && j <= N - 1) {
      if (j - 1 < H) r += 0.5 * (u1[id - P] + u1[id]) * w;
      if (j < H) r += 0.5 * (u1[id] + u1[id + P]) * w;
    }
    o1[id] = r;
  }
}

// ---- lid controls: piecewise-constant segments of N / nseg columns --------------------
__global__ void k_lid_expand(int N, int nseg, const double* seg, double* col) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) col[i] = seg[i / (N / nseg)];
}

// seg_acc[s] += coef * sum of the segment's column values (fixed order)
__global__ void k_lid_accum(int N, int nseg, const double* col, double coef, double* seg_acc) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int w = N / nseg;
  double a = 0.0;
  for (int k = 0; k < w; ++k) a += col[s * w + k];
  seg_acc[s] += coef * a;
}

#endif  // NS_ADJOINT_ARGS_ONLY

}  // namespace ns
