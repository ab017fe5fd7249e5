// Step-begin, Poisson right-hand side (P1) and projection (P2) kernels, 2D.
#pragma once
#include "ns_common.cuh"

namespace ns {

struct ProjArgs {
  Geom g;
  const double* u[2];     // velocity (faces)
  const double* uprev[2];
  double* du[2];
  double* S[2];           // fast/mixed: step-constant source
  const double* p;
  double* pw;             // p (written by P2)
  const double* phi;
  double* uout[2];
  double* f;              // Poisson RHS (cells)
  double* part;
  unsigned* counter;
  double* red_out;        // reduction results
};

// main.cpp:879-884: du = u^n - u^{n-1}; with the fast source also
// S = (-grad p + (0.5/dt) du) + (1.5/dt) u^n, grad p with mirrored / wrapped ghosts.
template <class AR, bool WITH_S>
__global__ void __launch_bounds__(256) k_step_begin2d(ProjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const long nu = (long)(N + 1) * N;  // faces per direction
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * nu; t += (long)gridDim.x * blockDim.x) {
    const int m = (t < nu) ? 0 : 1;
    const long q = (m == 0) ? t : t - nu;
    int a, b;
    if (m == 0) { a = (int)(q % (N + 1)); b = (int)(q / (N + 1)); }
    else { a = (int)(q % N); b = (int)(q / N); }
    const long id = (long)b * P + a;
    const double un = A.u[m][id];
    const double d = un - A.uprev[m][id];
    A.du[m][id] = d;
    if (WITH_S) {
      int ci = (m == 0) ? a : b, pi = ci - 1;
      if (ci == N) ci = g.ctx_mirror[m] ? N - 1 : 0;
      if (pi < 0) pi = g.ctx_mirror[m] ? 0 : N - 1;
      const double pc = (m == 0) ? A.p[(long)b * P + ci] : A.p[(long)ci * P + a];
      const double pm = (m == 0) ? A.p[(long)b * P + pi] : A.p[(long)pi * P + a];
      const double gp = AR::div(pc - pm, g.dx[m], g.inv_dx[m]);
      A.S[m][id] = (-gp + g.c05 * d) + g.c15 * un;
    }
  }
}

// poisson_righthand_side_calc (fn_rhs.cpp:71-125): f = (1.5/dt) div u, and the
// reductions max|div u| (norm0) and sum f. red_out = {max|div|, sum f}.
template <class AR>
__global__ void __launch_bounds__(256) k_poisson_rhs2d(ProjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  double v[2] = {0.0, 0.0};
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i < N && j < N) {
    const long id = (long)j * P + i;
    const double div = AR::div(A.u[0][id + 1] - A.u[0][id], g.dx[0], g.inv_dx[0]) +
                       AR::div(A.u[1][id + P] - A.u[1][id], g.dx[1], g.inv_dx[1]);
    v[0] = fabs(div);
    const double f = g.c15 * div;
    A.f[id] = f;
    v[1] = f;
  }
  if (grid_reduce_last<2>(v, A.part, A.counter, 1u) && threadIdx.x == 0) {
    A.red_out[0] = v[0];
    A.red_out[1] = v[1];
  }
}

// update_solution (poisson.cpp:192-392) with the phi ghost mirror of
// main.cpp:1078-1158: u = u* - (grad phi * dt / 1.5); p += phi; then the
// post-step divergence check (main.cpp:1180). One thread per cell computes the
// cell's low faces (and the domain's last face) plus the high faces it needs
// for the divergence. red_out = {max|div u|}.
template <class AR>
__global__ void __launch_bounds__(256) k_project2d(ProjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  double v[1] = {0.0};
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i < N && j < N) {
    const double dt = g.dt;
    auto face = [&](int m, int a, int b) -> double {
      // x-face (m=0) at (a,b) or y-face (m=1)
      int ci = (m == 0) ? a : b, pi = ci - 1;
      if (ci == N) ci = g.ctx_mirror[m] ? N - 1 : 0;
      if (pi < 0) pi = g.ctx_mirror[m] ? 0 : N - 1;
      const double pc = (m == 0) ? A.phi[(long)b * P + ci] : A.phi[(long)ci * P + a];
      const double pm = (m == 0) ? A.phi[(long)b * P + pi] : A.phi[(long)pi * P + a];
      const double gphi = AR::div(pc - pm, g.dx[m], g.inv_dx[m]);
      return A.u[m][(long)b * P + a] - AR::div(gphi * dt, 1.5, 1.0 / 1.5);
    };
    const long id = (long)j * P + i;
    const double u0 = face(0, i, j), u1 = face(0, i + 1, j);
    const double v0 = face(1, i, j), v1 = face(1, i, j + 1);
    A.uout[0][id] = u0;
    A.uout[1][id] = v0;
    if (i == N - 1) A.uout[0][id + 1] = u1;
    if (j == N - 1) A.uout[1][id + P] = v1;
    A.pw[id] = A.p[id] + A.phi[id];
    const double div = AR::div(u1 - u0, g.dx[0], g.inv_dx[0]) + AR::div(v1 - v0, g.dx[1], g.inv_dx[1]);
    v[0] = fabs(div);
  }
  if (grid_reduce_last<1>(v, A.part, A.counter, 1u) && threadIdx.x == 0) A.red_out[0] = v[0];
}

}  // namespace ns
