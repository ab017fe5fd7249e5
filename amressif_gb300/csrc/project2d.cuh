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
// Thread a of block row b takes the u face (a, b) (a <= N, b < N) and the v
// face (a, b) (a < N, b <= N): grid proj_face_grid(g).
template <class AR, bool WITH_S>
__global__ void __launch_bounds__(256) k_step_begin2d(ProjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int a = blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
  if (a > N) return;
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    if (m == 0 ? b >= N : a >= N) continue;
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

// one thread per face column a and row b of the (N+1) x (N+1) face index box
inline dim3 proj_face_grid(const Geom& g) { return dim3((unsigned)((g.N + 1 + 255) / 256), (unsigned)(g.N + 1), 1); }

// cell kernels below: a warp takes 32 columns and kProjRows rows, marching up
// them, so each face is evaluated once (the east face of a cell is the next
// lane's west face, the north face the next row's south face) and the FP64
// block reductions run once per kProjRows cells
constexpr int kProjRows = 8;
inline dim3 proj_grid(int n) { return dim3((unsigned)((n + 31) / 32), (unsigned)((n + 8 * kProjRows - 1) / (8 * kProjRows)), 1); }

// poisson_righthand_side_calc (fn_rhs.cpp:71-125): f = (1.5/dt) div u, and the
// reductions max|div u| (norm0) and sum f. red_out = {max|div|, sum f}.
// Grid proj_grid(N).
template <class AR>
__global__ void __launch_bounds__(256) k_poisson_rhs2d(ProjArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  double v[2] = {0.0, 0.0};
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j0 = (blockIdx.y * 8 + (threadIdx.x >> 5)) * kProjRows;
  if (i < N && j0 < N) {
    double vs = A.u[1][(long)j0 * P + i];  // south v face of the first row
    for (int r = 0; r < kProjRows; ++r) {
      const int j = j0 + r;
      if (j >= N) break;
      const long id = (long)j * P + i;
      const double vn = A.u[1][id + P];
      const double div = AR::div(A.u[0][id + 1] - A.u[0][id], g.dx[0], g.inv_dx[0]) +
                         AR::div(vn - vs, g.dx[1], g.inv_dx[1]);
      v[0] = fmax(v[0], fabs(div));
      const double f = g.c15 * div;
      A.f[id] = f;
      v[1] += f;
      vs = vn;
    }
  }
  if (grid_reduce_last<2>(v, A.part, A.counter, 1u) && threadIdx.x == 0) {
    A.red_out[0] = v[0];
    A.red_out[1] = v[1];
  }
}

// update_solution (poisson.cpp:192-392) with the phi ghost mirror of
// main.cpp:1078-1158: u = u* - (grad phi * dt / 1.5); p += phi; then the
// post-step divergence check (main.cpp:1180). A thread marches up kProjRows
// cells of its column: it evaluates the cell's west and south faces, takes the
// east face from the next lane (lane 31 and the domain's last column evaluate
// it) and the north face into the next row. red_out = {max|div u|}. Grid
// proj_grid(N).
template <class AR>
__global__ void __launch_bounds__(256) k_project2d(ProjArgs A) {
  constexpr unsigned FULL = 0xffffffffu;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  double v[1] = {0.0};
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 32 + lane;
  const int j0 = (blockIdx.y * 8 + (threadIdx.x >> 5)) * kProjRows;
  const bool in = i < N;
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
  if (j0 < N) {  // warp-uniform
    double v0 = in ? face(1, i, j0) : 0.0;
    for (int r = 0; r < kProjRows; ++r) {
      const int j = j0 + r;
      if (j >= N) break;  // warp-uniform
      const long id = (long)j * P + i;
      const double u0 = in ? face(0, i, j) : 0.0;
      const double ue = __shfl_down_sync(FULL, u0, 1);
      if (in) {
        const double u1 = (lane == 31 || i == N - 1) ? face(0, i + 1, j) : ue;
        const double v1 = face(1, i, j + 1);
        A.uout[0][id] = u0;
        A.uout[1][id] = v0;
        if (i == N - 1) A.uout[0][id + 1] = u1;
        if (j == N - 1) A.uout[1][id + P] = v1;
        A.pw[id] = A.p[id] + A.phi[id];
        const double div = AR::div(u1 - u0, g.dx[0], g.inv_dx[0]) + AR::div(v1 - v0, g.dx[1], g.inv_dx[1]);
        v[0] = fmax(v[0], fabs(div));
        v0 = v1;
      }
    }
  }
  if (grid_reduce_last<1>(v, A.part, A.counter, 1u) && threadIdx.x == 0) A.red_out[0] = v[0];
}

}  // namespace ns
