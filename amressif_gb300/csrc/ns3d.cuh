// Kernels of the 3D advance (AMREX_SPACEDIM = 3 build of the reference).
//
// Layout: every level-0 field is (N+1) planes x (N+1) rows x pitch P, element
// (i, j, k) at (k (N+1) + j) P + i; x faces u(i, j, k), i in [0, N], and so
// on. The predictor runs as four gather passes per RK stage (FP64):
//   k3_cart   ghosted cell velocity phi_m (cont2cart + wall / lid / periodic
//             ghosts, utilities.cpp:16-350) on [-2, N+1]^3,
//   k3_flux   QUICK fluxes of the three components at every face along the
//             three directions, each face once (fn_flux_calc.cpp:66-76),
//   k3_total  t_m = visc - conv at the cells (central viscous term; conv = 0
//             for convective_flux_calc, which never updates the total flux),
//   k3_face   G = S - (1.5/dt) u* + avg(t) with the flux-ghost rule of the
//             normal component (main.cpp:945-1014), the RK update and the
//             pseudo-norm of Error_Computation (utilities.cpp:421-493);
// the step source, the Poisson right-hand side and the projection as in 2D
// (project2d.cuh); a cell-centred 7-point geometric multigrid (red-black
// Gauss-Seidel, cell-average restriction, trilinear prolongation, Gauss-Seidel
// on the coarsest level in one block).
#pragma once
#include "ns_common.cuh"
#include "stage2d.cuh"

namespace ns {

struct Arg3 {
  Geom g;
  const double* u[3];    // current stage input u* (faces)
  const double* ub[3];   // pseudo-iteration base
  const double* un[3];   // u^n
  const double* uprev[3];
  double* du[3];
  double* S[3];          // step source
  double* out[3];        // RK stage output / projected velocity
  const double* p;
  double* pw;
  const double* phi;     // Poisson solution (cells)
  double* f;             // Poisson right-hand side (cells)
  double* ph[3];         // ghosted cell velocity, (N+4)^3
  double* fl[3][3];      // face fluxes: fl[d][m] at the faces along d, component m
  double* t[3];          // cell totals
  const double* cart[3];  // first stage after ns_init_fields(TGV): the analytic cell velocity (cells), else null
  double rk;
  int do_norm;
  double* part;
  unsigned* counter;
  double* red_out;
};

__host__ __device__ __forceinline__ long id3(const Geom& g, int i, int j, int k) {
  return ((long)k * (g.N + 1) + j) * g.pitch + i;
}
__host__ __device__ __forceinline__ long gid3(int N, int i, int j, int k) {
  return (long)(i + 2) + (long)(N + 4) * ((j + 2) + (long)(N + 4) * (k + 2));
}

#ifndef NS_3D_ARGS_ONLY

// thread mapping: x = 32 lanes x blockIdx.x, y = 8 rows x blockIdx.y, z = blockIdx.z
#define NS3_IJK(ox, oy, oz)                                           \
  const int i = (int)(blockIdx.x * 32 + (threadIdx.x & 31)) - (ox);  \
  const int j = (int)(blockIdx.y * 8 + (threadIdx.x >> 5)) - (oy);   \
  const int k = (int)blockIdx.z - (oz);

__device__ __forceinline__ double face_avg(const double* u, const Geom& g, int m, int i, int j, int k) {
  const long a = id3(g, i, j, k);
  const long b = a + (m == 0 ? 1 : (m == 1 ? g.pitch : g.plane));
  return 0.5 * (u[a] + u[b]);
}

// ghosted cell velocity; only cells with at most one index outside [0, N)
// are ever read by the stencils. The first stage after ns_init_fields(TGV)
// takes the analytic cell velocity of hybrid_grid_init (fn_init.cpp:160-229)
// in place of the face average, with the same ghost rules
__global__ void __launch_bounds__(256) k3_cart(Arg3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(2, 2, 2)
  if (i > N + 1 || j > N + 1 || k > N + 1) return;
  const int c[3] = {i, j, k};
  int out_d = -1, nout = 0;
  for (int d = 0; d < 3; ++d)
    if (c[d] < 0 || c[d] >= N) { out_d = d; ++nout; }
  // the cell value: cont2cart's face average, or the analytic override
  auto cell = [&](int m, int a, int b, int cc) {
    return A.cart[0] != nullptr ? A.cart[m][id3(g, a, b, cc)] : face_avg(A.u[m], g, m, a, b, cc);
  };
  for (int m = 0; m < 3; ++m) {
    double val = 0.0;
    if (nout == 0) {
      val = cell(m, i, j, k);
    } else if (nout == 1) {
      const int d = out_d;
      int cm[3] = {i, j, k};
      const int side = c[d] < 0 ? 0 : 1;
      if (g.periodic[d]) {
        cm[d] = wrapi(c[d], N);
        val = cell(m, cm[0], cm[1], cm[2]);
      } else {
        cm[d] = c[d] < 0 ? -c[d] - 1 : 2 * N - 1 - c[d];
        const double q = cell(m, cm[0], cm[1], cm[2]);
        val = cart_ghost(g.bc[2 * d + side], m, q);
      }
    }
    A.ph[m][gid3(N, i, j, k)] = val;
  }
}

// QUICK fluxes of the three components at every face along the three
// directions, each face once: face (i, j, k) along d lies between the cells
// c - e_d and c
__global__ void __launch_bounds__(256) k3_flux(Arg3 A) {
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
    const double ud = A.u[d][fc];
    for (int m = 0; m < 3; ++m) {
      const double* ph = A.ph[m];
      A.fl[d][m][fc] = quick_flux(ud, ph[gc + s], ph[gc], ph[gc - s], ph[gc - 2 * s]);
    }
  }
}

__global__ void __launch_bounds__(256) k3_total(Arg3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  if (i >= N || j >= N || k >= N) return;
  const long G1[3] = {1, N + 4, (long)(N + 4) * (N + 4)};
  const long gc = gid3(N, i, j, k);
  const long fc = id3(g, i, j, k);
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const double* ph = A.ph[m];
    double conv = 0.0, visc = 0.0;
    const double p0 = ph[gc];
    for (int d = 0; d < 3; ++d) {
      const long s = G1[d];
      const double* F = A.fl[d][m];
      if (g.conv_scheme == 0) conv += (F[fc + fstride[d]] - F[fc]) * g.inv_dx[d];
      visc += (ph[gc + s] - 2.0 * p0 + ph[gc - s]) * g.inv_dx2[d];
    }
    A.t[m][fc] = visc * g.inv_ren - conv;
  }
}

// total of component m at cell index a along m (other indices b, c in
// [0, N)), with the flux-ghost rule at a = -1 and a = N
__device__ __forceinline__ double t_along(const Arg3& A, int m, int a, long base, long st) {
  const Geom& g = A.g;
  const int N = g.N;
  if (a >= 0 && a < N) return A.t[m][base + a * st];
  const int fg = g.flux_ghost[m];
  if (fg == kWrap) return A.t[m][base + (long)wrapi(a, N) * st];
  if (fg == kZero) return 0.0;
  const int am = a < 0 ? 0 : N - 1;  // odd reflection
  return -A.t[m][base + (long)am * st];
}

// RK stage on every face of every component (fast FP64 arithmetic), norm of
// the stage-4 increment (weight 1/2 on the first and last face along m)
__global__ void __launch_bounds__(256) k3_face(Arg3 A) {
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
    const double tl = t_along(A, m, a - 1, base, st), tr = t_along(A, m, a, base, st);
    const double G = (A.S[m][id] - g.c15 * A.u[m][id]) + 0.5 * (tl + tr);
    const double o = A.ub[m][id] + A.rk * G;
    A.out[m][id] = o;
    if (A.do_norm) {
      const double q = A.ub[m][id] - o;
      const double w = (a == 0 || a == N) ? 0.5 : 1.0;
      nrm[m] += q * q * w;
    }
  }
  if (A.do_norm && grid_reduce_last<3>(nrm, A.part, A.counter, 0u) && threadIdx.x == 0) {
    const double npts = (double)N * N * N;
    double e = 0.0;
    for (int m = 0; m < 3; ++m) e = max_keep_nan(e, sqrt(nrm[m]) / sqrt(npts));
    *A.red_out = e;
  }
}

// p ghost of the gradient (ctx_mirror: mirrored, else wrapped)
__device__ __forceinline__ double cell_ghosted(const Geom& g, const double* p, int m, int a, long base, long st) {
  const int N = g.N;
  if (a >= N) a = g.ctx_mirror[m] ? N - 1 : 0;
  if (a < 0) a = g.ctx_mirror[m] ? 0 : N - 1;
  return p[base + (long)a * st];
}

// du = u^n - u^{n-1}; S = (-grad p + (0.5/dt) du) + (1.5/dt) u^n
__global__ void __launch_bounds__(256) k3_step_begin(Arg3 A) {
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
    const double un = A.un[m][id];
    const double d = un - A.uprev[m][id];
    A.du[m][id] = d;
    const double gp = (cell_ghosted(g, A.p, m, a, base, st) - cell_ghosted(g, A.p, m, a - 1, base, st)) * g.inv_dx[m];
    A.S[m][id] = (-gp + g.c05 * d) + g.c15 * un;
  }
}

// f = (1.5/dt) div u*; red_out = {max |div|, sum f}
__global__ void __launch_bounds__(256) k3_rhs(Arg3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  double v[2] = {0.0, 0.0};
  if (i < N && j < N && k < N) {
    const long id = id3(g, i, j, k);
    const double div = (A.u[0][id + 1] - A.u[0][id]) * g.inv_dx[0] + (A.u[1][id + g.pitch] - A.u[1][id]) * g.inv_dx[1] +
                       (A.u[2][id + g.plane] - A.u[2][id]) * g.inv_dx[2];
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

// u = u* - (dt/1.5) grad phi on every face (phi ghosts as p); p += phi
__global__ void __launch_bounds__(256) k3_project(Arg3 A) {
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
    const double gphi = (cell_ghosted(g, A.phi, m, a, base, st) - cell_ghosted(g, A.phi, m, a - 1, base, st)) * g.inv_dx[m];
    A.out[m][id] = A.u[m][id] - gphi * g.dt15;
  }
  if (i < N && j < N && k < N) {
    const long id = id3(g, i, j, k);
    A.pw[id] = A.p[id] + A.phi[id];
  }
}

// max |div u| after the projection (main.cpp:1180)
__global__ void __launch_bounds__(256) k3_div(Arg3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  double v[1] = {0.0};
  if (i < N && j < N && k < N) {
    const long id = id3(g, i, j, k);
    const double div = (A.out[0][id + 1] - A.out[0][id]) * g.inv_dx[0] +
                       (A.out[1][id + g.pitch] - A.out[1][id]) * g.inv_dx[1] +
                       (A.out[2][id + g.plane] - A.out[2][id]) * g.inv_dx[2];
    v[0] = fabs(div);
  }
  if (grid_reduce_last<1>(v, A.part, A.counter, 1u) && threadIdx.x == 0) A.red_out[0] = v[0];
}

#endif  // NS_3D_ARGS_ONLY

// ---- multigrid ----------------------------------------------------------------------
constexpr int kMaxLevels3 = 12;

template <typename T>
struct MG3 {
  int L;
  int n[kMaxLevels3];
  long pitch[kMaxLevels3], plane[kMaxLevels3];
  T* x[kMaxLevels3];
  T* f[kMaxLevels3];
  T ih[kMaxLevels3][3];  // 1/h^2 per direction
  int periodic[3];
  const double* fmean;   // subtracted from f at level 0 when non-null
};

// levels with n <= kBottom3N run in the persistent coarse block (k3_mg_coarse)
constexpr int kBottom3N = 16;

#ifndef NS_3D_ARGS_ONLY

template <typename T>
__device__ __forceinline__ T mg3_lap_terms(const MG3<T>& M, int l, int i, int j, int k, T xc, T* diag) {
  const int n = M.n[l];
  const long P = M.pitch[l], PL = M.plane[l];
  const T* x = M.x[l];
  const int c[3] = {i, j, k};
  const long st[3] = {1, P, PL};
  const long id = (long)k * PL + (long)j * P + i;
  T s = (T)0, dg = (T)0;
  for (int d = 0; d < 3; ++d) {
    const T h = M.ih[l][d];
    if (M.periodic[d] || c[d] + 1 < n) {
      const long o = (c[d] + 1 < n) ? st[d] : -(long)(n - 1) * st[d];
      s += x[id + o] * h;
      dg += h;
    }
    if (M.periodic[d] || c[d] > 0) {
      const long o = (c[d] > 0) ? -st[d] : (long)(n - 1) * st[d];
      s += x[id + o] * h;
      dg += h;
    }
  }
  (void)xc;
  *diag = dg;
  return s;
}

template <typename T>
__device__ __forceinline__ T mg3_f(const MG3<T>& M, int l, long id) {
  T v = M.f[l][id];
  if (l == 0 && M.fmean) v -= (T)(*M.fmean);
  return v;
}

// one red-black half-sweep at level l: x = (sum_nb x_nb / h^2 - f) / diag
template <typename T>
__global__ void __launch_bounds__(256) k3_mg_rb(MG3<T> M, int l, int color) {
  const int n = M.n[l];
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= n || j >= n || k >= n || ((i + j + k) & 1) != color) return;
  const long id = (long)k * M.plane[l] + (long)j * M.pitch[l] + i;
  T dg;
  const T s = mg3_lap_terms(M, l, i, j, k, M.x[l][id], &dg);
  if (dg > (T)0) M.x[l][id] = (s - mg3_f(M, l, id)) / dg;
}

// f_{l+1} = cell average of the residual f_l - L x_l over the 8 children; x_{l+1} = 0
template <typename T>
__global__ void __launch_bounds__(256) k3_mg_restrict(MG3<T> M, int l) {
  const int nc = M.n[l + 1];
  const int I = blockIdx.x * 32 + (threadIdx.x & 31), J = blockIdx.y * 8 + (threadIdx.x >> 5), K = blockIdx.z;
  if (I >= nc || J >= nc || K >= nc) return;
  T acc = (T)0;
  for (int c = 0; c < 8; ++c) {
    const int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + (c >> 2);
    const long id = (long)k * M.plane[l] + (long)j * M.pitch[l] + i;
    const T xc = M.x[l][id];
    T dg;
    const T s = mg3_lap_terms(M, l, i, j, k, xc, &dg);
    acc += mg3_f(M, l, id) - (s - dg * xc);
  }
  const long cid = (long)K * M.plane[l + 1] + (long)J * M.pitch[l + 1] + I;
  M.f[l + 1][cid] = acc * (T)0.125;
  M.x[l + 1][cid] = (T)0;
}

// x_l += trilinear interpolation of x_{l+1} (weights 3/4, 1/4 per direction;
// the neighbour beyond a Neumann side is the cell itself, wrapped when periodic)
template <typename T>
__global__ void __launch_bounds__(256) k3_mg_prolong(MG3<T> M, int l) {
  const int n = M.n[l], nc = M.n[l + 1];
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= n || j >= n || k >= n) return;
  const int c[3] = {i, j, k};
  int C[3], Nb[3];
  for (int d = 0; d < 3; ++d) {
    C[d] = c[d] >> 1;
    const int o = (c[d] & 1) ? 1 : -1;
    int nb = C[d] + o;
    if (nb < 0 || nb >= nc) nb = M.periodic[d] ? wrapi(nb, nc) : C[d];
    Nb[d] = nb;
  }
  const long Pc = M.pitch[l + 1], PLc = M.plane[l + 1];
  const T* xc = M.x[l + 1];
  T v = (T)0;
  for (int s = 0; s < 8; ++s) {
    const int a = (s & 1) ? Nb[0] : C[0], b = ((s >> 1) & 1) ? Nb[1] : C[1], e = (s >> 2) ? Nb[2] : C[2];
    const T w = (T)(((s & 1) ? 0.25 : 0.75) * (((s >> 1) & 1) ? 0.25 : 0.75) * ((s >> 2) ? 0.25 : 0.75));
    v += w * xc[(long)e * PLc + (long)b * Pc + a];
  }
  M.x[l][(long)k * M.plane[l] + (long)j * M.pitch[l] + i] += v;
}

// coarsest level (n^3 <= 1024 cells) in one block: red-black sweeps
template <typename T>
__global__ void __launch_bounds__(1024) k3_mg_bottom(MG3<T> M, int l, int sweeps) {
  const int n = M.n[l];
  const int cells = n * n * n;
  for (int q = threadIdx.x; q < cells; q += blockDim.x) {
    const int i = q % n, j = (q / n) % n, k = q / (n * n);
    M.x[l][(long)k * M.plane[l] + (long)j * M.pitch[l] + i] = (T)0;
  }
  __syncthreads();
  for (int it = 0; it < 2 * sweeps; ++it) {
    const int color = it & 1;
    for (int q = threadIdx.x; q < cells; q += blockDim.x) {
      const int i = q % n, j = (q / n) % n, k = q / (n * n);
      if (((i + j + k) & 1) != color) continue;
      const long id = (long)k * M.plane[l] + (long)j * M.pitch[l] + i;
      T dg;
      const T s = mg3_lap_terms(M, l, i, j, k, M.x[l][id], &dg);
      if (dg > (T)0) M.x[l][id] = (s - mg3_f(M, l, id)) / dg;
    }
    __syncthreads();
  }
}

// ---- the coarse levels (n <= kBottom3N) in one persistent block ------------------------
// The levels lb .. L-1 of a V-cycle in shared memory: on each the two
// red-black pre-sweeps and the restriction of its residual, on the coarsest a
// conjugate-gradient solve of L x = f - mean f (the constant mode projected
// out: every 3D box here is all-Neumann or periodic, so L is singular), then
// upward the trilinear prolongation and the two post-sweeps: the arithmetic of
// k3_mg_rb, k3_mg_restrict and k3_mg_prolong, with the coarsest level solved
// instead of swept 50 times. One launch in place of ten per level. The result
// replaces x at level lb in global memory.

template <typename T>
__device__ __forceinline__ T k3_block_sum(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = (T)0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

// shared-memory bytes of the persistent coarse block from level lb
template <typename T>
inline size_t mg3_bottom_smem(const MG3<T>& M, int lb) {
  size_t cells = 0;
  for (int l = lb; l < M.L; ++l) cells += (size_t)M.n[l] * M.n[l] * M.n[l];
  const size_t nc = (size_t)M.n[M.L - 1] * M.n[M.L - 1] * M.n[M.L - 1];
  return (3 * cells + 3 * nc) * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(1024) k3_mg_coarse(MG3<T> M, int lb) {
  extern __shared__ __align__(16) unsigned char mg3c_smem[];
  __shared__ T red[32];
  __shared__ int off[kMaxLevels3];
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool px = M.periodic[0], py = M.periodic[1], pz = M.periodic[2];
  int cells = 0;
  for (int l = lb; l < M.L; ++l) cells += M.n[l] * M.n[l] * M.n[l];
  const int Lc = M.L - 1;
  const int ncc = M.n[Lc] * M.n[Lc] * M.n[Lc];
  T* sx = reinterpret_cast<T*>(mg3c_smem);
  T* sf = sx + cells;
  T* sr = sf + cells;
  T* pcg = sr + cells;
  T* qcg = pcg + ncc;
  T* rcg = qcg + ncc;
  if (tid == 0) {
    int o = 0;
    for (int l = lb; l < M.L; ++l) { off[l] = o; o += M.n[l] * M.n[l] * M.n[l]; }
  }
  __syncthreads();
  {
    const int n = M.n[lb];
    for (int t = tid; t < n * n * n; t += NT) {
      const int i = t % n, j = (t / n) % n, k = t / (n * n);
      const long id = (long)k * M.plane[lb] + (long)j * M.pitch[lb] + i;
      sf[off[lb] + t] = mg3_f(M, lb, id);
      sx[off[lb] + t] = M.x[lb][id];  // zero below the finest level (the restriction clears it)
    }
  }
  __syncthreads();
  // the neighbour sum and diagonal of mg3_lap_terms on a dense n^3 level
  auto lap = [&](const T* x, int l, int i, int j, int k, T* dg) {
    const int n = M.n[l];
    const bool per[3] = {px, py, pz};
    const int c[3] = {i, j, k};
    const int st[3] = {1, n, n * n};
    const int id = (k * n + j) * n + i;
    T s = (T)0, d = (T)0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const T h = M.ih[l][q];
      if (per[q] || c[q] + 1 < n) {
        s += x[id + ((c[q] + 1 < n) ? st[q] : -(n - 1) * st[q])] * h;
        d += h;
      }
      if (per[q] || c[q] > 0) {
        s += x[id + ((c[q] > 0) ? -st[q] : (n - 1) * st[q])] * h;
        d += h;
      }
    }
    *dg = d;
    return s;
  };
  auto sweep = [&](int l, int color) {
    const int n = M.n[l];
    T* x = sx + off[l];
    const T* f = sf + off[l];
    for (int t = tid; t < n * n * n; t += NT) {
      const int i = t % n, j = (t / n) % n, k = t / (n * n);
      if (((i + j + k) & 1) != color) continue;
      T dg;
      const T s = lap(x, l, i, j, k, &dg);
      if (dg > (T)0) x[t] = (s - f[t]) / dg;
    }
    __syncthreads();
  };
  for (int l = lb; l < Lc; ++l) {
    for (int s = 0; s < 4; ++s) sweep(l, s & 1);
    const int n = M.n[l], nc = M.n[l + 1];
    const T* x = sx + off[l];
    const T* f = sf + off[l];
    for (int t = tid; t < nc * nc * nc; t += NT) {
      const int I = t % nc, J = (t / nc) % nc, K = t / (nc * nc);
      T acc = (T)0;
      for (int c = 0; c < 8; ++c) {
        const int i = 2 * I + (c & 1), j = 2 * J + ((c >> 1) & 1), k = 2 * K + (c >> 2);
        const int id = (k * n + j) * n + i;
        T dg;
        const T s = lap(x, l, i, j, k, &dg);
        acc += f[id] - (s - dg * x[id]);
      }
      sf[off[l + 1] + t] = acc * (T)0.125;
      sx[off[l + 1] + t] = (T)0;
    }
    __syncthreads();
  }
  {  // coarsest: CG on -L x = -(f - mean f)
    const int n = M.n[Lc], nn = ncc;
    T* x = sx + off[Lc];
    const T* b = sf + off[Lc];
    auto negL = [&](const T* in, T* out) {
      for (int t = tid; t < nn; t += NT) {
        const int i = t % n, j = (t / n) % n, k = t / (n * n);
        T dg;
        const T s = lap(in, Lc, i, j, k, &dg);
        out[t] = dg * in[t] - s;  // -L in
      }
    };
    T part = (T)0;
    for (int t = tid; t < nn; t += NT) part += b[t];
    const T mean = k3_block_sum<T>(part, red) / (T)nn;
    for (int t = tid; t < nn; t += NT) { rcg[t] = -(b[t] - mean); x[t] = (T)0; pcg[t] = rcg[t]; }
    __syncthreads();
    part = (T)0;
    for (int t = tid; t < nn; t += NT) part += rcg[t] * rcg[t];
    T rr = k3_block_sum<T>(part, red);
    const T rr0 = rr;
    const T eps = sizeof(T) == 8 ? (T)1e-28 : (T)1e-12;
    for (int it = 0; it < 4 * nn && rr > eps * rr0 && rr > (T)0; ++it) {
      negL(pcg, qcg);
      __syncthreads();
      part = (T)0;
      for (int t = tid; t < nn; t += NT) part += pcg[t] * qcg[t];
      const T pq = k3_block_sum<T>(part, red);
      if (!(pq > (T)0)) break;
      const T alpha = rr / pq;
      for (int t = tid; t < nn; t += NT) { x[t] += alpha * pcg[t]; rcg[t] -= alpha * qcg[t]; }
      __syncthreads();
      part = (T)0;
      for (int t = tid; t < nn; t += NT) part += rcg[t] * rcg[t];
      const T rr2 = k3_block_sum<T>(part, red);
      const T beta = rr2 / rr;
      rr = rr2;
      for (int t = tid; t < nn; t += NT) pcg[t] = rcg[t] + beta * pcg[t];
      __syncthreads();
    }
  }
  for (int l = Lc - 1; l >= lb; --l) {
    const int n = M.n[l], nc = M.n[l + 1];
    const T* xc = sx + off[l + 1];
    T* x = sx + off[l];
    const bool per[3] = {px, py, pz};
    for (int t = tid; t < n * n * n; t += NT) {
      const int c[3] = {t % n, (t / n) % n, t / (n * n)};
      int C[3], Nb[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        C[d] = c[d] >> 1;
        const int o = (c[d] & 1) ? 1 : -1;
        int nb = C[d] + o;
        if (nb < 0 || nb >= nc) nb = per[d] ? wrapi(nb, nc) : C[d];
        Nb[d] = nb;
      }
      T v = (T)0;
#pragma unroll
      for (int s = 0; s < 8; ++s) {
        const int a = (s & 1) ? Nb[0] : C[0], b = ((s >> 1) & 1) ? Nb[1] : C[1], e = (s >> 2) ? Nb[2] : C[2];
        const T w = (T)(((s & 1) ? 0.25 : 0.75) * (((s >> 1) & 1) ? 0.25 : 0.75) * ((s >> 2) ? 0.25 : 0.75));
        v += w * xc[(e * nc + b) * nc + a];
      }
      x[t] += v;
    }
    __syncthreads();
    for (int s = 0; s < 4; ++s) sweep(l, (s + 1) & 1);
  }
  {
    const int n = M.n[lb];
    for (int t = tid; t < n * n * n; t += NT) {
      const int i = t % n, j = (t / n) % n, k = t / (n * n);
      M.x[lb][(long)k * M.plane[lb] + (long)j * M.pitch[lb] + i] = sx[off[lb] + t];
    }
  }
}

// max |f - mean - L x| at level 0 (FP64 residual of the level-0 iterate)
template <typename T>
__global__ void __launch_bounds__(256) k3_mg_resnorm(MG3<T> M, double* part, unsigned* counter, double* red_out) {
  const int n = M.n[0];
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  double v[1] = {0.0};
  if (i < n && j < n && k < n) {
    const long id = (long)k * M.plane[0] + (long)j * M.pitch[0] + i;
    const T xc = M.x[0][id];
    T dg;
    const T s = mg3_lap_terms(M, 0, i, j, k, xc, &dg);
    v[0] = fabs((double)(mg3_f(M, 0, id) - (s - dg * xc)));
  }
  if (grid_reduce_last<1>(v, part, counter, 1u) && threadIdx.x == 0) red_out[0] = v[0];
}

#endif  // NS_3D_ARGS_ONLY

}  // namespace ns
