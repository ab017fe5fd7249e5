// Kernels of the GMRES option of the Poisson solve (GMRES_Poisson.cpp:56-131;
// FP64, cell fields of row pitch P and, in 3D, plane stride PL). The operator
// is the level-0 operator of the multigrid (five or seven points, absent
// neighbours dropped at Neumann sides, wrapped when periodic), so one V-cycle
// is a consistent right preconditioner. The Krylov scalars are reduced in
// fixed block order (deterministic).
#pragma once
#include "ns_common.cuh"

namespace ns {

constexpr int kGmMaxV = 32;    // Krylov vectors per multi-vector kernel call
constexpr int kGmBlocks = 304;  // grid of the dot-product kernel (2 blocks per SM)

struct GmVecs {
  const double* v[kGmMaxV];
};

// the cells of a field: n per direction, nz planes (1 in 2D), cell (i, j, k)
// at k PL + j P + i
struct GmGrid {
  int n, nz;
  long P, PL;
};

#ifndef NS_GMRES_ARGS_ONLY
// y = L x
__global__ void __launch_bounds__(256) k_gm_lap(int n, long P, int px, int py, double ihx, double ihy, const double* x,
                                                double* y) {
  const int a = blockIdx.x * 32 + (threadIdx.x & 31), b = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (a >= n || b >= n) return;
  const long id = (long)b * P + a;
  const double xc = x[id];
  double lap = 0.0;
  if (px || a + 1 < n) lap += (x[(long)b * P + wrapi(a + 1, n)] - xc) * ihx;
  if (px || a > 0) lap += (x[(long)b * P + wrapi(a - 1, n)] - xc) * ihx;
  if (py || b + 1 < n) lap += (x[(long)wrapi(b + 1, n) * P + a] - xc) * ihy;
  if (py || b > 0) lap += (x[(long)wrapi(b - 1, n) * P + a] - xc) * ihy;
  y[id] = lap;
}

// y = L x, seven points (3D)
__global__ void __launch_bounds__(256) k_gm_lap3(GmGrid G, int px, int py, int pz, double ihx, double ihy, double ihz,
                                                 const double* x, double* y) {
  const int n = G.n;
  const int a = blockIdx.x * 32 + (threadIdx.x & 31), b = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (a >= n || b >= n) return;
  const long row = (long)k * G.PL + (long)b * G.P;
  const long id = row + a;
  const double xc = x[id];
  double lap = 0.0;
  if (px || a + 1 < n) lap += (x[row + wrapi(a + 1, n)] - xc) * ihx;
  if (px || a > 0) lap += (x[row + wrapi(a - 1, n)] - xc) * ihx;
  if (py || b + 1 < n) lap += (x[(long)k * G.PL + (long)wrapi(b + 1, n) * G.P + a] - xc) * ihy;
  if (py || b > 0) lap += (x[(long)k * G.PL + (long)wrapi(b - 1, n) * G.P + a] - xc) * ihy;
  if (pz || k + 1 < n) lap += (x[(long)wrapi(k + 1, n) * G.PL + (long)b * G.P + a] - xc) * ihz;
  if (pz || k > 0) lap += (x[(long)wrapi(k - 1, n) * G.PL + (long)b * G.P + a] - xc) * ihz;
  y[id] = lap;
}

// out = a * x + b * y (+ c * (*sc) when sc != null: the mean subtraction f - mean)
__global__ void __launch_bounds__(256) k_gm_axpby(GmGrid G, double a, const double* x, double b, const double* y,
                                                  const double* sc, double c, double* out) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.n || j >= G.n) return;
  const long id = (long)blockIdx.z * G.PL + (long)j * G.P + i;
  double r = a * x[id];
  if (y) r += b * y[id];
  if (sc) r += c * sc[0];
  out[id] = r;
}

// out[k] = (w, v_k), k < nv (<= kGmMaxV); grid-stride over the cells
template <int NT>
__global__ void __launch_bounds__(NT) k_gm_mdot(GmGrid G, int nv, GmVecs V, const double* w, double* part,
                                                unsigned* counter, double* out) {
  double acc[kGmMaxV];
#pragma unroll
  for (int k = 0; k < kGmMaxV; ++k) acc[k] = 0.0;
  const long n = G.n, plane = n * n, cells = plane * G.nz;
  for (long t = blockIdx.x * (long)NT + threadIdx.x; t < cells; t += (long)gridDim.x * NT) {
    const long q = t % plane;
    const long id = (t / plane) * G.PL + (q / n) * G.P + q % n;
    const double wv = w[id];
#pragma unroll
    for (int k = 0; k < kGmMaxV; ++k)
      if (k < nv) acc[k] += wv * V.v[k][id];
  }
  if (grid_reduce_last<kGmMaxV>(acc, part, counter, 0u) && threadIdx.x == 0)
    for (int k = 0; k < nv; ++k) out[k] = acc[k];
}

// w += s * sum_k coef[k] v_k (coef: device array of nv values)
__global__ void __launch_bounds__(256) k_gm_maxpy(GmGrid G, int nv, GmVecs V, const double* coef, double s,
                                                  double* w) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.n || j >= G.n) return;
  const long id = (long)blockIdx.z * G.PL + (long)j * G.P + i;
  double r = w[id];
  for (int k = 0; k < nv; ++k) r += s * coef[k] * V.v[k][id];
  w[id] = r;
}

#endif  // NS_GMRES_ARGS_ONLY

}  // namespace ns
