// Fast-arithmetic instantiations (FMA contraction allowed): the FP64 fast
// stage, the mixed-precision anchor, the multigrid and the defect correction.
#include "gmres2d.cuh"
#include "launch.h"

namespace ns {

static inline dim3 stage_grid(const Geom& g) {
  return dim3((g.N + kStageTX - 1) / kStageTX, (g.N + kStageTY - 1) / kStageTY, 1);
}

cudaError_t launch_stage_fast(int mode, const StageArgs& a, cudaStream_t s) {
  if (mode == kFastRK)
    k_stage2d<ArithFast, kFastRK, kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  else if (mode == kAnchor)
    k_stage2d<ArithFast, kAnchor, kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_step_begin_fast(const ProjArgs& a, cudaStream_t s) {
  k_step_begin2d<ArithFast, true><<<proj_face_grid(a.g), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_poisson_rhs_fast(const ProjArgs& a, cudaStream_t s) {
  k_poisson_rhs2d<ArithFast><<<proj_grid(a.g.N), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_project_fast(const ProjArgs& a, cudaStream_t s) {
  k_project2d<ArithFast><<<proj_grid(a.g.N), 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---- multigrid ------------------------------------------------------------
constexpr int kMgTX = 64, kMgTY = 16;

template <typename T>
cudaError_t launch_mg_smooth(const MGLevels<T>& M, int l, int mode, int x_zero, cudaStream_t s) {
  const int n = M.n[l];
  if constexpr (sizeof(T) == 4) {  // FP32 finest levels: the warp-marching smoother (>= 4736 warps)
    if (n >= 4096) {
      const long warps = (long)((n + kColSmOut - 1) / kColSmOut) * ((n + kColSmH - 1) / kColSmH);
      k_mg_smooth_col<T><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(M, l, mode, x_zero);
      return cudaGetLastError();
    }
  }
  dim3 grid((n + kMgTX - 1) / kMgTX, (n + kMgTY - 1) / kMgTY, 1);
  k_mg_smooth<T, kMgTX, kMgTY><<<grid, 256, 0, s>>>(M, l, mode, x_zero);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mg_restrict(const MGLevels<T>& M, int l, cudaStream_t s) {
  const int nc = M.n[l + 1];
  dim3 grid((nc + 31) / 32, (nc + 7) / 8, 1);
  k_mg_restrict<T><<<grid, 256, 0, s>>>(M, l);
  return cudaGetLastError();
}

template <typename T>
static size_t bottom_smem(const MGLevels<T>& M, int lb) {
  size_t cells = 0;
  for (int l = lb; l < M.L; ++l) cells += (size_t)M.n[l] * M.n[l];
  const size_t nc = (size_t)M.n[M.L - 1] * M.n[M.L - 1];
  return (3 * cells + 3 * nc) * sizeof(T);
}

template <typename T>
cudaError_t launch_mg_bottom(const MGLevels<T>& M, int lb, int x_zero, cudaStream_t s) {
  const size_t smem = bottom_smem(M, lb);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_mg_bottom<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_set = true;
  }
  k_mg_bottom<T><<<1, 1024, smem, s>>>(M, lb, x_zero);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mg_resnorm(const MGLevels<T>& M, double* part, unsigned* counter, double* out, cudaStream_t s) {
  const int n = M.n[0];
  dim3 grid((n + 31) / 32, (n + 7) / 8, 1);
  k_mg_resnorm<T><<<grid, 256, 0, s>>>(M, part, counter, out);
  return cudaGetLastError();
}

cudaError_t launch_gm_lap(int n, long P, int px, int py, double ihx, double ihy, const double* x, double* y, cudaStream_t s) {
  const dim3 grid((n + 31) / 32, (n + 7) / 8, 1);
  k_gm_lap<<<grid, 256, 0, s>>>(n, P, px, py, ihx, ihy, x, y);
  return cudaGetLastError();
}

cudaError_t launch_gm_lap3(const GmGrid& G, int px, int py, int pz, double ihx, double ihy, double ihz, const double* x,
                           double* y, cudaStream_t s) {
  const dim3 grid((G.n + 31) / 32, (G.n + 7) / 8, G.nz);
  k_gm_lap3<<<grid, 256, 0, s>>>(G, px, py, pz, ihx, ihy, ihz, x, y);
  return cudaGetLastError();
}

cudaError_t launch_gm_axpby(const GmGrid& G, double a, const double* x, double b, const double* y, const double* sc,
                            double c, double* out, cudaStream_t s) {
  const dim3 grid((G.n + 31) / 32, (G.n + 7) / 8, G.nz);
  k_gm_axpby<<<grid, 256, 0, s>>>(G, a, x, b, y, sc, c, out);
  return cudaGetLastError();
}

cudaError_t launch_gm_mdot(const GmGrid& G, int nv, const GmVecs& V, const double* w, double* part, unsigned* counter,
                           double* out, cudaStream_t s) {
  if (nv < 1 || nv > kGmMaxV) return cudaErrorInvalidValue;
  k_gm_mdot<256><<<kGmBlocks, 256, 0, s>>>(G, nv, V, w, part, counter, out);
  return cudaGetLastError();
}

cudaError_t launch_gm_maxpy(const GmGrid& G, int nv, const GmVecs& V, const double* coef, double s_, double* w,
                            cudaStream_t s) {
  if (nv < 1 || nv > kGmMaxV) return cudaErrorInvalidValue;
  const dim3 grid((G.n + 31) / 32, (G.n + 7) / 8, G.nz);
  k_gm_maxpy<<<grid, 256, 0, s>>>(G, nv, V, coef, s_, w);
  return cudaGetLastError();
}

template cudaError_t launch_mg_smooth<double>(const MGLevels<double>&, int, int, int, cudaStream_t);
template cudaError_t launch_mg_smooth<float>(const MGLevels<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_mg_restrict<double>(const MGLevels<double>&, int, cudaStream_t);
template cudaError_t launch_mg_restrict<float>(const MGLevels<float>&, int, cudaStream_t);
template cudaError_t launch_mg_bottom<double>(const MGLevels<double>&, int, int, cudaStream_t);
template cudaError_t launch_mg_bottom<float>(const MGLevels<float>&, int, int, cudaStream_t);
template cudaError_t launch_mg_resnorm<double>(const MGLevels<double>&, double*, unsigned*, double*, cudaStream_t);

// ---- defect correction of the mixed-precision Poisson solve -----------------
// phi_out = phi_in + e; r = (f - mean f) - L phi_out in FP64; r32 = float(r);
// red_out[0] = max |r|. Tile 32x8 with a one-cell halo in shared memory.
__global__ void __launch_bounds__(256) k_dc_update(DCArgs A) {
  __shared__ double sp[10][34];
  const int n = A.n;
  const long P = A.pitch;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  const bool px = A.periodic[0], py = A.periodic[1];
  for (int t = threadIdx.x; t < 34 * 10; t += blockDim.x) {
    const int lx = t % 34, ly = t / 34;
    const int a = x0 - 1 + lx, b = y0 - 1 + ly;
    double v = 0.0;
    if ((px || (a >= 0 && a < n)) && (py || (b >= 0 && b < n)) && !A.first) {
      const long id = (long)wrapi(b, n) * P + wrapi(a, n);
      v = A.phi_in[id] + (double)A.e[id];
    }
    sp[ly][lx] = v;
  }
  __syncthreads();
  const int a = x0 + (threadIdx.x & 31), b = y0 + (threadIdx.x >> 5);
  double v[1] = {0.0};
  if (a < n && b < n) {
    const int lx = a - x0 + 1, ly = b - y0 + 1;
    const double c = sp[ly][lx];
    double lap = 0.0;
    if (px || a + 1 < n) lap += (sp[ly][lx + 1] - c) * A.invh2[0];
    if (px || a > 0) lap += (sp[ly][lx - 1] - c) * A.invh2[0];
    if (py || b + 1 < n) lap += (sp[ly + 1][lx] - c) * A.invh2[1];
    if (py || b > 0) lap += (sp[ly - 1][lx] - c) * A.invh2[1];
    const long id = (long)b * P + a;
    const double r = (A.f[id] - *A.fmean) - lap;
    A.phi_out[id] = c;
    A.r32[id] = (float)r;
    v[0] = fabs(r);
  }
  if (grid_reduce_last<1>(v, A.part, A.counter, 1u) && threadIdx.x == 0) A.red_out[0] = v[0];
}

cudaError_t launch_dc_update(const DCArgs& a, cudaStream_t s) {
  dim3 grid((a.n + 31) / 32, (a.n + 7) / 8, 1);
  k_dc_update<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// velCart of cont2cart (utilities.cpp:49-53) without ghosts: component d of
// the cell velocity, 0.5 (u_d(c) + u_d(c + e_d)), for 2D (plane = 0, one k)
// and 3D grids of the shared face / cell index map
__global__ void __launch_bounds__(256) k_cell_velocity(const double* u, double* out, int n, long pitch, long plane,
                                                      int d, int nk) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  const int k = blockIdx.z;
  if (i >= n || j >= n || k >= nk) return;
  const long id = (long)k * plane + (long)j * pitch + i;
  const long st = d == 0 ? 1 : (d == 1 ? pitch : plane);
  out[id] = 0.5 * (u[id] + u[id + st]);
}

cudaError_t launch_cell_velocity(const double* u, double* out, int n, long pitch, long plane, int d, int dim,
                                 cudaStream_t s) {
  const int nk = dim == 3 ? n : 1;
  k_cell_velocity<<<dim3((n + 31) / 32, (n + 7) / 8, nk), 256, 0, s>>>(u, out, n, pitch, plane, d, nk);
  return cudaGetLastError();
}

}  // namespace ns
