// Allocation-free Poisson right-hand side (no counterpart in the reference).
//
// Some callers cannot call cudaMalloc: an AMReX host that hands all device
// memory to its own arena allocator, or code that runs while a memory budget
// is fixed for the rest of a job. This entry point computes the same
// right-hand side as ns_poisson_rhs (f = (1.5/dt) div u, with max|div u| and
// sum f) from caller-owned device arrays and takes its reduction scratch from
// a fixed array in this file instead of allocating. Compiled with -fmad=false,
// like kernels_exact.cu, so its results are bit-identical to ns_poisson_rhs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/amressif_gpu.h"
#include "project2d.cuh"
#include "stage2d.cuh"

namespace ns {
namespace {

// Largest grid: 4096 x 4096 cells. k_poisson_rhs2d runs on proj_grid(n):
// blocks of 32 columns x (8 warps x kProjRows rows), 128 x 64 = 8192 blocks
// at n = 4096, each leaving two partials (max|div|, sum f).
constexpr int kNoAllocMaxCells = 4096;
constexpr int kNoAllocMaxBlocks =
    ((kNoAllocMaxCells + 31) / 32) * ((kNoAllocMaxCells + 8 * kProjRows - 1) / (8 * kProjRows));
static_assert(kNoAllocMaxBlocks == 8192, "proj_grid(4096) sizing changed: resize the scratch");
// layout: 2 * kNoAllocMaxBlocks doubles of block partials, 2 result doubles,
// one counter (must be zero when a launch starts)
constexpr size_t kNoAllocBytes = (2 * (size_t)kNoAllocMaxBlocks + 2) * sizeof(double) + 256;

// Held by every GPU that loads the library until the process exits (about
// 128 KB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

}  // namespace
}  // namespace ns

extern "C" int ns_poisson_rhs_noalloc(const double* u, const double* v, double* f, int n_cell, long long pitch,
                                      double dx, double dy, double dt, double* divmax_sum, void* stream) {
  using namespace ns;
  // NaN and infinite spacings or time steps fail these tests too
  if (!u || !v || !f || !divmax_sum || n_cell < 1 || pitch < n_cell + 1 || !(dx > 0 && std::isfinite(dx)) ||
      !(dy > 0 && std::isfinite(dy)) || !(dt > 0 && std::isfinite(dt)))
    return NS_ERR_ARG;
  if (n_cell > kNoAllocMaxCells) return NS_ERR_UNSUPPORTED;  // beyond the fixed scratch
  const dim3 grid = proj_grid(n_cell);
  if ((size_t)grid.x * grid.y > (size_t)kNoAllocMaxBlocks) return NS_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The array's name is a host-side stand-in: its device address on the
  // current device is looked up on every call (cheap, and still right after
  // a cudaDeviceReset has reloaded the module).
  void* sym = nullptr;
  if (cudaGetSymbolAddress(&sym, g_noalloc_scratch) != cudaSuccess) return NS_ERR_CUDA;
  unsigned char* base = static_cast<unsigned char*>(sym);
  double* part = reinterpret_cast<double*>(base);
  double* result = part + 2 * (size_t)kNoAllocMaxBlocks;
  unsigned* counter = reinterpret_cast<unsigned*>(result + 2);
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned), st) != cudaSuccess) return NS_ERR_CUDA;
  ProjArgs a;
  memset(&a, 0, sizeof(a));
  a.g.N = n_cell;
  a.g.dim = 2;
  a.g.pitch = (long)pitch;
  a.g.dx[0] = dx;
  a.g.dx[1] = dy;
  a.g.dx[2] = 1.0;
  a.g.inv_dx[0] = 1.0 / dx;
  a.g.inv_dx[1] = 1.0 / dy;
  a.g.dt = dt;
  a.g.c15 = 1.5 / dt;
  a.u[0] = u;
  a.u[1] = v;
  a.f = f;
  a.part = part;
  a.counter = counter;
  a.red_out = result;
  k_poisson_rhs2d<ArithExact><<<grid, 256, 0, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return NS_ERR_CUDA;
  if (cudaMemcpyAsync(divmax_sum, result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return NS_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return NS_ERR_CUDA;
  return NS_OK;
}
