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

#include <cstring>
#include <mutex>

#include "../../include/amressif_gpu.h"
#include "project2d.cuh"
#include "stage2d.cuh"

namespace ns {
namespace {

// Largest grid: 4096 x 4096 cells = 128 x 512 blocks of 32 x 8 cells.
constexpr int kNoAllocMaxCells = 4096;
constexpr int kNoAllocMaxBlocks = (kNoAllocMaxCells / 32) * (kNoAllocMaxCells / 8);
// layout: 2 * kNoAllocMaxBlocks doubles of block partials, 2 result doubles,
// one counter (must be zero when a launch starts)
constexpr size_t kNoAllocBytes = (2 * (size_t)kNoAllocMaxBlocks + 2) * sizeof(double) + 256;

// Held by every GPU that loads the library until the process exits (1 MB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (looked up once
// per device; the host-side symbol itself is not a device address).
cudaError_t scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace ns

extern "C" int ns_poisson_rhs_noalloc(const double* u, const double* v, double* f, int n_cell, long long pitch,
                                      double dx, double dy, double dt, double* divmax_sum, void* stream) {
  using namespace ns;
  if (!u || !v || !f || !divmax_sum || n_cell < 1 || pitch < n_cell + 1 || dx <= 0 || dy <= 0 || dt <= 0)
    return NS_ERR_ARG;
  if (n_cell > kNoAllocMaxCells) return NS_ERR_UNSUPPORTED;  // beyond the fixed scratch
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* base = nullptr;
  if (scratch_for_current_device(&base) != cudaSuccess) return NS_ERR_CUDA;
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
  k_poisson_rhs2d<ArithExact><<<proj_grid(n_cell), 256, 0, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return NS_ERR_CUDA;
  if (cudaMemcpyAsync(divmax_sum, result, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return NS_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return NS_ERR_CUDA;
  return NS_OK;
}
