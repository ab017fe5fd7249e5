// Mixed-precision predictor: float-float anchor stage, FP32 increment stages,
// and the FP64 <-> float-float conversions of the pseudo-iterate; float-float
// defect correction of the Poisson solve.
#include "anchor_ff2d.cuh"
#include "dc_ff2d.cuh"
#include "launch.h"
#include "stage_inc2d.cuh"

namespace ns {

constexpr int kMixTX = 32, kMixTY = 32, kMixNT = 512;

static inline dim3 mix_grid(const Geom& g) { return dim3((g.N + kMixTX - 1) / kMixTX, (g.N + kMixTY - 1) / kMixTY, 1); }

cudaError_t launch_inc_stage(const IncArgs& a, cudaStream_t s) {
  constexpr size_t smem = sizeof(IncSmem<kMixTX, kMixTY>);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_inc_stage2d<kMixTX, kMixTY, kMixNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_inc_stage2d<kMixTX, kMixTY, kMixNT><<<mix_grid(a.g), kMixNT, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_anchor_ff(const AnchorFFArgs& a, cudaStream_t s) {
  constexpr size_t smem = sizeof(AnchorSmem<kMixTX, kMixTY>);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_anchor_ff2d<kMixTX, kMixTY, kMixNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_anchor_ff2d<kMixTX, kMixTY, kMixNT><<<mix_grid(a.g), kMixNT, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_split_ff(const Geom& g, const double* const* x, float* const* h, float* const* l, cudaStream_t s) {
  k_split_ff2d<<<1024, 256, 0, s>>>(g, x[0], x[1], h[0], l[0], h[1], l[1]);
  return cudaGetLastError();
}

cudaError_t launch_dc_update_ff(const DCffArgs& a, cudaStream_t s) {
  dim3 grid((a.n + 31) / 32, (a.n + 7) / 8, 1);
  k_dc_update_ff2d<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_rhs_ff(int n, long pitch, const double* f, const double* mean, float* fh, float* fl, cudaStream_t s) {
  k_rhs_ff2d<<<1024, 256, 0, s>>>(n, pitch, f, mean, fh, fl);
  return cudaGetLastError();
}

cudaError_t launch_ff_to_double(int n, long pitch, const float* h, const float* l, double* out, cudaStream_t s) {
  k_ff_to_double2d<<<1024, 256, 0, s>>>(n, pitch, h, l, out);
  return cudaGetLastError();
}

cudaError_t launch_ff_add_inc(const Geom& g, const float* const* h, const float* const* l, const float* const* e,
                              double* const* out, cudaStream_t s) {
  k_ff_add_inc2d<<<1024, 256, 0, s>>>(g, h[0], l[0], h[1], l[1], e[0], e[1], out[0], out[1]);
  return cudaGetLastError();
}

}  // namespace ns
