// Mixed-precision predictor: float-float anchor stage, FP32 increment stages,
// and the FP64 <-> float-float conversions of the pseudo-iterate.
#include "anchor_ff2d.cuh"
#include "launch.h"
#include "stage_inc2d.cuh"

namespace ns {

static inline dim3 stage_grid(const Geom& g) {
  return dim3((g.N + kStageTX - 1) / kStageTX, (g.N + kStageTY - 1) / kStageTY, 1);
}

cudaError_t launch_inc_stage(const IncArgs& a, cudaStream_t s) {
  k_inc_stage2d<kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_anchor_ff(const AnchorFFArgs& a, cudaStream_t s) {
  k_anchor_ff2d<kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_split_ff(const Geom& g, const double* const* x, float* const* h, float* const* l, cudaStream_t s) {
  k_split_ff2d<<<1024, 256, 0, s>>>(g, x[0], x[1], h[0], l[0], h[1], l[1]);
  return cudaGetLastError();
}

cudaError_t launch_ff_add_inc(const Geom& g, const float* const* h, const float* const* l, const float* const* e,
                              double* const* out, cudaStream_t s) {
  k_ff_add_inc2d<<<1024, 256, 0, s>>>(g, h[0], l[0], h[1], l[1], e[0], e[1], out[0], out[1]);
  return cudaGetLastError();
}

}  // namespace ns
