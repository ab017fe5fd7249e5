// FP32 increment stages of the mixed-precision predictor.
#include "launch.h"
#include "stage_inc2d.cuh"

namespace ns {

cudaError_t launch_inc_stage(const IncArgs& a, cudaStream_t s) {
  dim3 grid((a.g.N + kStageTX - 1) / kStageTX, (a.g.N + kStageTY - 1) / kStageTY, 1);
  k_inc_stage2d<kStageTX, kStageTY><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_add_inc(const Geom& g, const double* const* base, const float* const* e, double* const* out, cudaStream_t s) {
  k_add_inc2d<<<1024, 256, 0, s>>>(g, base[0], base[1], e[0], e[1], out[0], out[1]);
  return cudaGetLastError();
}

}  // namespace ns
