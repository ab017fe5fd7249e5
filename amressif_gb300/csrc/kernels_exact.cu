// Exact-arithmetic instantiations: compiled with -fmad=false so that every
// product and sum is rounded separately, in the reference's order.
#include "conv_alt2d.cuh"  // its kernel is not a template: this unit alone includes it
#include "launch.h"

namespace ns {

static inline dim3 stage_grid(const Geom& g) {
  return dim3((g.N + kStageTX - 1) / kStageTX, (g.N + kStageTY - 1) / kStageTY, 1);
}

cudaError_t launch_stage_exact(int mode, const StageArgs& a, cudaStream_t s) {
  if (mode == kExactRK)
    k_stage2d<ArithExact, kExactRK, kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  else if (mode == kExplicit)
    k_stage2d<ArithExact, kExplicit, kStageTX, kStageTY><<<stage_grid(a.g), 256, 0, s>>>(a);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_conv_quick_exact(const StageArgs& a, cudaStream_t s) {
  const int N = a.g.N;
  k_conv_quick2d<<<dim3((N + 31) / 32, (N + 7) / 8, 1), dim3(32, 8, 1), 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_step_begin_exact(const ProjArgs& a, cudaStream_t s) {
  k_step_begin2d<ArithExact, false><<<proj_face_grid(a.g), 256, 0, s>>>(a);
  return cudaGetLastError();
}


cudaError_t launch_poisson_rhs_exact(const ProjArgs& a, cudaStream_t s) {
  k_poisson_rhs2d<ArithExact><<<proj_grid(a.g.N), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_project_exact(const ProjArgs& a, cudaStream_t s) {
  k_project2d<ArithExact><<<proj_grid(a.g.N), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace ns
