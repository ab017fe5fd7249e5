// Column-marching infrastructure shared by the 2D mixed-precision predictor
// kernels (stage_inc_col2d.cuh, anchor_col2d.cuh): a warp owns a strip of
// columns and marches up its rows; the raw face rows stream through a per-warp
// ring of shared memory filled by cp.async (a few rows in flight), so the
// loads of later rows are in flight while a row is computed and no block
// barrier is needed.
#pragma once
#include <cuda_runtime.h>

namespace ns {

__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async8(float* sdst, const float* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory"); }

}  // namespace ns
