// Mixed-precision predictor: float-float anchor stage, FP32 increment stages,
// and the FP64 <-> float-float conversions of the pseudo-iterate; float-float
// defect correction of the Poisson solve.
#include "anchor_ff2d.cuh"
#include "dc_ff2d.cuh"
#include "launch.h"
#include "stage_inc2d.cuh"
#include "stage_inc_col2d.cuh"
#include "anchor_col2d.cuh"

namespace ns {

// column-marching increment stage: one warp per 58-column x kIncH-row strip,
// a cp.async ring of raw face rows per warp in shared memory; the incremental
// anchor update (obh set) also writes the new float-float base
template <bool BASE>
static cudaError_t launch_inc_t(const IncArgs& a0, cudaStream_t s) {
  constexpr int NT = 128;
  IncArgs a = a0;
  a.rows = kIncH;
  const int N = a.g.N;
  const long warps = (long)((N + 1 + kIncOut - 1) / kIncOut) * ((N + a.rows - 1) / a.rows);
  const unsigned blocks = (unsigned)((warps + NT / 32 - 1) / (NT / 32));
  constexpr size_t smem = inc_col_smem<NT, BASE>();
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_inc_col2d<NT, BASE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_inc_col2d<NT, BASE><<<blocks, NT, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_inc_stage(const IncArgs& a, cudaStream_t s) {
  if (a.obh[0] != nullptr) {
    if (a.bl[0] == nullptr || a.bl[1] == nullptr || a.obh[1] == nullptr || a.obl[0] == nullptr || a.obl[1] == nullptr ||
        a.ein[0] == nullptr)
      return cudaErrorInvalidValue;
    return launch_inc_t<true>(a, s);
  }
  return launch_inc_t<false>(a, s);
}

// column-marching float-float anchor: one warp per 26-column x kAncH-row strip,
// a cp.async ring of raw face rows per warp in shared memory
cudaError_t launch_anchor_ff(const AnchorFFArgs& a0, cudaStream_t s) {
  constexpr int NT = 128;
  AnchorFFArgs a = a0;
  a.rows = kAncH;
  const int N = a.g.N;
  const long warps = (long)((N + 1 + kAncOut - 1) / kAncOut) * ((N + a.rows - 1) / a.rows);
  const unsigned blocks = (unsigned)((warps + NT / 32 - 1) / (NT / 32));
  constexpr size_t smem = anchor_col_smem<NT>();
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_anchor_col2d<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_anchor_col2d<NT><<<blocks, NT, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_split_ff(const Geom& g, const double* const* x, float* const* h, float* const* l, cudaStream_t s) {
  k_split_ff2d<<<dim3((g.N + 1 + 255) / 256, g.N + 1), 256, 0, s>>>(g, x[0], x[1], h[0], l[0], h[1], l[1]);
  return cudaGetLastError();
}

cudaError_t launch_dc_update_ff(const DCffArgs& a, cudaStream_t s) {
  dim3 grid((a.n + 31) / 32, (a.n + kDcTY - 1) / kDcTY, 1);
  k_dc_update_ff2d<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_rhs_ff(int n, long pitch, const double* f, const double* mean, float* fh, float* fl, cudaStream_t s) {
  k_rhs_ff2d<<<dim3((n + 255) / 256, n), 256, 0, s>>>(n, pitch, f, mean, fh, fl);
  return cudaGetLastError();
}

cudaError_t launch_ff_to_double(int n, long pitch, const float* h, const float* l, double* out, cudaStream_t s) {
  k_ff_to_double2d<<<dim3((n + 255) / 256, n), 256, 0, s>>>(n, pitch, h, l, out);
  return cudaGetLastError();
}

cudaError_t launch_ff_add_inc(const Geom& g, const float* const* h, const float* const* l, const float* const* e,
                              double* const* out, cudaStream_t s) {
  k_ff_add_inc2d<<<dim3((g.N + 1 + 255) / 256, g.N + 1), 256, 0, s>>>(g, h[0], l[0], h[1], l[1], e[0], e[1], out[0], out[1]);
  return cudaGetLastError();
}

}  // namespace ns
