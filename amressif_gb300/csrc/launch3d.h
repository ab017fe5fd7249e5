// Host-side launchers of the 3D kernels (kernels3d.cu).
#pragma once
#include <cuda_runtime.h>

#define NS_3D_ARGS_ONLY
#include "ns3d.cuh"
#include "ns3d_mixed.cuh"
#undef NS_3D_ARGS_ONLY

namespace ns {

cudaError_t launch3_cart(const Arg3& a, cudaStream_t s);
cudaError_t launch3_total(const Arg3& a, cudaStream_t s);
cudaError_t launch3_face(const Arg3& a, cudaStream_t s);
cudaError_t launch3_step_begin(const Arg3& a, cudaStream_t s);
cudaError_t launch3_rhs(const Arg3& a, cudaStream_t s);
cudaError_t launch3_project(const Arg3& a, cudaStream_t s);
cudaError_t launch3_div(const Arg3& a, cudaStream_t s);
long blocks3_face(int N);  // blocks of the largest reducing launch
// mixed-precision predictor (ns3d_mixed.cuh)
cudaError_t launch3f_cart(const AncFF& a, cudaStream_t s);
cudaError_t launch3f_base32(const AncFF& a, cudaStream_t s);  // FP32 cell velocity of a moved float-float base
cudaError_t launch3f_total(const AncFF& a, cudaStream_t s);  // fluxes, then cell totals
cudaError_t launch3f_face(const AncFF& a, cudaStream_t s);
cudaError_t launch3f_store(const Geom& g, const float2* const* in, double* const* out, cudaStream_t s);
cudaError_t launch3_dcff(const DCff3& a, cudaStream_t s);
cudaError_t launch3_dc64(const DCff3& a, cudaStream_t s);  // dc_residual = 1
cudaError_t launch3_rhs_ff(int n, long pitch, long plane, const double* f, const double* mean, float2* out, cudaStream_t s);
cudaError_t launch3_ff_cells(int n, long pitch, long plane, const float2* in, double* out, cudaStream_t s);
cudaError_t launch3i_cart(const Inc3& a, cudaStream_t s);
cudaError_t launch3i_total(const Inc3& a, cudaStream_t s);  // flux increments and cell totals, one pass
cudaError_t launch3i_face(const Inc3& a, cudaStream_t s);

template <typename T>
cudaError_t launch3_mg_rb(const MG3<T>& M, int l, int color, cudaStream_t s);
template <typename T>
cudaError_t launch3_mg_restrict(const MG3<T>& M, int l, cudaStream_t s);
template <typename T>
cudaError_t launch3_mg_prolong(const MG3<T>& M, int l, cudaStream_t s);
template <typename T>
cudaError_t launch3_mg_bottom(const MG3<T>& M, int l, int sweeps, cudaStream_t s);
template <typename T>
cudaError_t launch3_mg_coarse(const MG3<T>& M, int lb, cudaStream_t s);  // levels lb..L-1 in one block
template <typename T>
cudaError_t launch3_mg_resnorm(const MG3<T>& M, double* part, unsigned* counter, double* out, cudaStream_t s);

}  // namespace ns
