// Launchers of the 3D kernels (ns3d.cuh).
#include "ns3d.cuh"  // kernels (before launch3d.h, which includes the argument structs only)
#include "ns3d_mixed.cuh"
#include "launch3d.h"

namespace ns {

static inline dim3 grid3(int nx, int ny, int nz) { return dim3((nx + 31) / 32, (ny + 7) / 8, nz); }

cudaError_t launch3_cart(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_cart<<<grid3(N + 4, N + 4, N + 4), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_total(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  // convective_flux_calc (conv_scheme 2) adds no convective term: no fluxes
  if (a.g.conv_scheme == 0) k3_flux<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  k3_total<<<grid3(N, N, N), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_face(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_face<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_step_begin(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_step_begin<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_rhs(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_rhs<<<grid3(N, N, N), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_project(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_project<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_div(const Arg3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3_div<<<grid3(N, N, N), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3f_cart(const AncFF& a, cudaStream_t s) {
  const int N = a.g.N;
  k3f_cart<<<grid3(N + 4, N + 4, N + 4), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3f_base32(const AncFF& a, cudaStream_t s) {
  const int N = a.g.N;
  k3f_cart<<<grid3(N + 4, N + 4, N + 4), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3f_total(const AncFF& a, cudaStream_t s) {
  const int N = a.g.N;
  k3f_flux<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  k3f_total<<<grid3(N, N, N), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3f_face(const AncFF& a, cudaStream_t s) {
  const int N = a.g.N;
  k3f_face<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3f_store(const Geom& g, const float2* const* in, double* const* out, cudaStream_t s) {
  const int N = g.N;
  k3f_store<<<grid3(N + 1, N + 1, N + 1), 256, 0, s>>>(g, in[0], in[1], in[2], out[0], out[1], out[2]);
  return cudaGetLastError();
}
cudaError_t launch3_dcff(const DCff3& a, cudaStream_t s) {
  k3_dcff<<<grid3(a.n, a.n, a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_dc64(const DCff3& a, cudaStream_t s) {
  k3_dc64<<<grid3(a.n, a.n, a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3_rhs_ff(int n, long pitch, long plane, const double* f, const double* mean, float2* out, cudaStream_t s) {
  k3_rhs_ff<<<grid3(n, n, n), 256, 0, s>>>(n, pitch, plane, f, mean, out);
  return cudaGetLastError();
}
cudaError_t launch3_ff_cells(int n, long pitch, long plane, const float2* in, double* out, cudaStream_t s) {
  k3_ff_cells<<<grid3(n, n, n), 256, 0, s>>>(n, pitch, plane, in, out);
  return cudaGetLastError();
}
cudaError_t launch3i_cart(const Inc3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3i_cart<<<grid3(N + 4, N + 4, N + 4), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3i_total(const Inc3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3i_fluxtot<<<dim3((N + 31) / 32, (N + 7) / 8, (N + kFtKZ - 1) / kFtKZ), 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3i_face(const Inc3& a, cudaStream_t s) {
  const int N = a.g.N;
  k3i_face<<<grid3(N + 1, N + 1, (N + kIncFaceKZ) / kIncFaceKZ), 256, 0, s>>>(a);
  return cudaGetLastError();
}
long blocks3_face(int N) { return (long)((N + 1 + 31) / 32) * ((N + 1 + 7) / 8) * (N + 1); }

template <typename T>
cudaError_t launch3_mg_rb(const MG3<T>& M, int l, int color, cudaStream_t s) {
  const int n = M.n[l];
  k3_mg_rb<T><<<grid3(n, n, n), 256, 0, s>>>(M, l, color);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch3_mg_restrict(const MG3<T>& M, int l, cudaStream_t s) {
  const int n = M.n[l + 1];
  k3_mg_restrict<T><<<grid3(n, n, n), 256, 0, s>>>(M, l);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch3_mg_prolong(const MG3<T>& M, int l, cudaStream_t s) {
  const int n = M.n[l];
  k3_mg_prolong<T><<<grid3(n, n, n), 256, 0, s>>>(M, l);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch3_mg_bottom(const MG3<T>& M, int l, int sweeps, cudaStream_t s) {
  k3_mg_bottom<T><<<1, 1024, 0, s>>>(M, l, sweeps);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch3_mg_coarse(const MG3<T>& M, int lb, cudaStream_t s) {
  const size_t smem = mg3_bottom_smem(M, lb);
  static bool attr_set = false;
  if (!attr_set) {
    const cudaError_t e = cudaFuncSetAttribute(k3_mg_coarse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  k3_mg_coarse<T><<<1, 1024, smem, s>>>(M, lb);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch3_mg_resnorm(const MG3<T>& M, double* part, unsigned* counter, double* out, cudaStream_t s) {
  const int n = M.n[0];
  k3_mg_resnorm<T><<<grid3(n, n, n), 256, 0, s>>>(M, part, counter, out);
  return cudaGetLastError();
}

#define NS3_INST(T)                                                                               \
  template cudaError_t launch3_mg_rb<T>(const MG3<T>&, int, int, cudaStream_t);                   \
  template cudaError_t launch3_mg_restrict<T>(const MG3<T>&, int, cudaStream_t);                  \
  template cudaError_t launch3_mg_prolong<T>(const MG3<T>&, int, cudaStream_t);                   \
  template cudaError_t launch3_mg_bottom<T>(const MG3<T>&, int, int, cudaStream_t);               \
  template cudaError_t launch3_mg_coarse<T>(const MG3<T>&, int, cudaStream_t);                    \
  template cudaError_t launch3_mg_resnorm<T>(const MG3<T>&, double*, unsigned*, double*, cudaStream_t);
NS3_INST(double)
NS3_INST(float)
#undef NS3_INST

}  // namespace ns
