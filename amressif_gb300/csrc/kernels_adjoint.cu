// Launchers of the tangent-linear / adjoint operators (FP64).
#include "adjoint2d.cuh"
#include "launch.h"

namespace ns {

static inline dim3 face_grid(const Geom& g) { return dim3((g.N + 1 + 127) / 128, g.N + 1, 1); }
static inline dim3 ghost_grid(const Geom& g) { return dim3((g.N + 4 + 127) / 128, g.N + 4, 1); }

cudaError_t launch_adj_cart(const Geom& g, const double* s0, const double* s1, double* d0, double* d1, const double* lid,
                            int homogeneous, cudaStream_t s) {
  k_adj_cart<<<ghost_grid(g), 128, 0, s>>>(g, s0, s1, d0, d1, lid, homogeneous);
  return cudaGetLastError();
}

cudaError_t launch_jvp(const AdjArgs& a, cudaStream_t s) {
  k_adj_cart<<<ghost_grid(a.g), 128, 0, s>>>(a.g, a.v[0], a.v[1], a.dphi[0], a.dphi[1], a.dlid, 1);
  k_jvp_flux<<<face_grid(a.g), 128, 0, s>>>(a);
  k_jvp_total<<<face_grid(a.g), 128, 0, s>>>(a);
  k_jvp_faces<<<face_grid(a.g), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_vjp(const AdjArgs& a, cudaStream_t s) {
  k_vjp_tbar<<<face_grid(a.g), 128, 0, s>>>(a);
  k_vjp_flux<<<face_grid(a.g), 128, 0, s>>>(a);
  k_vjp_phibar<<<ghost_grid(a.g), 128, 0, s>>>(a);
  k_vjp_faces<<<face_grid(a.g), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_div(const Geom& g, const double* u0, const double* u1, const double* pb, double coef, double* f,
                           double* part, unsigned* counter, double* sum_out, double* max_out, cudaStream_t s) {
  dim3 grid((g.N + 31) / 32, (g.N + 7) / 8, 1);
  k_adj_div<<<grid, 256, 0, s>>>(g, u0, u1, pb, coef, f, part, counter, sum_out, max_out);
  return cudaGetLastError();
}

cudaError_t launch_adj_gradsub(const Geom& g, const double* in0, const double* in1, const double* psi, double coef, double* o0,
                               double* o1, cudaStream_t s) {
  k_adj_gradsub<<<face_grid(g), 128, 0, s>>>(g, in0, in1, psi, coef, o0, o1);
  return cudaGetLastError();
}

cudaError_t launch_adj_lincomb(const Geom& g, double a, const double* x0, const double* x1, double b, const double* y0,
                               const double* y1, double* o0, double* o1, cudaStream_t s) {
  k_adj_lincomb<<<face_grid(g), 128, 0, s>>>(g, a, x0, x1, b, y0, y1, o0, o1);
  return cudaGetLastError();
}

cudaError_t launch_adj_cells(const Geom& g, double a, const double* x, double b, const double* y, double* o, cudaStream_t s) {
  k_adj_cells<<<face_grid(g), 128, 0, s>>>(g, a, x, b, y, o);
  return cudaGetLastError();
}

cudaError_t launch_tlm_rhs(const Geom& g, const double* const* jl, const double* dp, const double* const* du,
                           const double* const* dup, double* const* out, cudaStream_t s) {
  k_tlm_rhs<<<face_grid(g), 128, 0, s>>>(g, jl ? jl[0] : nullptr, jl ? jl[1] : nullptr, dp, du[0], du[1], dup[0], dup[1],
                                         out[0], out[1]);
  return cudaGetLastError();
}

cudaError_t launch_bcg(int phase, const BcgArgs& a, cudaStream_t s) {
  const dim3 grid((a.g.N + 1 + 31) / 32, (a.g.N + 1 + 7) / 8, 1);
  switch (phase) {
    case kBcgInit: k_bcg_init<<<grid, 256, 0, s>>>(a); break;
    case kBcgAlpha: k_bcg_alpha<<<grid, 256, 0, s>>>(a); break;
    case kBcgS: k_bcg_s<<<grid, 256, 0, s>>>(a); break;
    case kBcgOmega: k_bcg_omega<<<grid, 256, 0, s>>>(a); break;
    case kBcgXR: k_bcg_xr<<<grid, 256, 0, s>>>(a); break;
    case kBcgP: k_bcg_p<<<grid, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_adj_objective(const Geom& g, const double* u0, const double* u1, double* part, unsigned* counter,
                                 double* red_out, cudaStream_t s) {
  const int H = g.N / 2;
  const dim3 grid((H + 31) / 32, (H + 7) / 8, 1);
  k_adj_objective<<<grid, 256, 0, s>>>(g, u0, u1, part, counter, red_out);
  return cudaGetLastError();
}

cudaError_t launch_adj_objective_grad(const Geom& g, const double* u0, const double* u1, double* o0, double* o1,
                                      cudaStream_t s) {
  k_adj_objective_grad<<<face_grid(g), 128, 0, s>>>(g, u0, u1, o0, o1);
  return cudaGetLastError();
}

cudaError_t launch_lid_expand(int N, int nseg, const double* seg, double* col, cudaStream_t s) {
  k_lid_expand<<<(N + 127) / 128, 128, 0, s>>>(N, nseg, seg, col);
  return cudaGetLastError();
}

cudaError_t launch_lid_accum(int N, int nseg, const double* col, double coef, double* seg_acc, cudaStream_t s) {
  k_lid_accum<<<(nseg + 127) / 128, 128, 0, s>>>(N, nseg, col, coef, seg_acc);
  return cudaGetLastError();
}

}  // namespace ns
