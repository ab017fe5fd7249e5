// Host-side launchers of the device kernels. The exact-arithmetic kernels
// live in kernels_exact.cu (compiled with -fmad=false), the others in
// kernels_fast.cu.
#pragma once
#include <cuda_runtime.h>

#include "mg2d.cuh"
#include "project2d.cuh"
#include "stage2d.cuh"

namespace ns {

constexpr int kStageTX = 32, kStageTY = 16;

// kernels_exact.cu
cudaError_t launch_stage_exact(int mode, const StageArgs& a, cudaStream_t s);
cudaError_t launch_step_begin_exact(const ProjArgs& a, cudaStream_t s);
cudaError_t launch_poisson_rhs_exact(const ProjArgs& a, cudaStream_t s);
cudaError_t launch_project_exact(const ProjArgs& a, cudaStream_t s);
cudaError_t launch_conv_quick_exact(const StageArgs& a, cudaStream_t s);  // writes a.conv[0..1]

// kernels_fast.cu
cudaError_t launch_stage_fast(int mode, const StageArgs& a, cudaStream_t s);
cudaError_t launch_step_begin_fast(const ProjArgs& a, cudaStream_t s);
cudaError_t launch_poisson_rhs_fast(const ProjArgs& a, cudaStream_t s);
cudaError_t launch_project_fast(const ProjArgs& a, cudaStream_t s);

template <typename T>
cudaError_t launch_mg_smooth(const MGLevels<T>& M, int l, int mode, int x_zero, cudaStream_t s);
template <typename T>
cudaError_t launch_mg_restrict(const MGLevels<T>& M, int l, cudaStream_t s);
template <typename T>
cudaError_t launch_mg_bottom(const MGLevels<T>& M, int lb, int x_zero, cudaStream_t s);
template <typename T>
cudaError_t launch_mg_resnorm(const MGLevels<T>& M, double* part, unsigned* counter, double* out, cudaStream_t s);

// kernels_mixed.cu
struct IncArgs;
struct AnchorFFArgs;
struct DCffArgs;
cudaError_t launch_dc_update_ff(const DCffArgs& a, cudaStream_t s);
cudaError_t launch_rhs_ff(int n, long pitch, const double* f, const double* mean, float* fh, float* fl, cudaStream_t s);
cudaError_t launch_ff_to_double(int n, long pitch, const float* h, const float* l, double* out, cudaStream_t s);
cudaError_t launch_inc_stage(const IncArgs& a, cudaStream_t s);
cudaError_t launch_anchor_ff(const AnchorFFArgs& a, cudaStream_t s);
cudaError_t launch_split_ff(const Geom& g, const double* const* x, float* const* h, float* const* l, cudaStream_t s);
cudaError_t launch_ff_add_inc(const Geom& g, const float* const* h, const float* const* l, const float* const* e,
                              double* const* out, cudaStream_t s);

// kernels_adjoint.cu
struct AdjArgs;
cudaError_t launch_adj_cart(const Geom& g, const double* s0, const double* s1, double* d0, double* d1, const double* lid,
                            int homogeneous, cudaStream_t s);
cudaError_t launch_jvp(const AdjArgs& a, cudaStream_t s);
cudaError_t launch_vjp(const AdjArgs& a, cudaStream_t s);
cudaError_t launch_adj_div(const Geom& g, const double* u0, const double* u1, const double* pb, double coef, double* f,
                           double* part, unsigned* counter, double* sum_out, double* max_out, cudaStream_t s);
cudaError_t launch_adj_gradsub(const Geom& g, const double* in0, const double* in1, const double* psi, double coef, double* o0,
                               double* o1, cudaStream_t s);
cudaError_t launch_adj_lincomb(const Geom& g, double a, const double* x0, const double* x1, double b, const double* y0,
                               const double* y1, double* o0, double* o1, cudaStream_t s);
cudaError_t launch_adj_cells(const Geom& g, double a, const double* x, double b, const double* y, double* o, cudaStream_t s);
cudaError_t launch_tlm_rhs(const Geom& g, const double* const* jl, const double* dp, const double* const* du,
                           const double* const* dup, double* const* out, cudaStream_t s);
struct BcgArgs;
enum BcgPhase { kBcgInit = 0, kBcgAlpha, kBcgS, kBcgOmega, kBcgXR, kBcgP };
cudaError_t launch_bcg(int phase, const BcgArgs& a, cudaStream_t s);
cudaError_t launch_adj_objective(const Geom& g, const double* u0, const double* u1, double* part, unsigned* counter,
                                 double* red_out, cudaStream_t s);
cudaError_t launch_adj_objective_grad(const Geom& g, const double* u0, const double* u1, double* o0, double* o1,
                                      cudaStream_t s);
cudaError_t launch_lid_expand(int N, int nseg, const double* seg, double* col, cudaStream_t s);
cudaError_t launch_lid_accum(int N, int nseg, const double* col, double coef, double* seg_acc, cudaStream_t s);

// kernels_fast.cu: GMRES option of the Poisson solve
struct GmVecs;
struct GmGrid;
cudaError_t launch_gm_lap(int n, long P, int px, int py, double ihx, double ihy, const double* x, double* y, cudaStream_t s);
cudaError_t launch_gm_lap3(const GmGrid& G, int px, int py, int pz, double ihx, double ihy, double ihz, const double* x,
                           double* y, cudaStream_t s);
cudaError_t launch_gm_axpby(const GmGrid& G, double a, const double* x, double b, const double* y, const double* sc,
                            double c, double* out, cudaStream_t s);
cudaError_t launch_gm_mdot(const GmGrid& G, int nv, const GmVecs& V, const double* w, double* part, unsigned* counter,
                           double* out, cudaStream_t s);
cudaError_t launch_gm_maxpy(const GmGrid& G, int nv, const GmVecs& V, const double* coef, double s_, double* w,
                            cudaStream_t s);

struct DCArgs {
  int n;
  long pitch;
  int periodic[2];
  double invh2[2];
  const double* phi_in;
  double* phi_out;
  const float* e;      // FP32 correction (level-0 x of the FP32 hierarchy)
  float* r32;          // FP32 residual (level-0 f of the FP32 hierarchy)
  const double* f;
  const double* fmean;
  int first;           // phi_in is zero and e is absent
  double* part;
  unsigned* counter;
  double* red_out;     // {max |r|}
};
cudaError_t launch_dc_update(const DCArgs& a, cudaStream_t s);
// the cell velocity (face average) of component d, 2D or 3D index map
cudaError_t launch_cell_velocity(const double* u, double* out, int n, long pitch, long plane, int d, int dim,
                                 cudaStream_t s);

}  // namespace ns
