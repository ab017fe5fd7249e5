// Private: fields of a dim = 3 context, shared by the 3D forward driver
// (ns3d_api.cu) and the 3D adjoint (adjoint3d_api.cu).
#pragma once
#include <vector>

#include "ctx.h"
#include "launch3d.h"

namespace nsh {

struct Adj3;

struct State3D {
  std::vector<void*> allocs;
  size_t fb = 0;  // bytes of one level-0 field
  double* U[3] = {nullptr, nullptr, nullptr};
  double* UP[3] = {nullptr, nullptr, nullptr};
  double* DU[3] = {nullptr, nullptr, nullptr};
  double* S[3] = {nullptr, nullptr, nullptr};
  double* B[3][3] = {};
  double* Pp = nullptr;
  double* PHI = nullptr;
  double* PHI2 = nullptr;  // dc_residual = 1: the other FP64 phi of the defect correction
  double* F = nullptr;
  double* PH[3] = {nullptr, nullptr, nullptr};  // ghosted cell velocity
  double* CART[3] = {nullptr, nullptr, nullptr};  // analytic first-stage cell velocity (allocated on first use)
  double* T[3] = {nullptr, nullptr, nullptr};   // cell totals
  double* FL[3][3] = {};                         // face fluxes
  double* part = nullptr;
  // mixed-precision predictor (FP32): u_b copy, anchor G0, increments, base
  // cell velocity; the flux / total / cell-velocity increments reuse FL, T, PH
  float* UB32[3] = {nullptr, nullptr, nullptr};
  float* UB32b[3] = {nullptr, nullptr, nullptr};  // the other FP32 base: the last stage writes the moved base here
  float* G0[3] = {nullptr, nullptr, nullptr};
  float* G0b[3] = {nullptr, nullptr, nullptr};  // G0 of an incremental anchor update
  int mix_it = 0;          // mixed pseudo-iterations of this step
  int mix_last_exact = 0;  // the iteration of the last exact anchor
  bool mix_exact = false;  // the current iteration's anchor is exact
  double mix_norm = 0.0, mix_norm_exact = 0.0;  // pseudo-norm of the last iteration / of the last exact one
  float* E[2][3] = {};
  float* PHB32[3] = {nullptr, nullptr, nullptr};
  float2* BF[2][3] = {};  // u_b as float-float pairs between pseudo-iterations
  float2* PHF[2] = {};    // Poisson phi as float-float pairs (mixed defect correction)
  float2* FF = nullptr;   // f - mean f as float-float pairs
  int bf = -1;            // BF slot holding u_b; -1: u_b is the FP64 u^n
  ns::MG3<double> M64;
  ns::MG3<float> M32;
  int base = -1, cur = -1;
  ns_ctx::VGraph vg3[2];  // V-cycle graphs: [0] FP32 (with the memset of the correction), [1] FP64
  Adj3* adj = nullptr;
};

// the pieces of the 3D step the adjoint reuses (ns3d_api.cu)
int predictor3d(ns_ctx* c, ns_step_stats* s);      // u* into face3(c, S.cur)
int poisson3d(ns_ctx* c, int* cycles, double* res);  // L PHI = F - mean(F), sum(F) in red[kRedSum]
double* face3_ptr(ns_ctx* c, int id, int m);
// host <-> device in the ns_set_state layout (async on the context's stream)
int copy_faces3(ns_ctx* c, int d, const double* host, double* dev, bool put);
int copy_cells3(ns_ctx* c, const double* host, double* dev, bool put);
// 3D adjoint (adjoint3d_api.cu)
struct Adj3;
void free_adj3(ns_ctx* c);
int adjoint_fwd3(ns_ctx* c, const ns_adjoint_opts* opts, double* J, ns_adjoint_stats* stats);
int adjoint_bwd3(ns_ctx* c, ns_adjoint_stats* stats);
int adjoint_state_grad3(ns_ctx* c, double* const* ubar, double* const* uprevbar, double* pbar);
int step_jvp3(ns_ctx* c, const double* const* du, const double* const* duprev, const double* dp, double* const* du_out,
              double* const* duprev_out, double* dp_out);
int step_vjp3(ns_ctx* c, const double* const* ubar_out, const double* const* uprevbar_out, const double* pbar_out,
              double* const* ubar, double* const* uprevbar, double* pbar);
int adjoint_op3(ns_ctx* c, int transpose, const double* const* x, double* const* y);

}  // namespace nsh
