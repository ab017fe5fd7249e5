// Private host-side definition of the solver context (ns_ctx) and the helpers
// shared by the translation units of the C ABI (ns_api.cu: forward advance;
// adjoint_api.cu: tangent-linear / adjoint of the advance).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/amressif_gpu.h"
#include "mg2d.cuh"
#include "ns_common.cuh"

namespace nsh {
struct AdjState;  // adjoint workspace (adjoint_api.cu)
struct State3D;   // fields of a dim = 3 context (ns3d_api.cu)
}

struct ns_ctx {
  ns_params P;
  ns::Geom g;
  int N = 0;
  long pitch = 0;
  size_t fbytes = 0;  // bytes of one FP64 field
  cudaStream_t st = nullptr;
  bool own_stream = false;
  double dt = 0, time = 0, rk[4] = {0, 0, 0, 0};
  long long step = 0;  // completed ns_step calls since init / checkpoint put
  // FP64 fields
  double* U[2] = {nullptr, nullptr};
  double* UP[2] = {nullptr, nullptr};
  double* DU[2] = {nullptr, nullptr};
  double* B[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  double* S[2] = {nullptr, nullptr};
  double* Pp = nullptr;
  double* PHI[2] = {nullptr, nullptr};
  double* F = nullptr;
  double* CART[2] = {nullptr, nullptr};
  double* CONV[2] = {nullptr, nullptr};  // NS_CONV_QUICK: cell convective term of the stage
  bool cart_pending = false;
  // pseudo-iteration state: buffer ids, -1 = UP, 0..2 = B[i]
  int base = -1, cur = -1;
  bool in_step = false;
  bool norm_ready = false;
  // mixed predictor
  float* SH[2] = {nullptr, nullptr};
  float* G0[2] = {nullptr, nullptr};
  float* G0b[2] = {nullptr, nullptr};  // the other anchor buffer (incremental anchor updates)
  float* E[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // multigrid
  ns::MGLevels<double> M64;
  ns::MGLevels<float> M32;
  int lb = 0;
  int phi_cur = 0;
  // reductions
  double* part = nullptr;
  unsigned* counter = nullptr;
  double* red = nullptr;    // device scalars
  double* red_h = nullptr;  // pinned mirror
  // the pseudo-norm as the reducing increment launch writes it straight into
  // mapped pinned host memory: (norm, sequence number); null if unavailable
  double* note_h = nullptr;
  double* note_d = nullptr;
  double note_seq = 0.0;
  cudaEvent_t ev[8];  // 0..3: phases of ns_step; 4..7: the copies of ns_step_host
  bool ev_ok = false;
  // mixed iteration: E[0] holds an increment not yet added to the base
  bool mix_pending = false;
  int mix_it = 0;          // mixed pseudo-iterations of this step
  int mix_last_exact = 0;  // the iteration of the last exact anchor
  double mix_norm = 0.0, mix_norm_exact = 0.0;  // pseudo-norm of the last iteration / of the last exact one
  // float-float pseudo-iterate (hi, lo) ping-pong and the split source S
  float* BH[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  float* BL[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  float* SFh[2] = {nullptr, nullptr};
  float* SFl[2] = {nullptr, nullptr};
  int mb = 0;
  bool base_ff_valid = false, s_ff_valid = false;
  // float-float phi (ping-pong) and RHS of the mixed Poisson solve
  float* PFh[2] = {nullptr, nullptr};
  float* PFl[2] = {nullptr, nullptr};
  float* FFh = nullptr;
  float* FFl = nullptr;
  long long dc_fallbacks = 0;
  // warm start of the mixed solve: the float-float phi buffer (PFh/PFl) that
  // holds the last converged phi (-1: none, after a state was set), and the
  // zero-guess residual max|f - mean f| of the current right-hand side
  // (c15 * max|div u*| from ns_poisson_rhs; rhs_fmax_valid until the solve)
  int pf_warm = -1;
  double rhs_fmax = 0.0;
  bool rhs_fmax_valid = false;
  // per-kernel timing (CUDA events around each launch) and launch count
  bool prof = false;
  std::vector<cudaEvent_t> evpool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pend;
  // V-cycles captured once as CUDA graphs and replayed: [FP64 hierarchy][x0 starts at 0],
  // keyed by the level-0 buffers the graph was captured with
  struct VGraph {
    cudaGraphExec_t exec = nullptr;
    const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
    long long nlaunch = 0;
    bool unusable = false;
  } vg[2][2];
  double pms[NS_PROF_KINDS] = {0};
  long long pcnt[NS_PROF_KINDS] = {0};
  long long launches = 0;
  // initial guess of the next FP64 Poisson solve (the adjoint's warm starts;
  // null: start from zero) and whether its tolerance is relative to max|f|
  // (in red[kRedF], written by the kernel that formed f) instead of r0
  const double* phi_guess = nullptr;
  bool tol_from_f = false;
  // GMRES option of the Poisson solve: Krylov basis and scratch (lazily allocated)
  std::vector<double*> gm_v;
  double* gm_w = nullptr;
  double* gm_z = nullptr;
  double* gm_b = nullptr;
  double* gm_part = nullptr;
  double* gm_dev = nullptr;   // device scalars: dot products, coefficients
  double* gm_host = nullptr;  // pinned mirror
  // ns_step_host: a second stream that copies u_prev back while the step
  // runs (the buffer holds the step's input u^n, unchanged by the step), and
  // the host destinations of that copy, set only for the duration of the call
  cudaStream_t side = nullptr;
  cudaEvent_t side_ev[2] = {nullptr, nullptr};
  double* const* early_uprev = nullptr;
  // bounds-check build: status words of the checked kernels (bounds.cuh)
  unsigned long long* check = nullptr;
  // cell-velocity output of ns_get_cell_velocity (lazily allocated)
  double* cell_tmp = nullptr;
  // lid profile (one value per cell column) when controls are set
  double* lid_col = nullptr;
  int nseg = 0;
  nsh::AdjState* adj = nullptr;
  nsh::State3D* s3 = nullptr;
  std::string err;
};

namespace nsh {

enum RedSlot { kRedNorm = 0, kRedDivBefore = 1, kRedSum = 2, kRedMean = 3, kRedRes = 4, kRedDivAfter = 5, kRedF = 6, kRedObj = 7, kRedScratch = 8 };

int fail(ns_ctx* c, int code, const std::string& msg);
int cuda_check(ns_ctx* c, cudaError_t e, const char* what);
int sync_red(ns_ctx* c, int first, int count);
int alloc_field(ns_ctx* c, double** p);
void prof_resolve(ns_ctx* c);
cudaEvent_t pool_get(ns_ctx* c);
// predictor of one step (ns_step_begin, pseudo-iterations, finalisation); the
// converged u* is face_ptr(c, c->cur, .)
int run_predictor(ns_ctx* c, ns_step_stats* s);
void free_adjoint(ns_ctx* c);
// dim = 3 (ns3d_api.cu)
int create3d(ns_ctx* c);
void free3d(ns_ctx* c);
int set_state3d(ns_ctx* c, const double* const* u, const double* const* up, const double* p, double time);
int get_state3d(ns_ctx* c, double* const* u, double* const* up, double* p, double* phi);
int step3d(ns_ctx* c, ns_step_stats* s);
// the per-call-site building blocks of a 3D context
int step_begin3d(ns_ctx* c);
int rk_stage3d(ns_ctx* c, int sub);
int pseudo_norm3d(ns_ctx* c, double* norm);
int explicit_predictor3d(ns_ctx* c, double* norm);
int ensure_cart3(ns_ctx* c);  // the cell arrays of NS_FIELD_CART
// the GMRES option of the Poisson solve (ns_api.cu), 2D and 3D: L phi = f - mean f
int poisson_gmres(ns_ctx* c, double tol_rel, double div_tol_res, int maxc, int* cycles, double* rnorm0, double* rn);
// its 3D parts (ns3d_api.cu): phi, f and the level-0 1/h^2; one FP64 V-cycle
// from zero as the preconditioner; the max-norm residual into red[kRedRes]
void gm3_fields(ns_ctx* c, double** phi, const double** f, double ih[3]);
int gm3_precond(ns_ctx* c, const double* in, double* out);
int gm3_resnorm(ns_ctx* c);
int poisson_rhs3d(ns_ctx* c, double* divmax, double* sum);
int poisson_solve3d(ns_ctx* c, int precision, int* cycles, double* res);
int project3d(ns_ctx* c, double* divmax);
// device array of an NS_FIELD_* of a 3D context (nullptr if the field has no
// 3D array); *is_face tells whether it is a face field of direction comp
double* field_ptr3d(ns_ctx* c, int field, int comp, bool* is_face);

inline double* face_ptr(ns_ctx* c, int id, int m) { return id < 0 ? c->UP[m] : c->B[id][m]; }

// events created when profiling is switched on (two per launch), and the
// pending launches after which the timings are read out (a stream sync)
constexpr int kProfPool = 16384;
constexpr int kProfPending = 8192;

// Launch one kernel (a callable returning cudaError_t), counting it and, when
// profiling is on, bracketing it with events on the context's stream.
template <class F>
int launch(ns_ctx* c, int kind, const char* what, F&& f) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (c->prof) {
    a = pool_get(c);
    b = pool_get(c);
    if (a) cudaEventRecord(a, c->st);
  }
  const cudaError_t e = f();
  c->launches++;
  if (c->prof && a && b) {
    cudaEventRecord(b, c->st);
    c->pend.push_back({kind, {a, b}});
    if (c->pend.size() > (size_t)kProfPending) {
      cudaStreamSynchronize(c->st);
      prof_resolve(c);
    }
  }
  return cuda_check(c, e, what);
}

}  // namespace nsh

#define CK(expr, what)                                  \
  do {                                                  \
    int _r = nsh::cuda_check(c, (expr), what);          \
    if (_r != NS_OK) return _r;                         \
  } while (0)

#define LAUNCH(kind, what, expr)                                                    \
  do {                                                                              \
    int _r = nsh::launch(c, kind, what, [&]() -> cudaError_t { return (expr); });   \
    if (_r != NS_OK) return _r;                                                     \
  } while (0)
