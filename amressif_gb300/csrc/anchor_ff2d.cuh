// Anchor stage of the mixed-precision pseudo-iteration in float-float
// arithmetic (2D): arguments, the float-float QUICK flux and ghost rule (the
// kernel is k_anchor_col2d), and the FP64 <-> float-float conversions.
//
// The anchor evaluates the stencil of k_stage2d (cont2cart + ghosts, QUICK
// half-node fluxes, viscous term, flux ghost rule, face RHS; main.cpp:931-1017)
// at u_base = base + e4 with ~48-bit float-float numbers on the FP32 pipes, so
// that G(u_base) = S - (1.5/dt) u_base + avg(-conv + visc) keeps FP64-class
// accuracy although its terms cancel to the pseudo-residual. The base itself
// is stored as two float arrays (hi, lo); hi doubles as the FP32 copy read by
// the increment stages.
#pragma once
#include "ff.cuh"
#include "ns_common.cuh"

namespace ns {

struct AnchorFFArgs {
  Geom g;
  const float* bh[2];   // base, hi part (faces)
  const float* bl[2];   // base, lo part
  const float* e4[2];   // pending increment (nullable)
  const float* Sh[2];   // step-constant source S, hi / lo
  const float* Sl[2];
  float* obh[2];        // new base hi / lo
  float* obl[2];
  float* g0[2];         // G(u_base) rounded to FP32
  // constants as float-float (hi, lo) pairs
  float inv_dx[2][2], vcoef[2][2], c15[2];
  int rows;             // rows per strip of the column-marching kernel (set by its launcher)
};

__device__ __forceinline__ ff anchor_u(const AnchorFFArgs& A, int m, long id) {
  ff u = ff_make(A.bh[m][id], A.bl[m][id]);
  if (A.e4[m] != nullptr) u = ff_add_f(u, A.e4[m][id]);
  return u;
}

// QUICK flux (fn_flux_calc.cpp:66-76): u>0 -> u*Q_L, u<0 -> u*Q_R, where
// ud = ucon+|ucon| and up = ucon-|ucon| are exactly u or 0.
__device__ __forceinline__ ff quick_flux_ff(ff u, ff a, ff b, ff c, ff e) {
  if (u.hi > 0.f) {
    const ff q = (ff_scale2(-e - ff_scale2(c, 2.f) + 3.f * b, 0.125f)) + c;
    return u * q;
  } else if (u.hi < 0.f) {
    const ff q = (ff_scale2(-a - ff_scale2(b, 2.f) + 3.f * c, 0.125f)) + b;
    return u * q;
  }
  return ff_make(0.f, 0.f);
}

__device__ __forceinline__ ff cart_ghost_ff(const CartBC& b, int m, ff q) {
  const int r = b.rule[m];
  if (r == kInlet) return ff_from_double(b.add[m]) - q;
  return r == kNeg ? -q : q;
}

// FP64 field -> float-float (hi, lo) arrays, integer split (no FP64 pipe), on
// every face. Thread a of block row b takes the
// u face (a, b) (a <= N, b < N) and the v face (a, b) (a < N, b <= N); grid
// ((N + 1 + 255) / 256, N + 1).
static __global__ void __launch_bounds__(256) k_split_ff2d(Geom g, const double* x0, const double* x1, float* h0, float* l0,
                                                           float* h1, float* l1) {
  const int N = g.N;
  const int a = blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
  if (a > N) return;
  const long id = (long)b * g.pitch + a;
  if (b < N) {
    const ff v = ff_from_double(x0[id]);
    h0[id] = v.hi;
    l0[id] = v.lo;
  }
  if (a < N) {
    const ff v = ff_from_double(x1[id]);
    h1[id] = v.hi;
    l1[id] = v.lo;
  }
}

// u* = (hi + lo) + e (FP64) once the mixed iteration stops; the face layout
// and grid of k_split_ff2d
static __global__ void __launch_bounds__(256) k_ff_add_inc2d(Geom g, const float* h0, const float* l0, const float* h1,
                                                             const float* l1, const float* e0, const float* e1, double* o0,
                                                             double* o1) {
  const int N = g.N;
  const int a = blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
  if (a > N) return;
  const long id = (long)b * g.pitch + a;
  if (b < N) o0[id] = ((double)h0[id] + (double)l0[id]) + (e0 ? (double)e0[id] : 0.0);
  if (a < N) o1[id] = ((double)h1[id] + (double)l1[id]) + (e1 ? (double)e1[id] : 0.0);
}

}  // namespace ns
