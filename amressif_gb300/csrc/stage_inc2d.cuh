// FP32 increment stages of the mixed-precision pseudo-time iteration (2D):
// arguments and the flux-difference arithmetic (the kernel is k_inc_col2d).
//
// The reference's RK pseudo-iteration (main.cpp:929-1026) evaluates, from a
// base u_b, the stages u*_{s+1} = u_b + rk[s] G(u*_s) with G the BDF2 residual
// of the QUICK + viscous momentum equation. Writing u*_s = u_b + e_s,
//   G(u_b + e_s) = G(u_b) + dG(u_b; e_s),
//   dG = -(1.5/dt) e_s + avg(-[conv(u_b+e_s) - conv(u_b)] + visc(e_s)).
// G(u_b) is evaluated once per iteration in float-float arithmetic (the anchor
// stage). dG only involves the small increment e_s: it is evaluated in FP32
// from the FP32 part of u_b, with the QUICK flux difference expanded so that
// no term subtracts two nearly equal FP32 numbers:
//   dF = dud * Q_L(phi) + ud' * Q_L(eps) + dup * Q_R(phi) + up' * Q_R(eps),
// with phi = cart(u_b), eps = cart(e_s) and the upwind switch differences
// dud, dup taken from the signs of u_b and u_b + e_s. Its rounding error is
// relative to the increment, so the iteration keeps the FP64 fixed point and
// follows the FP64 iterates up to terms proportional to the final increment.
#pragma once
#include "ns_common.cuh"

namespace ns {

struct IncArgs {
  Geom g;
  const float* sh[2];   // FP32 part of u_base (faces)
  const float* g0[2];   // G(u_base) (faces)
  const float* ein[2];  // e_s (faces); nullptr => e_s = rk_prev * g0
  float rk_prev;
  float* eout[2];       // e_{s+1} = rk * (G0 + dG)
  // incremental anchor update only (nullptr otherwise): the lo part of the
  // float-float base, and the new base (hi, lo) = (sh, bl) + e_s written to
  // the other buffer of the pair, at the faces the launch writes eout
  const float* bl[2];
  float* obh[2];
  float* obl[2];
  float rk;
  float inv_dx[2];      // 1/dx, 1/dy
  float vcoef[2];       // 1/(ren dx^2), 1/(ren dy^2)
  float c15;            // 1.5/dt
  int do_norm;
  int rows;             // rows per strip (set by the launcher)
  float2* part;         // float-float block partials of the norm
  unsigned* counter;
  double* norm_out;
  double* note;         // nullable: mapped host pair (norm, note_seq) written after norm_out
  double note_seq;
};

// Packed FP32 pairs (the add / mul / fma f32x2 instructions of sm_100 and
// later, each lane of the pair rounded like the scalar operation): the
// column-marching kernel keeps two adjacent columns per lane and evaluates
// both with one instruction where the operands form register pairs.
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 p_splat(float x) { return make_float2(x, x); }

// float-float pair + FP32 pair, each lane as ff_add_f (two_sum of the hi
// parts, then fast2sum with the lo parts)
__device__ __forceinline__ void ff_add_f2(float2 h, float2 l, float2 y, float2& oh, float2& ol) {
  const float2 s = p_add(h, y);
  const float2 bb = p_sub(s, h);
  const float2 t = p_add(p_add(p_sub(h, p_sub(s, bb)), p_sub(y, bb)), l);
  oh = p_add(s, t);
  ol = p_sub(t, p_sub(oh, s));
}

// Upwind split of the new advecting velocity un = ub + e and its change
// against ub (fn_flux_calc.cpp:66-68): udn = max(un, 0) and upn = min(un, 0)
// (formed as un - udn, exact); dud = udn - max(ub, 0) without subtracting
// nearly equal numbers: max(eb, -ub) + min(ub, 0), which is eb while both are
// positive, -ub after a sign change to negative, and for ub <= 0 the sum
// eb + ub = un (rounded as un is) or -ub + ub = 0, i.e. udn; dup = eb - dud
// (exact except after a sign change from negative to positive, where it
// differs from -ub by one rounding). The min / max form needs no compare and
// select (two fewer ALU instructions per column pair).
struct QSign2 {
  float2 udn, upn, dud, dup;
};

__device__ __forceinline__ QSign2 quick_sign2(float2 ub, float2 eb) {
  QSign2 q;
  const float2 un = p_add(ub, eb);
  q.udn = make_float2(fmaxf(un.x, 0.f), fmaxf(un.y, 0.f));
  q.upn = p_sub(un, q.udn);
  q.dud = p_add(make_float2(fmaxf(eb.x, -ub.x), fmaxf(eb.y, -ub.y)), make_float2(fminf(ub.x, 0.f), fminf(ub.y, 0.f)));
  q.dup = p_sub(eb, q.dud);
  return q;
}

// QUICK face value (fn_flux_calc.cpp:71-76) mid + (-up - 2 mid + 3 dn) / 8 =
// 0.75 mid + 0.375 dn - 0.125 up, for a pair of faces
__device__ __forceinline__ float2 quick_q2(float2 up, float2 mid, float2 dn) {
  return p_fma(up, p_splat(-0.125f), p_fma(dn, p_splat(0.375f), p_mul(mid, p_splat(0.75f))));
}

// QUICK flux difference F(ub + e, phi + eps) - F(ub, phi) at a pair of faces;
// a, b, c, e: phi at i+1, i, i-1, i-2; pa..pe the same for eps:
//   dF = dud Q_L(phi) + udn Q_L(eps) + dup Q_R(phi) + upn Q_R(eps)
__device__ __forceinline__ float2 quick_dflux2(const QSign2& q, float2 a, float2 b, float2 c, float2 e, float2 pa,
                                               float2 pb, float2 pc, float2 pe) {
  const float2 qr_phi = quick_q2(a, b, c);
  const float2 ql_phi = quick_q2(e, c, b);
  const float2 qr_eps = quick_q2(pa, pb, pc);
  const float2 ql_eps = quick_q2(pe, pc, pb);
  return p_fma(q.dud, ql_phi, p_fma(q.udn, ql_eps, p_fma(q.dup, qr_phi, p_mul(q.upn, qr_eps))));
}

}  // namespace ns
