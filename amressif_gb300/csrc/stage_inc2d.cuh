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
  float2* part;         // float-float block partials of the norm
  unsigned* counter;
  double* norm_out;
};

// QUICK flux difference F(ub + e, phi + eps) - F(ub, phi) (fn_flux_calc.cpp:66-76)
// a, b, c, e: phi at i+1, i, i-1, i-2; pa..pe the same for eps. Branch-free.
// udn = max(un, 0) and upn = min(un, 0) are the upwind parts of the new
// velocity; dud = udn - max(ub, 0) is formed without a subtraction (eb when
// both signs are positive), and dup = eb - dud (exact except after a sign
// change from negative to positive, where it differs from -ub by one rounding).
__device__ __forceinline__ float quick_dflux(float ub, float eb, float a, float b, float c, float e, float pa, float pb_,
                                             float pc, float pe) {
  const float un = ub + eb;
  const float udn = fmaxf(un, 0.f), upn = fminf(un, 0.f);
  const float dud = (ub > 0.f) ? ((un > 0.f) ? eb : -ub) : udn;
  const float dup = eb - dud;
  const float qr_phi = fmaf(0.125f, (-a - 2.f * b) + 3.f * c, b);
  const float ql_phi = fmaf(0.125f, (-e - 2.f * c) + 3.f * b, c);
  const float qr_eps = fmaf(0.125f, (-pa - 2.f * pb_) + 3.f * pc, pb_);
  const float ql_eps = fmaf(0.125f, (-pe - 2.f * pc) + 3.f * pb_, pc);
  return fmaf(dud, ql_phi, fmaf(udn, ql_eps, fmaf(dup, qr_phi, upn * qr_eps)));
}

}  // namespace ns
