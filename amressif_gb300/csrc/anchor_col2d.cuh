// Float-float anchor stage, column-marching form (2D).
//
// G(u_base) with u_base = base + e4 in float-float (anchor_ff2d.cuh),
// organised like k_inc_col2d: one
// warp per strip of 32 columns (26 output columns), marching upward with a
// 5-row register window of cell velocities, x neighbours by warp shuffles, and
// the raw face rows streamed through a per-warp cp.async ring in shared
// memory (kAncRing rows in flight), so the loads never stall the arithmetic.
#pragma once
#include <type_traits>
#include "anchor_ff2d.cuh"
#include "bounds.cuh"
#include "ff.cuh"
#include "col2d.cuh"

namespace ns {

constexpr int kAncOut = 26;    // output columns per warp (lanes 3..28; 3 halo lanes each side)
// rows per strip (passed as A.rows; a 4096^2 sweep of 16..128 rows peaked at
// 40; one-wave strips of 274 rows took a launch from 0.615 to 0.731 ms)
constexpr int kAncH = 40;
constexpr int kAncRing = 4;    // rows in flight per warp (6, 4 and 3 rows: 0.626, 0.620, 0.619 ms a launch at 4096^2)
constexpr int kAncWords = 16;  // words per lane and row in the ring

struct CellFF {
  ff p0, p1;
};

template <int NT>
constexpr size_t anchor_col_smem() { return (size_t)(NT / 32) * kAncRing * kAncWords * 32 * sizeof(float); }

__device__ __forceinline__ ff shfl_ff(ff x, int src) {
  return ff_make(__shfl_sync(0xffffffffu, x.hi, src), __shfl_sync(0xffffffffu, x.lo, src));
}
__device__ __forceinline__ ff shfl_up_ff(ff x, int d) {
  return ff_make(__shfl_up_sync(0xffffffffu, x.hi, d), __shfl_up_sync(0xffffffffu, x.lo, d));
}
__device__ __forceinline__ ff shfl_down_ff(ff x, int d) {
  return ff_make(__shfl_down_sync(0xffffffffu, x.hi, d), __shfl_down_sync(0xffffffffu, x.lo, d));
}

template <int NT>
__global__ void __launch_bounds__(NT) k_anchor_col2d(AnchorFFArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int lane = threadIdx.x & 31;
  const int nsx = (N + 1 + kAncOut - 1) / kAncOut;
  const int H = A.rows;
  const int nsy = (N + H - 1) / H;
  const int gw = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
  if (gw >= nsx * nsy) return;  // warp-uniform; no block-wide barrier below
  const int sx = gw % nsx, sy = gw / nsx;
  const int xs = sx * kAncOut, ys = sy * H;
  const int i = xs - 3 + lane;
  const bool perx = g.periodic[0], pery = g.periodic[1];
  const bool has_e = A.e4[0] != nullptr;
  const bool xghost = !perx && (i < 0 || i >= N);
  int ic, iface;
  if (perx) {
    ic = wrapi(i, N);
    iface = (i >= 0 && i <= N) ? i : ic;
  } else {
    ic = i < 0 ? -i - 1 : (i >= N ? 2 * N - 1 - i : i);
    ic = ic < 0 ? 0 : (ic >= N ? N - 1 : ic);
    iface = i < 0 ? 0 : (i > N ? N : i);
  }
  int src_lane = xghost ? (ic - (xs - 3)) : lane;
  src_lane = src_lane < 0 ? 0 : (src_lane > 31 ? 31 : src_lane);
  const bool warp_xghost = __any_sync(0xffffffffu, xghost);
  const CartBC& bx = g.bc[i < 0 ? 0 : 1];
  const ff lid = (g.lid_u != nullptr) ? ff_from_double(2.0 * g.lid_u[ic]) : ff_from_double(g.bc[3].add[0]);

  extern __shared__ __align__(16) float anc_ring[];
  float* ring = anc_ring + (size_t)(threadIdx.x >> 5) * kAncRing * kAncWords * 32 + lane;
  auto row_of = [&](int k) {
    if (k >= 0 && k < N) return k;
    if (pery) return wrapi(k, N);
    int kk = k < 0 ? -k - 1 : 2 * N - 1 - k;
    return kk < 0 ? 0 : (kk >= N ? N - 1 : kk);
  };
  // ring slots count from the strip's first row (row r_first - 2 in slot 0); row
  // k + kAncRing is issued into the slot row k was just read from
  auto slot_ptr = [&](int sl) { return ring + (size_t)sl * kAncWords * 32; };
  // words: 0-2 u face (ic): hi, lo, e4; 3-5 u face (ic+1); 6-8 v face (ic, kk);
  // 9-11 v face (ic, kk+1); 12-13 S_u (iface): hi, lo; 14-15 S_v (ic): hi, lo
  unsigned long long* const chk = g.check;  // bounds-check build only (bounds.cuh)
  (void)chk;
  auto issue_row = [&](int k, int sl) {
    const long r0 = (long)row_of(k) * P;
    float* d = slot_ptr(sl);
    // every level-0 field is P x (N + 1) elements
    if (!NS_BCHK(chk, r0 + ic, P, N + 1, N - 1, 21) || !NS_BCHK(chk, r0 + P + ic, P, N + 1, N, 22) ||
        !NS_BCHK(chk, r0 + iface, P, N + 1, N, 23)) {
      cp_async_commit();
      return;
    }
    cp_async4(d + 0 * 32, A.bh[0] + r0 + ic);
    cp_async4(d + 1 * 32, A.bl[0] + r0 + ic);
    cp_async4(d + 3 * 32, A.bh[0] + r0 + ic + 1);
    cp_async4(d + 4 * 32, A.bl[0] + r0 + ic + 1);
    cp_async4(d + 6 * 32, A.bh[1] + r0 + ic);
    cp_async4(d + 7 * 32, A.bl[1] + r0 + ic);
    cp_async4(d + 9 * 32, A.bh[1] + r0 + P + ic);
    cp_async4(d + 10 * 32, A.bl[1] + r0 + P + ic);
    if (has_e) {
      cp_async4(d + 2 * 32, A.e4[0] + r0 + ic);
      cp_async4(d + 5 * 32, A.e4[0] + r0 + ic + 1);
      cp_async4(d + 8 * 32, A.e4[1] + r0 + ic);
      cp_async4(d + 11 * 32, A.e4[1] + r0 + P + ic);
    }
    cp_async4(d + 12 * 32, A.Sh[0] + r0 + iface);
    cp_async4(d + 13 * 32, A.Sl[0] + r0 + iface);
    cp_async4(d + 14 * 32, A.Sh[1] + r0 + ic);
    cp_async4(d + 15 * 32, A.Sl[1] + r0 + ic);
    cp_async_commit();
  };
  // u_base at a face of the ring row: hi + lo (+ e4)
  auto ubase = [&](const float* d, int w) {
    ff u = ff_make(d[w * 32], d[(w + 1) * 32]);
    if (has_e) u = ff_add_f(u, d[(w + 2) * 32]);
    return u;
  };
  auto ubase_direct = [&](int m, long id) {
    if (!NS_BCHK(chk, id, P, N + 1, N, 24)) return ff_make(0.f, 0.f);
    ff u = ff_make(A.bh[m][id], A.bl[m][id]);
    if (has_e) u = ff_add_f(u, A.e4[m][id]);
    return u;
  };
  int k_next = 0, k_end = 0;
  int rslot = 0;  // ring slot of the next row to read
  // consume row k: cell velocities (with ghosts), the u face (iface, k), the
  // lower v face (ic, k) and S at the lane's faces
  // FAST (a strip whose columns and rows all lie inside the domain, away
  // from every wall and the periodic seam): the ghost, image-column and face
  // row N branches are compiled out; the remaining operations, and so the
  // bits, are the same
  auto cell_row = [&](auto fast_c, int k, CellFF& c, ff& uf, ff& vl, ff& su, ff& sv) {
    constexpr bool FAST = decltype(fast_c)::value;
    cp_async_wait<kAncRing - 1>();
    const float* d = slot_ptr(rslot);
    const ff ua = ubase(d, 0), ub = ubase(d, 3), va = ubase(d, 6), vb = ubase(d, 9);
    su = ff_make(d[12 * 32], d[13 * 32]);
    sv = ff_make(d[14 * 32], d[15 * 32]);
    if (!FAST && iface != ic) uf = ubase_direct(0, (long)row_of(k) * P + iface);  // boundary / periodic lanes only
    else uf = ua;
    vl = va;
    if (k_next <= k_end) issue_row(k_next, rslot);
    else cp_async_commit();
    ++k_next;
    rslot = (rslot == kAncRing - 1) ? 0 : rslot + 1;
    c.p0 = ff_scale2(ua + ub, 0.5f);
    c.p1 = ff_scale2(va + vb, 0.5f);
    if (!FAST && warp_xghost) {
      const ff q0 = shfl_ff(c.p0, src_lane), q1 = shfl_ff(c.p1, src_lane);
      if (xghost) {
        c.p0 = cart_ghost_ff(bx, 0, q0);
        c.p1 = cart_ghost_ff(bx, 1, q1);
      }
    }
    if (!FAST && !pery && (k < 0 || k >= N)) {
      const CartBC& by = g.bc[k < 0 ? 2 : 3];
      if (k >= N && by.rule[0] == kInlet) c.p0 = lid - c.p0;
      else c.p0 = cart_ghost_ff(by, 0, c.p0);
      c.p1 = cart_ghost_ff(by, 1, c.p1);
    }
  };

  const int r_first = ys - 2, r_last = (ys + H >= N) ? N : ys + H - 1;
  // the strip's row march, instantiated once for fast strips and once for
  // the others (the choice at its end)
  auto march = [&](auto fast_c) {
  constexpr bool FAST = decltype(fast_c)::value;
  k_next = r_first - 2;
  k_end = r_last + 2;
  for (int q = 0; q < kAncRing; ++q) {
    if (k_next <= k_end) issue_row(k_next, q);
    else cp_async_commit();
    ++k_next;
  }
  CellFF w[5];
  ff uf[3], vl[3], su[3], sv[3], xa, xb, xc, xd;
  cell_row(fast_c, r_first - 2, w[0], xa, xb, xc, xd);
  cell_row(fast_c, r_first - 1, w[1], xa, xb, xc, xd);
  cell_row(fast_c, r_first, w[2], uf[0], vl[0], su[0], sv[0]);
  cell_row(fast_c, r_first + 1, w[3], uf[1], vl[1], su[1], sv[1]);
  const ff idx_ = ff_make(A.inv_dx[0][0], A.inv_dx[0][1]), idy_ = ff_make(A.inv_dx[1][0], A.inv_dx[1][1]);
  const ff vx = ff_make(A.vcoef[0][0], A.vcoef[0][1]), vy = ff_make(A.vcoef[1][0], A.vcoef[1][1]);
  const ff c15 = ff_make(A.c15[0], A.c15[1]);
  const ff zero = ff_make(0.f, 0.f);
  const int fgx = g.flux_ghost[0], fgy = g.flux_ghost[1];
  const bool out_lane = lane >= 3 && lane < 3 + kAncOut;
  ff fyp0 = zero, fyp1 = zero, t1p = zero;
  for (int r = r_first; r <= r_last; ++r) {
    cell_row(fast_c, r + 2, w[4], uf[2], vl[2], su[2], sv[2]);
    // y flux at face r+1 (rows r, r+1); face row N as stored
    ff vf = vl[1];
    if (!FAST && r + 1 == N) vf = ubase_direct(1, (long)N * P + ic);
    const ff fy0 = quick_flux_ff(vf, w[4].p0, w[3].p0, w[2].p0, w[1].p0);
    const ff fy1 = quick_flux_ff(vf, w[4].p1, w[3].p1, w[2].p1, w[1].p1);
    if (r >= ys - 1) {
      const CellFF& c = w[2];
      const ff p0r = shfl_down_ff(c.p0, 1), p0l = shfl_up_ff(c.p0, 1), p0ll = shfl_up_ff(c.p0, 2);
      const ff p1r = shfl_down_ff(c.p1, 1), p1l = shfl_up_ff(c.p1, 1), p1ll = shfl_up_ff(c.p1, 2);
      const ff fx0 = quick_flux_ff(uf[0], p0r, c.p0, p0l, p0ll);
      const ff fx1 = quick_flux_ff(uf[0], p1r, c.p1, p1l, p1ll);
      const ff fx0r = shfl_down_ff(fx0, 1), fx1r = shfl_down_ff(fx1, 1);
      const ff conv0 = (fx0r - fx0) * idx_ + (fy0 - fyp0) * idy_;
      const ff conv1 = (fx1r - fx1) * idx_ + (fy1 - fyp1) * idy_;
      const ff c20 = ff_scale2(c.p0, 2.f), c21 = ff_scale2(c.p1, 2.f);
      const ff visc0 = (p0r - c20 + p0l) * vx + (w[3].p0 - c20 + w[1].p0) * vy;
      const ff visc1 = (p1r - c21 + p1l) * vx + (w[3].p1 - c21 + w[1].p1) * vy;
      const ff t0 = visc0 - conv0, t1 = visc1 - conv1;
      const ff t0l = shfl_up_ff(t0, 1);
      if (r >= ys && out_lane) {
        if ((FAST || (r < N && i >= 0 && i <= N)) && NS_BCHK(chk, (long)r * P + i, P, N + 1, N, 25)) {  // u face (i, r)
          ff avg = ff_scale2(t0l + t0, 0.5f);
          if (!FAST && fgx != kWrap && (i == 0 || i == N)) avg = (fgx == kReflect) ? zero : ff_scale2(i == 0 ? t0 : t0l, 0.5f);
          const long id = (long)r * P + i;
          const ff u = uf[0];
          const ff G = (su[0] - c15 * u) + avg;
          A.obh[0][id] = u.hi;
          A.obl[0][id] = u.lo;
          A.g0[0][id] = G.hi + G.lo;
        }
        if ((FAST || (i >= 0 && i < N)) && NS_BCHK(chk, (long)r * P + i, P, N + 1, N, 26)) {  // v face (i, r), r <= N
          ff avg = ff_scale2(t1p + t1, 0.5f);
          if (!FAST && fgy != kWrap && (r == 0 || r == N)) avg = (fgy == kReflect) ? zero : ff_scale2(r == 0 ? t1 : t1p, 0.5f);
          const long id = (long)r * P + i;
          const ff u = (!FAST && r == N) ? ubase_direct(1, id) : vl[0];  // face row N as stored
          const ff S = (!FAST && r == N) ? ff_make(A.Sh[1][id], A.Sl[1][id]) : sv[0];
          const ff G = (S - c15 * u) + avg;
          A.obh[1][id] = u.hi;
          A.obl[1][id] = u.lo;
          A.g0[1][id] = G.hi + G.lo;
        }
      }
      t1p = t1;
    }
    fyp0 = fy0;
    fyp1 = fy1;
    w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
    uf[0] = uf[1]; uf[1] = uf[2];
    vl[0] = vl[1]; vl[1] = vl[2];
    su[0] = su[1]; su[1] = su[2];
    sv[0] = sv[1]; sv[1] = sv[2];
  }
  };
  const bool fast = xs >= 3 && xs + 29 <= N && ys >= 4 && ys + H + 2 <= N;
  if (fast) march(std::true_type{});
  else march(std::false_type{});
  cp_async_wait<0>();
}

}  // namespace ns
