// FP32 increment stage, column-marching form (2D).
//
// dG(u_b; e_s) with the expanded QUICK flux difference (stage_inc2d.cuh),
// organised for latency hiding and the issue rate of an SM:
//   * one warp owns a strip of 32 consecutive cell columns i = xs - 3 + lane;
//     lanes 3..28 produce output faces, lanes 0-2 / 29-31 carry the x halo;
//   * the warp marches upward through the strip's rows keeping a 5-row window
//     of cell values (u_b and e_s, both components) in registers, so every
//     y-neighbour is a register and every x-neighbour one warp shuffle;
//   * the raw face rows stream through a per-warp cp.async ring in shared
//     memory (kColRing rows in flight), so loads never stall the arithmetic;
//   * no block barrier until the final norm reduction: warps run independently.
// Boundary handling: wall / lid ghosts of the cell
// velocity (utilities.cpp:62-349; x ghosts by a shuffle from the mirror lane,
// y ghosts from the mirror row), face column N and face row N loaded as they
// are (the periodic image included), and the normal-component flux ghosts of
// main.cpp:945-1014 applied at the boundary faces.
#pragma once
#include "ns_common.cuh"
#include "stage_inc2d.cuh"

namespace ns {

constexpr int kColOut = 26;  // output columns per warp
constexpr int kColH = 40;    // rows per strip (a 4096^2 sweep of 16..128 rows peaked at 40)

struct ColCells {
  float p0, p1, e0, e1;  // cart(u_b), cart(e_s)
};

struct RawRow {
  float ua, ub, ea, eb, va, vb, fa, fb, uf, ue, gu, gv;  // faces of one row as loaded
};

// rows of raw faces in flight per warp (cp.async ring in shared memory), and
// the words one lane keeps per row
constexpr int kColRing = 6;
constexpr int kColWords = 10;

__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory"); }

// dynamic shared memory of one block of NT threads
template <int NT>
constexpr size_t inc_col_smem() { return (size_t)(NT / 32) * kColRing * kColWords * 32 * sizeof(float); }

template <int NT>
__global__ void __launch_bounds__(NT, 768 / NT) k_inc_col2d(IncArgs A) {  // 24 warps per SM
  constexpr unsigned FULL = 0xffffffffu;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int lane = threadIdx.x & 31;
  const int nsx = (N + 1 + kColOut - 1) / kColOut;
  const int nsy = (N + kColH - 1) / kColH;
  const int gw = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
  float n0 = 0.f, n1 = 0.f;
  if (gw < nsx * nsy) {  // warp-uniform
    const int sx = gw % nsx, sy = gw / nsx;
    const int xs = sx * kColOut, ys = sy * kColH;
    const int i = xs - 3 + lane;  // this lane's cell / face column
    const bool perx = g.periodic[0], pery = g.periodic[1];
    const float* __restrict__ shu = A.sh[0];
    const float* __restrict__ shv = A.sh[1];
    const bool e_from_g0 = (A.ein[0] == nullptr);
    const float* __restrict__ eu = e_from_g0 ? A.g0[0] : A.ein[0];
    const float* __restrict__ ev = e_from_g0 ? A.g0[1] : A.ein[1];
    const float es = e_from_g0 ? A.rk_prev : 1.f;
    // ic: cell column of the loads (wrapped, or the mirror column of an x
    // ghost); iface: face column of the x flux's advecting velocity
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
    int src_lane = xghost ? (ic - (xs - 3)) : lane;  // the mirror column's lane
    src_lane = src_lane < 0 ? 0 : (src_lane > 31 ? 31 : src_lane);  // lanes past the halo are unused
    const bool warp_xghost = __any_sync(FULL, xghost);
    const CartBC& bx = g.bc[i < 0 ? 0 : 1];
    const float lid = (g.lid_u != nullptr) ? (float)(2.0 * g.lid_u[ic]) : (float)g.bc[3].add[0];

    // The rows k of the strip stream through a ring of kColRing slots: issue_row
    // starts the cp.async copies of row k's faces (this lane's words), read_row
    // waits for the oldest row and returns its raw faces.
    extern __shared__ __align__(16) float col_ring[];
    float* ring = col_ring + (size_t)(threadIdx.x >> 5) * kColRing * kColWords * 32 + lane;
    auto row_of = [&](int k) {
      if (k >= 0 && k < N) return k;
      if (pery) return wrapi(k, N);
      int kk = k < 0 ? -k - 1 : 2 * N - 1 - k;
      return kk < 0 ? 0 : (kk >= N ? N - 1 : kk);
    };
    // ring slots count from the strip's first row (row r_first - 2 in slot 0); row
    // k + kColRing is issued into the slot row k was just read from
    auto issue_row = [&](int k, int slot) {
      const long r0 = (long)row_of(k) * P;
      float* d = ring + (size_t)slot * kColWords * 32;
      cp_async4(d + 0 * 32, shu + r0 + ic);
      cp_async4(d + 1 * 32, shu + r0 + ic + 1);
      cp_async4(d + 2 * 32, eu + r0 + ic);
      cp_async4(d + 3 * 32, eu + r0 + ic + 1);
      cp_async4(d + 4 * 32, shv + r0 + ic);
      cp_async4(d + 5 * 32, shv + r0 + P + ic);
      cp_async4(d + 6 * 32, ev + r0 + ic);
      cp_async4(d + 7 * 32, ev + r0 + P + ic);
      cp_async4(d + 8 * 32, A.g0[0] + r0 + iface);
      cp_async4(d + 9 * 32, A.g0[1] + r0 + ic);
      cp_async_commit();
    };
    auto read_row = [&](int k, int slot, RawRow& R) {
      cp_async_wait<kColRing - 1>();
      const float* d = ring + (size_t)slot * kColWords * 32;
      R.ua = d[0 * 32]; R.ub = d[1 * 32]; R.ea = d[2 * 32]; R.eb = d[3 * 32];
      R.va = d[4 * 32]; R.vb = d[5 * 32]; R.fa = d[6 * 32]; R.fb = d[7 * 32];
      R.gu = d[8 * 32]; R.gv = d[9 * 32];
      if (iface != ic) {  // boundary / periodic lanes only
        const long r0 = (long)row_of(k) * P;
        R.uf = shu[r0 + iface];
        R.ue = eu[r0 + iface];
      } else {
        R.uf = R.ua;
        R.ue = R.ea;
      }
    };
    int k_next = 0, k_end = 0;  // next row to issue, last row of the strip
    int slot = 0;               // ring slot of the next row to read
    auto finish_row = [&](const RawRow& R, int k, ColCells& c, float& ufb, float& ufe, float& vlb, float& vle) {
      c.p0 = 0.5f * (R.ua + R.ub);
      c.e0 = 0.5f * es * (R.ea + R.eb);
      c.p1 = 0.5f * (R.va + R.vb);
      c.e1 = 0.5f * es * (R.fa + R.fb);
      ufb = R.uf;
      ufe = es * R.ue;
      vlb = R.va;
      vle = es * R.fa;
      if (warp_xghost) {  // x ghosts: the mirror lane's value under the side's rule
        const float q0 = __shfl_sync(FULL, c.p0, src_lane), q1 = __shfl_sync(FULL, c.p1, src_lane);
        const float s0 = __shfl_sync(FULL, c.e0, src_lane), s1 = __shfl_sync(FULL, c.e1, src_lane);
        if (xghost) {
          c.p0 = cart_ghost_f(bx, 0, q0, false);
          c.p1 = cart_ghost_f(bx, 1, q1, false);
          c.e0 = cart_ghost_f(bx, 0, s0, true);
          c.e1 = cart_ghost_f(bx, 1, s1, true);
        }
      }
      if (!pery && (k < 0 || k >= N)) {  // y ghosts from the mirror row; the lid profile on the north u
        const CartBC& by = g.bc[k < 0 ? 2 : 3];
        if (k >= N && by.rule[0] == kInlet) c.p0 = lid - c.p0;
        else c.p0 = cart_ghost_f(by, 0, c.p0, false);
        c.p1 = cart_ghost_f(by, 1, c.p1, false);
        c.e0 = cart_ghost_f(by, 0, c.e0, true);
        c.e1 = cart_ghost_f(by, 1, c.e1, true);
      }
    };
    // consume row k (the oldest in flight) and put the next row in flight
    auto cell_row = [&](int k, ColCells& c, float& ufb, float& ufe, float& vlb, float& vle, float& gu, float& gv) {
      RawRow R;
      read_row(k, slot, R);
      if (k_next <= k_end) issue_row(k_next, slot);
      else cp_async_commit();  // empty group: the wait count stays one row per call
      ++k_next;
      slot = (slot == kColRing - 1) ? 0 : slot + 1;
      finish_row(R, k, c, ufb, ufe, vlb, vle);
      gu = R.gu;
      gv = R.gv;
    };

    // w[0..4]: cell rows r-2 .. r+2; uf*[0..2]: u face of rows r .. r+2;
    // vl*[0..2]: lower v face of rows r .. r+2
    ColCells w[5];
    float ufb[3], ufe[3], vlb[3], vle[3], gqu[3], gqv[3], xb, xe;
    const int r_first = ys - 2;  // fy at face ys-1, then the totals of row ys-1
    const int r_last = (ys + kColH >= N) ? N : ys + kColH - 1;
    k_next = r_first - 2;
    k_end = r_last + 2;
    for (int q = 0; q < kColRing; ++q) {
      if (k_next <= k_end) issue_row(k_next, q);
      else cp_async_commit();
      ++k_next;
    }
    cell_row(r_first - 2, w[0], xb, xe, xb, xe, xb, xe);
    cell_row(r_first - 1, w[1], xb, xe, xb, xe, xb, xe);
    cell_row(r_first, w[2], ufb[0], ufe[0], vlb[0], vle[0], gqu[0], gqv[0]);
    cell_row(r_first + 1, w[3], ufb[1], ufe[1], vlb[1], vle[1], gqu[1], gqv[1]);
    const float idx_ = A.inv_dx[0], idy_ = A.inv_dx[1], vx = A.vcoef[0], vy = A.vcoef[1];
    const float c15 = A.c15, rk = A.rk;
    const int fgx = g.flux_ghost[0], fgy = g.flux_ghost[1];
    const bool out_lane = lane >= 3 && lane < 3 + kColOut;
    // per-lane output predicates (loop invariant)
    const bool out_u = out_lane && i >= 0 && i <= N, out_v = out_lane && i >= 0 && i < N;
    const bool edge_u = (i == 0 || i == N);
    const bool rule_u = fgx != kWrap && edge_u;
    const float wgt_u = edge_u ? 0.5f : 1.f;
    float fyp0 = 0.f, fyp1 = 0.f;  // y flux at face r
    float t1p = 0.f;               // v total of row r-1
    for (int r = r_first; r <= r_last; ++r) {
      cell_row(r + 2, w[4], ufb[2], ufe[2], vlb[2], vle[2], gqu[2], gqv[2]);
      // y flux at face r+1 (rows r, r+1), cells r-1 .. r+2; face row N as stored
      float vfb = vlb[1], vfe = vle[1];
      if (r + 1 == N) {
        const long id = (long)N * P + ic;
        vfb = shv[id];
        vfe = es * ev[id];
      }
      const float fy0 = quick_dflux(vfb, vfe, w[4].p0, w[3].p0, w[2].p0, w[1].p0, w[4].e0, w[3].e0, w[2].e0, w[1].e0);
      const float fy1 = quick_dflux(vfb, vfe, w[4].p1, w[3].p1, w[2].p1, w[1].p1, w[4].e1, w[3].e1, w[2].e1, w[1].e1);
      if (r >= ys - 1) {  // warp-uniform
        // x flux at face i of row r: cells i-2 .. i+1
        const ColCells& c = w[2];
        const float p0r = __shfl_down_sync(FULL, c.p0, 1), p0l = __shfl_up_sync(FULL, c.p0, 1);
        const float p0ll = __shfl_up_sync(FULL, c.p0, 2);
        const float p1r = __shfl_down_sync(FULL, c.p1, 1), p1l = __shfl_up_sync(FULL, c.p1, 1);
        const float p1ll = __shfl_up_sync(FULL, c.p1, 2);
        const float e0r = __shfl_down_sync(FULL, c.e0, 1), e0l = __shfl_up_sync(FULL, c.e0, 1);
        const float e0ll = __shfl_up_sync(FULL, c.e0, 2);
        const float e1r = __shfl_down_sync(FULL, c.e1, 1), e1l = __shfl_up_sync(FULL, c.e1, 1);
        const float e1ll = __shfl_up_sync(FULL, c.e1, 2);
        const float fx0 = quick_dflux(ufb[0], ufe[0], p0r, c.p0, p0l, p0ll, e0r, c.e0, e0l, e0ll);
        const float fx1 = quick_dflux(ufb[0], ufe[0], p1r, c.p1, p1l, p1ll, e1r, c.e1, e1l, e1ll);
        const float fx0r = __shfl_down_sync(FULL, fx0, 1), fx1r = __shfl_down_sync(FULL, fx1, 1);
        // totals of cell (i, r)
        const float conv0 = (fx0r - fx0) * idx_ + (fy0 - fyp0) * idy_;
        const float conv1 = (fx1r - fx1) * idx_ + (fy1 - fyp1) * idy_;
        const float visc0 = (e0r - 2.f * c.e0 + e0l) * vx + (w[3].e0 - 2.f * c.e0 + w[1].e0) * vy;
        const float visc1 = (e1r - 2.f * c.e1 + e1l) * vx + (w[3].e1 - 2.f * c.e1 + w[1].e1) * vy;
        const float t0 = visc0 - conv0, t1 = visc1 - conv1;
        const float t0l = __shfl_up_sync(FULL, t0, 1);
        if (r >= ys) {  // warp-uniform
          const long id = (long)r * P + i;
          if (out_u && r < N) {  // u face (i, r)
            float avg = 0.5f * (t0l + t0);
            if (rule_u) avg = (fgx == kReflect) ? 0.f : 0.5f * (i == 0 ? t0 : t0l);
            const float e = rk * (gqu[0] + (avg - c15 * ufe[0]));
            A.eout[0][id] = e;
            n0 = fmaf(wgt_u * e, e, n0);
          }
          if (out_v) {  // v face (i, r), r <= N
            const bool edge_v = (r == 0 || r == N);
            float avg = 0.5f * (t1p + t1);
            if (fgy != kWrap && edge_v) avg = (fgy == kReflect) ? 0.f : 0.5f * (r == 0 ? t1 : t1p);
            float ecur = vle[0], gcur = gqv[0];
            if (r == N) {  // face row N as stored
              ecur = es * ev[id];
              gcur = A.g0[1][id];
            }
            const float e = rk * (gcur + (avg - c15 * ecur));
            A.eout[1][id] = e;
            n1 = fmaf(edge_v ? 0.5f * e : e, e, n1);
          }
        }
        t1p = t1;
      }
      fyp0 = fy0;
      fyp1 = fy1;
      w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
      ufb[0] = ufb[1]; ufe[0] = ufe[1]; ufb[1] = ufb[2]; ufe[1] = ufe[2];
      gqu[0] = gqu[1]; gqv[0] = gqv[1]; gqu[1] = gqu[2]; gqv[1] = gqv[2];
      vlb[0] = vlb[1]; vle[0] = vle[1]; vlb[1] = vlb[2]; vle[1] = vle[2];
    }
    cp_async_wait<0>();
  }
  if (A.do_norm) {
    float v[2] = {n0, n1};
    double out[2];
    if (grid_reduce_last_f<2, NT>(v, A.part, A.counter, 0u, out) && threadIdx.x == 0) {
      const double npts = (double)N * (double)N;
      *A.norm_out = fmax(sqrt(out[0]) / sqrt(npts), sqrt(out[1]) / sqrt(npts));
    }
  }
}

}  // namespace ns
