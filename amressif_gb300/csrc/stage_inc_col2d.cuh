// FP32 increment stage, column-marching form (2D).
//
// dG(u_b; e_s) with the expanded QUICK flux difference (stage_inc2d.cuh).
// One warp owns a strip of 64 columns and kIncH rows and marches up the rows
// with a 5-row register window of cell values (u_b and e_s, both components):
// y neighbours are registers, x neighbours warp shuffles, and the raw face
// rows stream through the per-warp cp.async ring of col2d.cuh. One lane owns
// the column pair (a, b) = (xs - 4 + 2 lane, a + 1):
//   * a warp writes kIncOut = 58 of its 64 columns (the x stencils need 3
//     columns on the left and 2 on the right);
//   * the cell-indexed face words of a row come in 8-byte pairs: 10 cp.async
//     copies per row for two columns;
//   * x neighbours need three shuffles per field for both columns.
// Compared with one column per lane (26 output columns per warp) this issues
// about a quarter fewer instructions per output face; it runs at 12 warps per
// SM (150 registers), and at 4096^2 a launch takes 0.243 ms against 0.273.
// The incremental anchor update (BASE = true) also writes the new float-float
// base (hi, lo) + e_s at its output faces, into the other buffer of the pair:
// the lo words of row k - 2 travel in row k's ring slot, so they arrive with
// the cell values read in the iteration that writes the faces of row k - 2.
// Boundary handling: wall / lid ghosts of the cell velocity
// (utilities.cpp:62-349; x ghosts from the mirror lane, y ghosts from the
// mirror row), face column N and face row N loaded as they are (the periodic
// image included), and the normal-component flux ghosts of main.cpp:945-1014
// applied at the boundary faces.
// a is even and N is even, so a pair never straddles a wall or the periodic
// seam: after wrapping (periodic) or mirroring (wall ghosts) the two columns
// stay adjacent, and a wall ghost pair mirrors onto one lane's pair with the
// slots swapped. Face-indexed words whose face is not the lane's cell column
// (face N, the periodic image, wall faces) are loaded directly, per slot, as
// in k_inc_col2d.
#pragma once
#include "col2d.cuh"
#include "ff.cuh"
#include "ns_common.cuh"
#include "stage_inc2d.cuh"

namespace ns {

constexpr int kIncOut = 58;    // output columns per warp
constexpr int kIncH = 24;      // rows per strip (a 4096^2 sweep of 12..56 rows peaked at 24)
// ring words per lane and row: 8 float2 pairs and 2 singles, plus the two lo
// pairs of the base update
__host__ __device__ constexpr int inc_words(bool base) { return base ? 22 : 18; }

struct ColCells2 {
  float p0[2], p1[2], e0[2], e1[2];  // cart(u_b), cart(e_s) of columns a, b
};

template <int NT, bool BASE>
constexpr size_t inc_col_smem() { return (size_t)(NT / 32) * kColRing * inc_words(BASE) * 32 * sizeof(float); }

template <int NT, bool BASE>
__global__ void __launch_bounds__(NT, 384 / NT) k_inc_col2d(IncArgs A) {  // 12 warps per SM
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int kWords = inc_words(BASE), kPairs = BASE ? 10 : 8;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int lane = threadIdx.x & 31;
  const int nsx = (N + 1 + kIncOut - 1) / kIncOut;
  const int nsy = (N + kIncH - 1) / kIncH;
  const int gw = blockIdx.x * (NT / 32) + (threadIdx.x >> 5);
  float n0 = 0.f, n1 = 0.f;
  if (gw < nsx * nsy) {  // warp-uniform
    const int sx = gw % nsx, sy = gw / nsx;
    const int xs = sx * kIncOut, ys = sy * kIncH;
    const int a = xs - 4 + 2 * lane;  // column of slot 0; slot 1 is a + 1
    const bool perx = g.periodic[0], pery = g.periodic[1];
    const float* __restrict__ shu = A.sh[0];
    const float* __restrict__ shv = A.sh[1];
    const bool e_from_g0 = (A.ein[0] == nullptr);
    const float* __restrict__ eu = e_from_g0 ? A.g0[0] : A.ein[0];
    const float* __restrict__ ev = e_from_g0 ? A.g0[1] : A.ein[1];
    const float es = e_from_g0 ? A.rk_prev : 1.f;
    // per slot s (column a + s): icm = cell column of k_inc_col2d (wrapped, or
    // the clamped mirror of an x ghost), iface = face column of the x flux's
    // advecting velocity; the pair loads use the even column pc (the lane's
    // own pair, wrapped; any valid pair for a ghost lane, whose values are
    // replaced by the mirror lane's)
    const bool xghost = !perx && (a < 0 || a >= N);  // both slots (a even, N even)
    int icm[2], iface[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int i = a + s;
      if (perx) {
        icm[s] = wrapi(i, N);
        iface[s] = (i >= 0 && i <= N) ? i : icm[s];
      } else {
        int ic = i < 0 ? -i - 1 : (i >= N ? 2 * N - 1 - i : i);
        icm[s] = ic < 0 ? 0 : (ic >= N ? N - 1 : ic);
        iface[s] = i < 0 ? 0 : (i > N ? N : i);
      }
    }
    const int pc = perx ? icm[0] : (xghost ? (a < 0 ? 0 : N - 2) : a);
    const bool irr0 = iface[0] != pc, irr1 = iface[1] != pc + 1;  // face words not in the pair loads
    int src_lane = xghost ? ((icm[0] - (xs - 4)) >> 1) : lane;  // the mirror pair's lane (slots swapped)
    src_lane = src_lane < 0 ? 0 : (src_lane > 31 ? 31 : src_lane);
    const bool warp_xghost = __any_sync(FULL, xghost);
    const CartBC& bx = g.bc[a < 0 ? 0 : 1];
    float lid[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) lid[s] = (g.lid_u != nullptr) ? (float)(2.0 * g.lid_u[icm[s]]) : (float)g.bc[3].add[0];

    // ring slot layout (per warp): float2 pairs[kPairs][32] then float
    // singles[2][32]; pairs: 0 shu(pc, pc+1), 1 eu, 2 shv row k, 3 shv row k+1,
    // 4 ev row k, 5 ev row k+1, 6 g0u, 7 g0v, with BASE 8 base lo u row k-2,
    // 9 base lo v row k-2; singles: 0 shu(pc+2), 1 eu(pc+2)
    extern __shared__ __align__(16) float inc_ring[];
    float* wring = inc_ring + (size_t)(threadIdx.x >> 5) * kColRing * kWords * 32;
    auto pair_ptr = [&](int sl, int w) { return reinterpret_cast<float2*>(wring + (size_t)sl * kWords * 32) + w * 32 + lane; };
    auto single_ptr = [&](int sl, int w) { return wring + (size_t)sl * kWords * 32 + 2 * kPairs * 32 + w * 32 + lane; };
    auto row_of = [&](int k) {
      if (k >= 0 && k < N) return k;
      if (pery) return wrapi(k, N);
      int kk = k < 0 ? -k - 1 : 2 * N - 1 - k;
      return kk < 0 ? 0 : (kk >= N ? N - 1 : kk);
    };
    auto issue_row = [&](int k, int sl) {
      const long r0 = (long)row_of(k) * P + pc;
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 0)), shu + r0);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 1)), eu + r0);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 2)), shv + r0);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 3)), shv + r0 + P);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 4)), ev + r0);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 5)), ev + r0 + P);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 6)), A.g0[0] + r0);
      cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 7)), A.g0[1] + r0);
      cp_async4(single_ptr(sl, 0), shu + r0 + 2);
      cp_async4(single_ptr(sl, 1), eu + r0 + 2);
      if constexpr (BASE) {
        const long r2 = (long)row_of(k - 2) * P + pc;
        cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 8)), A.bl[0] + r2);
        cp_async8(reinterpret_cast<float*>(pair_ptr(sl, 9)), A.bl[1] + r2);
      }
      cp_async_commit();
    };
    int k_next = 0, k_end = 0;  // next row to issue, last row of the strip
    int slot = 0;               // ring slot of the next row to read (row r_first - 2 in slot 0)
    float blu[2] = {0.f, 0.f}, blv[2] = {0.f, 0.f};  // base lo of the u / v faces of row k - 2
    // consume row k: cell values of both columns (with ghosts), the u face
    // (iface), the lower v face and G0 at the lane's faces; put the next row in flight
    auto cell_row = [&](int k, ColCells2& c, float (&ufb)[2], float (&ufe)[2], float (&vlb)[2], float (&vle)[2],
                        float (&gu)[2], float (&gv)[2]) {
      cp_async_wait<kColRing - 1>();
      const float2 U = *pair_ptr(slot, 0), E = *pair_ptr(slot, 1), Vk = *pair_ptr(slot, 2), Vk1 = *pair_ptr(slot, 3);
      const float2 Fk = *pair_ptr(slot, 4), Fk1 = *pair_ptr(slot, 5), GU = *pair_ptr(slot, 6), GV = *pair_ptr(slot, 7);
      const float U2 = *single_ptr(slot, 0), E2 = *single_ptr(slot, 1);
      if constexpr (BASE) {
        const float2 LU = *pair_ptr(slot, 8), LV = *pair_ptr(slot, 9);
        blu[0] = LU.x;
        blu[1] = LU.y;
        blv[0] = LV.x;
        blv[1] = LV.y;
      }
      if (k_next <= k_end) issue_row(k_next, slot);
      else cp_async_commit();  // empty group: the wait count stays one row per call
      ++k_next;
      slot = (slot == kColRing - 1) ? 0 : slot + 1;
      c.p0[0] = 0.5f * (U.x + U.y);
      c.p0[1] = 0.5f * (U.y + U2);
      c.e0[0] = 0.5f * es * (E.x + E.y);
      c.e0[1] = 0.5f * es * (E.y + E2);
      c.p1[0] = 0.5f * (Vk.x + Vk1.x);
      c.p1[1] = 0.5f * (Vk.y + Vk1.y);
      c.e1[0] = 0.5f * es * (Fk.x + Fk1.x);
      c.e1[1] = 0.5f * es * (Fk.y + Fk1.y);
      ufb[0] = U.x;
      ufb[1] = U.y;
      ufe[0] = es * E.x;
      ufe[1] = es * E.y;
      gu[0] = GU.x;
      gu[1] = GU.y;
      if (irr0 || irr1) {  // face N, the periodic image, wall faces: direct loads (edge lanes only)
        const long rr = (long)row_of(k) * P;
        if (irr0) { ufb[0] = shu[rr + iface[0]]; ufe[0] = es * eu[rr + iface[0]]; gu[0] = A.g0[0][rr + iface[0]]; }
        if (irr1) { ufb[1] = shu[rr + iface[1]]; ufe[1] = es * eu[rr + iface[1]]; gu[1] = A.g0[0][rr + iface[1]]; }
      }
      vlb[0] = Vk.x;
      vlb[1] = Vk.y;
      vle[0] = es * Fk.x;
      vle[1] = es * Fk.y;
      gv[0] = GV.x;
      gv[1] = GV.y;
      if (warp_xghost) {  // x ghosts: the mirror pair's values (slots swapped) under the side's rule
        const float q00 = __shfl_sync(FULL, c.p0[1], src_lane), q01 = __shfl_sync(FULL, c.p0[0], src_lane);
        const float q10 = __shfl_sync(FULL, c.p1[1], src_lane), q11 = __shfl_sync(FULL, c.p1[0], src_lane);
        const float s00 = __shfl_sync(FULL, c.e0[1], src_lane), s01 = __shfl_sync(FULL, c.e0[0], src_lane);
        const float s10 = __shfl_sync(FULL, c.e1[1], src_lane), s11 = __shfl_sync(FULL, c.e1[0], src_lane);
        if (xghost) {
          c.p0[0] = cart_ghost_f(bx, 0, q00, false);
          c.p0[1] = cart_ghost_f(bx, 0, q01, false);
          c.p1[0] = cart_ghost_f(bx, 1, q10, false);
          c.p1[1] = cart_ghost_f(bx, 1, q11, false);
          c.e0[0] = cart_ghost_f(bx, 0, s00, true);
          c.e0[1] = cart_ghost_f(bx, 0, s01, true);
          c.e1[0] = cart_ghost_f(bx, 1, s10, true);
          c.e1[1] = cart_ghost_f(bx, 1, s11, true);
        }
      }
      if (!pery && (k < 0 || k >= N)) {  // y ghosts from the mirror row; the lid profile on the north u
        const CartBC& by = g.bc[k < 0 ? 2 : 3];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          if (k >= N && by.rule[0] == kInlet) c.p0[s] = lid[s] - c.p0[s];
          else c.p0[s] = cart_ghost_f(by, 0, c.p0[s], false);
          c.p1[s] = cart_ghost_f(by, 1, c.p1[s], false);
          c.e0[s] = cart_ghost_f(by, 0, c.e0[s], true);
          c.e1[s] = cart_ghost_f(by, 1, c.e1[s], true);
        }
      }
    };

    // w[0..4]: cell rows r-2 .. r+2; uf*/vl*/gq*[0..2]: faces of rows r .. r+2
    ColCells2 w[5];
    float ufb[3][2], ufe[3][2], vlb[3][2], vle[3][2], gqu[3][2], gqv[3][2], xb[2], xe[2];
    const int r_first = ys - 2;  // fy at face ys-1, then the totals of row ys-1
    const int r_last = (ys + kIncH >= N) ? N : ys + kIncH - 1;
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
    const bool out_lane = lane >= 2 && lane <= 30;  // columns xs .. xs + 57, both slots
    bool out_u[2], out_v[2], edge_u[2], rule_u[2];
    float wgt_u[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int i = a + s;
      out_u[s] = out_lane && i >= 0 && i <= N;
      out_v[s] = out_lane && i >= 0 && i < N;
      edge_u[s] = (i == 0 || i == N);
      rule_u[s] = fgx != kWrap && edge_u[s];
      wgt_u[s] = edge_u[s] ? 0.5f : 1.f;
    }
    float fyp0[2] = {0.f, 0.f}, fyp1[2] = {0.f, 0.f};  // y flux at face r
    float t1p[2] = {0.f, 0.f};                          // v total of row r-1
    for (int r = r_first; r <= r_last; ++r) {
      cell_row(r + 2, w[4], ufb[2], ufe[2], vlb[2], vle[2], gqu[2], gqv[2]);
      // y flux at face r+1 (rows r, r+1), cells r-1 .. r+2; face row N as stored
      float fy0[2], fy1[2];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        float vfb = vlb[1][s], vfe = vle[1][s];
        if (r + 1 == N) {
          const long id = (long)N * P + pc + s;
          vfb = shv[id];
          vfe = es * ev[id];
        }
        fy0[s] = quick_dflux(vfb, vfe, w[4].p0[s], w[3].p0[s], w[2].p0[s], w[1].p0[s], w[4].e0[s], w[3].e0[s],
                             w[2].e0[s], w[1].e0[s]);
        fy1[s] = quick_dflux(vfb, vfe, w[4].p1[s], w[3].p1[s], w[2].p1[s], w[1].p1[s], w[4].e1[s], w[3].e1[s],
                             w[2].e1[s], w[1].e1[s]);
      }
      if (r >= ys - 1) {  // warp-uniform
        const ColCells2& c = w[2];
        // x neighbours: U1 = column a - 1, U0 = column a - 2, D0 = column b + 1
        const float p0U1 = __shfl_up_sync(FULL, c.p0[1], 1), p0U0 = __shfl_up_sync(FULL, c.p0[0], 1);
        const float p0D0 = __shfl_down_sync(FULL, c.p0[0], 1);
        const float p1U1 = __shfl_up_sync(FULL, c.p1[1], 1), p1U0 = __shfl_up_sync(FULL, c.p1[0], 1);
        const float p1D0 = __shfl_down_sync(FULL, c.p1[0], 1);
        const float e0U1 = __shfl_up_sync(FULL, c.e0[1], 1), e0U0 = __shfl_up_sync(FULL, c.e0[0], 1);
        const float e0D0 = __shfl_down_sync(FULL, c.e0[0], 1);
        const float e1U1 = __shfl_up_sync(FULL, c.e1[1], 1), e1U0 = __shfl_up_sync(FULL, c.e1[0], 1);
        const float e1D0 = __shfl_down_sync(FULL, c.e1[0], 1);
        // x fluxes at faces a (cells a-2 .. a+1) and b (cells b-2 .. b+1)
        const float fx0a = quick_dflux(ufb[0][0], ufe[0][0], c.p0[1], c.p0[0], p0U1, p0U0, c.e0[1], c.e0[0], e0U1, e0U0);
        const float fx1a = quick_dflux(ufb[0][0], ufe[0][0], c.p1[1], c.p1[0], p1U1, p1U0, c.e1[1], c.e1[0], e1U1, e1U0);
        const float fx0b = quick_dflux(ufb[0][1], ufe[0][1], p0D0, c.p0[1], c.p0[0], p0U1, e0D0, c.e0[1], c.e0[0], e0U1);
        const float fx1b = quick_dflux(ufb[0][1], ufe[0][1], p1D0, c.p1[1], c.p1[0], p1U1, e1D0, c.e1[1], c.e1[0], e1U1);
        const float fx0r = __shfl_down_sync(FULL, fx0a, 1), fx1r = __shfl_down_sync(FULL, fx1a, 1);  // face b + 1
        // totals of cells a and b
        const float conv0a = (fx0b - fx0a) * idx_ + (fy0[0] - fyp0[0]) * idy_;
        const float conv1a = (fx1b - fx1a) * idx_ + (fy1[0] - fyp1[0]) * idy_;
        const float conv0b = (fx0r - fx0b) * idx_ + (fy0[1] - fyp0[1]) * idy_;
        const float conv1b = (fx1r - fx1b) * idx_ + (fy1[1] - fyp1[1]) * idy_;
        const float visc0a = (c.e0[1] - 2.f * c.e0[0] + e0U1) * vx + (w[3].e0[0] - 2.f * c.e0[0] + w[1].e0[0]) * vy;
        const float visc1a = (c.e1[1] - 2.f * c.e1[0] + e1U1) * vx + (w[3].e1[0] - 2.f * c.e1[0] + w[1].e1[0]) * vy;
        const float visc0b = (e0D0 - 2.f * c.e0[1] + c.e0[0]) * vx + (w[3].e0[1] - 2.f * c.e0[1] + w[1].e0[1]) * vy;
        const float visc1b = (e1D0 - 2.f * c.e1[1] + c.e1[0]) * vx + (w[3].e1[1] - 2.f * c.e1[1] + w[1].e1[1]) * vy;
        const float t0[2] = {visc0a - conv0a, visc0b - conv0b};
        const float t1[2] = {visc1a - conv1a, visc1b - conv1b};
        const float t0l[2] = {__shfl_up_sync(FULL, t0[1], 1), t0[0]};  // u total of cells a - 1 and a
        if (r >= ys) {  // warp-uniform
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const int i = a + s;
            const long id = (long)r * P + i;
            if (out_u[s] && r < N) {  // u face (i, r)
              float avg = 0.5f * (t0l[s] + t0[s]);
              if (rule_u[s]) avg = (fgx == kReflect) ? 0.f : 0.5f * (i == 0 ? t0[s] : t0l[s]);
              const float e = rk * (gqu[0][s] + (avg - c15 * ufe[0][s]));
              A.eout[0][id] = e;
              n0 = fmaf(wgt_u[s] * e, e, n0);
              if constexpr (BASE) {  // u_b + e_s at u face (i, r); face words off the pair loads directly
                const float lo = (s == 0 ? irr0 : irr1) ? A.bl[0][id] : blu[s];
                const ff nb = ff_add_f(ff_make(ufb[0][s], lo), ufe[0][s]);
                A.obh[0][id] = nb.hi;
                A.obl[0][id] = nb.lo;
              }
            }
            if (out_v[s]) {  // v face (i, r), r <= N
              const bool edge_v = (r == 0 || r == N);
              float avg = 0.5f * (t1p[s] + t1[s]);
              if (fgy != kWrap && edge_v) avg = (fgy == kReflect) ? 0.f : 0.5f * (r == 0 ? t1[s] : t1p[s]);
              float ecur = vle[0][s], gcur = gqv[0][s];
              float bh = vlb[0][s], bo = blv[s];
              if (r == N) {  // face row N as stored
                ecur = es * ev[id];
                gcur = A.g0[1][id];
                if constexpr (BASE) {
                  bh = shv[id];
                  bo = A.bl[1][id];
                }
              }
              const float e = rk * (gcur + (avg - c15 * ecur));
              A.eout[1][id] = e;
              n1 = fmaf(edge_v ? 0.5f * e : e, e, n1);
              if constexpr (BASE) {  // u_b + e_s at v face (i, r)
                const ff nb = ff_add_f(ff_make(bh, bo), ecur);
                A.obh[1][id] = nb.hi;
                A.obl[1][id] = nb.lo;
              }
            }
          }
        }
        t1p[0] = t1[0];
        t1p[1] = t1[1];
      }
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        fyp0[s] = fy0[s];
        fyp1[s] = fy1[s];
      }
      w[0] = w[1]; w[1] = w[2]; w[2] = w[3]; w[3] = w[4];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        ufb[0][s] = ufb[1][s]; ufe[0][s] = ufe[1][s]; ufb[1][s] = ufb[2][s]; ufe[1][s] = ufe[2][s];
        gqu[0][s] = gqu[1][s]; gqv[0][s] = gqv[1][s]; gqu[1][s] = gqu[2][s]; gqv[1][s] = gqv[2][s];
        vlb[0][s] = vlb[1][s]; vle[0][s] = vle[1][s]; vlb[1][s] = vlb[2][s]; vle[1][s] = vle[2][s];
      }
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
