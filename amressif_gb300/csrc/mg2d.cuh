// Geometric multigrid for the pressure Poisson equation L phi = f (2D).
//
// Replaces the AMReX MLMG / MLABecLaplacian solve of poisson.cpp:41-186 (a=0,
// b=-1, B=1: L is the 5-point Laplacian, homogeneous Neumann on walls,
// periodic where both sides are periodic). Cell-centred hierarchy, levels
// coarsened by 2 while n % 4 == 0 and n > 4, rediscretised operators, cell
// averaging restriction, bilinear prolongation, red-black Gauss-Seidel
// smoothing. Levels with n >= 64 run as tiled kernels whose two smoothing
// sweeps are temporally blocked in shared memory; every level with n <= 32
// runs inside one persistent CTA that ends with a conjugate-gradient solve on
// the coarsest level. T = double (plain FP64 solver) or float (V-cycles of the
// mixed-precision defect correction).
#pragma once
#include <type_traits>
#include "bounds.cuh"
#include "ns_common.cuh"

namespace ns {

constexpr int kMaxLevels = 16;
// levels with n <= kBottomN live in the bottom CTA: x, f, r of each level and
// the coarsest level's CG vectors in dynamic shared memory, at most 43 KB in
// FP64 (a lone 30^2 coarsest level), within the default 48 KB. The 64^2 level
// in the block as well made the 4096^2 V-cycle slower (0.4855 against 0.476 ms).
constexpr int kBottomN = 32;

template <typename T>
struct MGLevels {
  int L;                          // number of levels
  int n[kMaxLevels];
  long pitch[kMaxLevels];
  T* x[kMaxLevels];
  T* x2[kMaxLevels];              // smoother output: the smoothers read x and write x2 (the
                                  // caller swaps them), so no block reads a halo another block
                                  // has already overwritten
  T* f[kMaxLevels];
  double invh2[kMaxLevels][2];
  // 1/diagonal for the (east+west, north+south) neighbour counts: index a + 3 b
  double invdiag[kMaxLevels][9];
  // the same constants in T, so that no conversion runs per update
  T ih[kMaxLevels][2];
  T idg[kMaxLevels][9];
  int periodic[2];
  const double* fmean;            // subtracted from f at level 0 when non-null
  unsigned long long* check;      // bounds-check build: status words (bounds.cuh); null otherwise
};

// Gauss-Seidel update of one cell from its four neighbours; w* = 0 removes an
// absent (Neumann) neighbour from both the sum and the diagonal.
// explicitly rounded operations: every smoother kernel (tiled, warp-marching)
// forms exactly the same value, whatever the compiler contracts elsewhere
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }

// bilinear cell-centred prolongation weights 9/16, 3/16, 3/16, 1/16 (explicitly rounded)
template <typename T>
__device__ __forceinline__ T prolong_add(T x, T c00, T c10, T c01, T c11) {
  const T a = rn_mul((T)0.5625, c00), b = rn_mul((T)0.1875, rn_add(c10, c01)), d = rn_mul((T)0.0625, c11);
  return rn_add(x, rn_add(rn_add(a, b), d));
}

template <typename T>
__device__ __forceinline__ T gs_update(T xe, T xw, T xn, T xs, bool we, bool ww, bool wn, bool wsn, T ihx, T ihy, T f,
                                       const T* idg) {
  const T zero = (T)0;
  const T sx = rn_mul(rn_add(we ? xe : zero, ww ? xw : zero), ihx);
  const T sy = rn_mul(rn_add(wn ? xn : zero, wsn ? xs : zero), ihy);
  const int k = (int)we + (int)ww + 3 * ((int)wn + (int)wsn);
  return rn_mul(rn_add(rn_add(sx, sy), -f), idg[k]);
}

template <typename T>
__device__ __forceinline__ T level_f(const MGLevels<T>& M, int l, long id) {
  T v = M.f[l][id];
  if (l == 0 && M.fmean != nullptr) v = v - (T)(*M.fmean);
  return v;
}

// ---------------------------------------------------------------------------
// Tiled smoother: optional bilinear prolongation + correction, then 2 RB-GS
// sweeps (4 half-sweeps) with temporal blocking (halo 4).
// mode: 0 = pre-smoothing (colours red, black, red, black; x may start at 0)
//       1 = prolongate coarse x, add, then post-smoothing (black first)
// ---------------------------------------------------------------------------
template <typename T, int TX, int TY>
struct SmoothSmem {
  static constexpr int H = 4;
  static constexpr int W = TX + 2 * H, HH = TY + 2 * H;
  T x[HH][W];
  T f[HH][W];
};

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(256) k_mg_smooth(MGLevels<T> M, int l, int mode, int x_zero) {
  using SM = SmoothSmem<T, TX, TY>;
  constexpr int H = SM::H;
  __shared__ SM sm;
  const int n = M.n[l];
  const long P = M.pitch[l];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool px = M.periodic[0], py = M.periodic[1];
  const T ihx = M.ih[l][0], ihy = M.ih[l][1];
  // FAST: the tile and its halo (and, for the prolongation, every coarse
  // neighbour) lie at least two cells inside the domain, so no wrap, wall
  // weight or range test is needed; the remaining operations, and the bits,
  // are those of the general path
  auto body = [&](auto fast_c) {
  constexpr bool FAST = decltype(fast_c)::value;
  for (int t = tid; t < SM::W * SM::HH; t += NT) {
    const int lx = t % SM::W, ly = t / SM::W;
    const int a = x0 - H + lx, b = y0 - H + ly;
    const bool in = FAST || ((px || (a >= 0 && a < n)) && (py || (b >= 0 && b < n)));
    T xv = (T)0, fv = (T)0;
    if (in && NS_BCHK(M.check, (long)(FAST ? b : wrapi(b, n)) * P + (FAST ? a : wrapi(a, n)), P, n + 1, n - 1, 51)) {
      const int aa = FAST ? a : wrapi(a, n), bb = FAST ? b : wrapi(b, n);
      const long id = (long)bb * P + aa;
      if (!x_zero) xv = M.x[l][id];
      fv = level_f(M, l, id);
      if (mode == 1) {
        // bilinear cell-centred prolongation of the coarse correction
        const int nc = M.n[l + 1];
        const long Pc = M.pitch[l + 1];
        const int I = aa >> 1, J = bb >> 1;
        int I2 = I + ((aa & 1) ? 1 : -1), J2 = J + ((bb & 1) ? 1 : -1);
        if (!FAST) {
          I2 = px ? wrapi(I2, nc) : min(max(I2, 0), nc - 1);
          J2 = py ? wrapi(J2, nc) : min(max(J2, 0), nc - 1);
        }
        const T* xc = M.x[l + 1];
        if (!NS_BCHK(M.check, (long)J * Pc + I, Pc, nc + 1, nc - 1, 52) || !NS_BCHK(M.check, (long)J2 * Pc + I2, Pc, nc + 1, nc - 1, 53))
          continue;
        const T c00 = xc[(long)J * Pc + I], c10 = xc[(long)J * Pc + I2];
        const T c01 = xc[(long)J2 * Pc + I], c11 = xc[(long)J2 * Pc + I2];
        xv = prolong_add(xv, c00, c10, c01, c11);
      }
    }
    sm.x[ly][lx] = xv;
    sm.f[ly][lx] = fv;
  }
  __syncthreads();
  const int cfirst = (mode == 1) ? 1 : 0;
#pragma unroll  // r, w, h, w2 become constants: no runtime integer division per cell
  for (int s = 0; s < 4; ++s) {
    const int color = (cfirst + s) & 1;
    const int r = H - 1 - s;
    const int w = TX + 2 * r, h = TY + 2 * r;
    const int w2 = (w + 1) / 2;  // cells of one colour per row (at most)
    for (int t = tid; t < w2 * h; t += NT) {
      const int b = y0 - r + t / w2;
      const int a0 = x0 - r;
      const int a = a0 + 2 * (t % w2) + (((a0 + b) & 1) != color ? 1 : 0);
      if (a >= a0 + w) continue;
      if (!FAST && !px && (a < 0 || a >= n)) continue;
      if (!FAST && !py && (b < 0 || b >= n)) continue;
      const int lx = a - (x0 - H), ly = b - (y0 - H);
      const bool we = FAST || px || a + 1 < n, ww = FAST || px || a > 0;
      const bool wn = FAST || py || b + 1 < n, wsn = FAST || py || b > 0;
      sm.x[ly][lx] = gs_update<T>(sm.x[ly][lx + 1], sm.x[ly][lx - 1], sm.x[ly + 1][lx], sm.x[ly - 1][lx],
                                  we, ww, wn, wsn, ihx, ihy, sm.f[ly][lx], M.idg[l]);
    }
    __syncthreads();
  }
  for (int t = tid; t < TX * TY; t += NT) {
    const int a = x0 + t % TX, b = y0 + t / TX;
    if ((FAST || (a < n && b < n)) && NS_BCHK(M.check, (long)b * P + a, P, n + 1, n - 1, 54)) M.x2[l][(long)b * P + a] = sm.x[b - (y0 - H)][a - (x0 - H)];
  }
  };
  const bool fast = x0 - H >= 2 && x0 + TX + H <= n - 2 && y0 - H >= 2 && y0 + TY + H <= n - 2;
  if (fast) body(std::true_type{});
  else body(std::false_type{});
}

// ---------------------------------------------------------------------------
// Warp-marching smoother for the fine levels: the two red-black sweeps of
// k_mg_smooth (same colours, same update arithmetic, same prolongation), laid
// out for the GPU's issue rate instead of block barriers. One warp owns a
// strip of 64 columns, two per lane (kColSmOut = 56 output columns between
// four halo columns on each side), and a chunk of kColSmH rows, and climbs it
// with the four half-sweeps as a skewed wavefront: at step t half-sweep s
// works on row t - s, over the rows the tiled kernel gives it, so a row is
// final once half-sweep 3 has passed it. y neighbours sit in a six-row
// register window, x neighbours come by warp shuffle, the next row is loaded
// one step ahead. Halo columns may take wrong values from the strip edge; an
// error moves one column per half-sweep, so four halo columns keep the output
// columns exact.
// ---------------------------------------------------------------------------
constexpr int kColSmOut = 56, kColSmH = 64;

template <typename T>
struct SmRow {
  T x0, x1, f0, f1;
};

template <typename T>
__device__ __forceinline__ SmRow<T> sm_load_row(const MGLevels<T>& M, int l, int mode, int x_zero, int r, int c0, bool cin) {
  SmRow<T> o;
  o.x0 = o.x1 = o.f0 = o.f1 = (T)0;
  const int n = M.n[l];
  const bool px = M.periodic[0], py = M.periodic[1];
  if (!cin || !(py || (r >= 0 && r < n))) return o;
  const int rr = wrapi(r, n), w0 = wrapi(c0, n);  // w0 even, w0 + 1 < n
  const long id = (long)rr * M.pitch[l] + w0;
  // level arrays are pitch x (n + 1) elements (bounds-check build only)
  if (!NS_BCHK(M.check, id, M.pitch[l], n + 1, n - 2, 41)) return o;
  if (!x_zero) { o.x0 = M.x[l][id]; o.x1 = M.x[l][id + 1]; }
  o.f0 = level_f(M, l, id);
  o.f1 = level_f(M, l, id + 1);
  if (mode == 1) {  // bilinear prolongation of the coarse correction (as k_mg_smooth)
    const int nc = M.n[l + 1];
    const long Pc = M.pitch[l + 1];
    const int I = w0 >> 1, J = rr >> 1;
    int Im = I - 1, Ip = I + 1, J2 = J + ((rr & 1) ? 1 : -1);
    Im = px ? wrapi(Im, nc) : max(Im, 0);
    Ip = px ? wrapi(Ip, nc) : min(Ip, nc - 1);
    J2 = py ? wrapi(J2, nc) : min(max(J2, 0), nc - 1);
    const T* xc = M.x[l + 1];
    if (!NS_BCHK(M.check, (long)J * Pc + Im, Pc, nc + 1, nc - 1, 42) || !NS_BCHK(M.check, (long)J2 * Pc + Ip, Pc, nc + 1, nc - 1, 43) ||
        !NS_BCHK(M.check, (long)J2 * Pc + Im, Pc, nc + 1, nc - 1, 44) || !NS_BCHK(M.check, (long)J * Pc + Ip, Pc, nc + 1, nc - 1, 44))
      return o;
    const T c00 = xc[(long)J * Pc + I], c01 = xc[(long)J2 * Pc + I];
    const T cm0 = xc[(long)J * Pc + Im], cm1 = xc[(long)J2 * Pc + Im];  // column w0 - 1 side (w0 even)
    const T cp0 = xc[(long)J * Pc + Ip], cp1 = xc[(long)J2 * Pc + Ip];  // column w0 + 2 side (w0 + 1 odd)
    o.x0 = prolong_add(o.x0, c00, cm0, c01, cm1);
    o.x1 = prolong_add(o.x1, c00, cp0, c01, cp1);
  }
  return o;
}

// The climb of one warp. FAST: every column of the warp and every row of its
// wavefront lies inside the domain away from the walls (or the direction is
// periodic), so each update has all four neighbours and the diagonal entry of
// a full stencil: the boundary weights, the diagonal-table index and the
// domain tests drop out. The arithmetic (and so every bit of the result) is
// that of gs_update with all weights set.
template <typename T, bool FAST>
__device__ __forceinline__ void smooth_col_march(const MGLevels<T>& M, int l, int mode, int x_zero, int xs, int y0,
                                                 int lane) {
  constexpr unsigned FULL = 0xffffffffu;
  const int n = M.n[l];
  const long P = M.pitch[l];
  const bool px = M.periodic[0], py = M.periodic[1];
  const T ihx = M.ih[l][0], ihy = M.ih[l][1];
  const T idg_full = M.idg[l][8];  // a + 3 b with two neighbours in each direction
  const int cfirst = (mode == 1) ? 1 : 0;
  const int c0 = xs - 4 + 2 * lane, c1 = c0 + 1;   // c0 even; both columns in or both out (n even)
  const bool cin = px || (c0 >= 0 && c1 < n);
  const bool we0 = true, ww0 = px || c0 > 0;     // neighbours of c0 (its east neighbour is c1)
  const bool we1 = px || c1 + 1 < n, ww1 = true; // neighbours of c1
  const bool out_lane = lane >= 2 && lane <= 29; // columns xs .. xs + 55
  // window: xw[k] = row t - 4 + k (k = 0..5), fw[k] = f of row t - 3 + k (k = 0..3)
  T xw[6][2], fw[4][2];
#pragma unroll
  for (int k = 0; k < 6; ++k) xw[k][0] = xw[k][1] = (T)0;
#pragma unroll
  for (int k = 0; k < 4; ++k) fw[k][0] = fw[k][1] = (T)0;
  const int t0 = y0 - 3, t1 = y0 + kColSmH + 2;  // rows of half-sweep 0; half-sweep s runs for t >= t0 + 2 s
  {
    const SmRow<T> a = sm_load_row(M, l, mode, x_zero, t0 - 1, c0, cin);
    const SmRow<T> b = sm_load_row(M, l, mode, x_zero, t0, c0, cin);
    xw[3][0] = a.x0; xw[3][1] = a.x1;
    xw[4][0] = b.x0; xw[4][1] = b.x1;
    fw[3][0] = b.f0; fw[3][1] = b.f1;
  }
  SmRow<T> nxt = sm_load_row(M, l, mode, x_zero, t0 + 1, c0, cin);
  for (int t = t0; t <= t1; ++t) {
    const SmRow<T> cur = nxt;  // row t + 1
    nxt = sm_load_row(M, l, mode, x_zero, t + 2, c0, cin);
    xw[5][0] = cur.x0;
    xw[5][1] = cur.x1;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int r = t - s, k = 4 - s;
      const int color = (cfirst + s) & 1;
      const bool upd1 = ((r & 1) != color);  // c0 has the colour r & 1, c1 the other
      const T e_of_0 = __shfl_down_sync(FULL, xw[k][0], 1);  // column c1 + 1 (lane + 1's c0)
      const T w_of_1 = __shfl_up_sync(FULL, xw[k][1], 1);    // column c0 - 1 (lane - 1's c1)
      if constexpr (FAST) {
        if (t >= t0 + 2 * s) {  // warp-uniform
          const T xe = upd1 ? e_of_0 : xw[k][1], xwv = upd1 ? xw[k][0] : w_of_1;
          const T xn = upd1 ? xw[k + 1][1] : xw[k + 1][0], xs_ = upd1 ? xw[k - 1][1] : xw[k - 1][0];
          const T fv = upd1 ? fw[3 - s][1] : fw[3 - s][0];
          const T sx = rn_mul(rn_add(xe, xwv), ihx), sy = rn_mul(rn_add(xn, xs_), ihy);
          const T v = rn_mul(rn_add(rn_add(sx, sy), -fv), idg_full);
          if (upd1) xw[k][1] = v;
          else xw[k][0] = v;
        }
      } else {
        const bool rok = r >= y0 - 3 + s && r <= y0 + kColSmH + 2 - s && (py || (r >= 0 && r < n)) && cin;
        const bool wn = py || r + 1 < n, wsn = py || r > 0;
        if (rok) {
          if (!upd1) {
            xw[k][0] = gs_update<T>(xw[k][1], w_of_1, xw[k + 1][0], xw[k - 1][0], we0, ww0, wn, wsn, ihx, ihy, fw[3 - s][0], M.idg[l]);
          } else {
            xw[k][1] = gs_update<T>(e_of_0, xw[k][0], xw[k + 1][1], xw[k - 1][1], we1, ww1, wn, wsn, ihx, ihy, fw[3 - s][1], M.idg[l]);
          }
        }
      }
    }
    const int ro = t - 3;
    if (out_lane && c0 >= 0 && c1 < n && ro >= y0 && ro < y0 + kColSmH && ro < n &&
        NS_BCHK(M.check, (long)ro * P + c0, P, n + 1, n - 2, 45)) {  // real cells only
      const long id = (long)ro * P + c0;
      M.x2[l][id] = xw[1][0];
      M.x2[l][id + 1] = xw[1][1];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) { xw[k][0] = xw[k + 1][0]; xw[k][1] = xw[k + 1][1]; }
#pragma unroll
    for (int k = 0; k < 3; ++k) { fw[k][0] = fw[k + 1][0]; fw[k][1] = fw[k + 1][1]; }
    fw[3][0] = cur.f0;
    fw[3][1] = cur.f1;
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_mg_smooth_col(MGLevels<T> M, int l, int mode, int x_zero) {
  const int n = M.n[l];
  const int lane = threadIdx.x & 31;
  const int nsx = (n + kColSmOut - 1) / kColSmOut, nsy = (n + kColSmH - 1) / kColSmH;
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (gw >= nsx * nsy) return;  // warp-uniform; the kernel has no block barrier
  const int xs = (gw % nsx) * kColSmOut, y0 = (gw / nsx) * kColSmH;
  const bool px = M.periodic[0], py = M.periodic[1];
  // the fast climb needs both columns of every lane inside the domain with
  // both x neighbours, and every row of the wavefront (y0 - 3 .. y0 + kColSmH
  // + 2, plus the rows above and below it) inside with both y neighbours
  const int c0 = xs - 4 + 2 * lane;
  const bool lane_inner = px || (c0 >= 1 && c0 + 2 < n);
  const bool rows_inner = py || (y0 - 3 >= 1 && y0 + kColSmH + 2 <= n - 2);
  if (__all_sync(0xffffffffu, lane_inner) && rows_inner)
    smooth_col_march<T, true>(M, l, mode, x_zero, xs, y0, lane);
  else
    smooth_col_march<T, false>(M, l, mode, x_zero, xs, y0, lane);
}

// residual at level l restricted (cell average) to the RHS of level l+1
template <typename T>
__global__ void __launch_bounds__(256) k_mg_restrict(MGLevels<T> M, int l) {
  const int nc = M.n[l + 1];
  const int I = blockIdx.x * 32 + (threadIdx.x & 31);
  const int J = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (I >= nc || J >= nc) return;
  const int n = M.n[l];
  const long P = M.pitch[l];
  const bool px = M.periodic[0], py = M.periodic[1];
  const T ihx = M.ih[l][0], ihy = M.ih[l][1];
  const T* x = M.x[l];
  // FAST: the four fine cells and their neighbours lie inside the domain
  // (no wrap, no wall); the same operations, and the same bits
  auto body = [&](auto fast_c) {
    constexpr bool FAST = decltype(fast_c)::value;
    T s = (T)0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int a = 2 * I + (q & 1), b = 2 * J + (q >> 1);
      const long id = (long)b * P + a;
      const T xc = x[id];
      T lap = (T)0;
      if (FAST || px || a + 1 < n) lap += (x[(long)b * P + (FAST ? a + 1 : wrapi(a + 1, n))] - xc) * ihx;
      if (FAST || px || a > 0) lap += (x[(long)b * P + (FAST ? a - 1 : wrapi(a - 1, n))] - xc) * ihx;
      if (FAST || py || b + 1 < n) lap += (x[(long)(FAST ? b + 1 : wrapi(b + 1, n)) * P + a] - xc) * ihy;
      if (FAST || py || b > 0) lap += (x[(long)(FAST ? b - 1 : wrapi(b - 1, n)) * P + a] - xc) * ihy;
      s += level_f(M, l, id) - lap;
    }
    M.f[l + 1][(long)J * M.pitch[l + 1] + I] = (T)0.25 * s;
  };
  if (I >= 1 && 2 * I + 2 < n && J >= 1 && 2 * J + 2 < n) body(std::true_type{});
  else body(std::false_type{});
}

// max |f - L x| at level 0 (plain solver convergence check); red_out[0]
template <typename T>
__global__ void __launch_bounds__(256) k_mg_resnorm(MGLevels<T> M, double* part, unsigned* counter, double* red_out) {
  const int n = M.n[0];
  const long P = M.pitch[0];
  const int a = blockIdx.x * 32 + (threadIdx.x & 31);
  const int b = blockIdx.y * 8 + (threadIdx.x >> 5);
  double v[1] = {0.0};
  if (a < n && b < n) {
    const bool px = M.periodic[0], py = M.periodic[1];
    const T ihx = M.ih[0][0], ihy = M.ih[0][1];
    const T* x = M.x[0];
    const long id = (long)b * P + a;
    const T xc = x[id];
    T lap = (T)0;
    if (px || a + 1 < n) lap += (x[(long)b * P + wrapi(a + 1, n)] - xc) * ihx;
    if (px || a > 0) lap += (x[(long)b * P + wrapi(a - 1, n)] - xc) * ihx;
    if (py || b + 1 < n) lap += (x[(long)wrapi(b + 1, n) * P + a] - xc) * ihy;
    if (py || b > 0) lap += (x[(long)wrapi(b - 1, n) * P + a] - xc) * ihy;
    v[0] = fabs((double)(level_f(M, 0, id) - lap));
  }
  if (grid_reduce_last<1>(v, part, counter, 1u) && threadIdx.x == 0) red_out[0] = v[0];
}

// ---------------------------------------------------------------------------
// Persistent bottom CTA: every level from lb (n <= 32) to the coarsest, one
// V(2,2) cycle, CG on the coarsest level (constant mode projected out).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = (T)0;
  for (int w = 0; w < nw; ++w) s += red[w];
  return s;
}

// Dynamic shared memory: x, f, r for every level from lb, then the three CG
// vectors of the coarsest level.
template <typename T>
__global__ void __launch_bounds__(1024) k_mg_bottom(MGLevels<T> M, int lb, int x_zero) {
  extern __shared__ __align__(16) unsigned char bottom_smem_raw[];
  __shared__ T red[32];
  __shared__ int off[kMaxLevels];
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool px = M.periodic[0], py = M.periodic[1];
  int cells = 0;
  for (int l = lb; l < M.L; ++l) cells += M.n[l] * M.n[l];
  const int ncc = M.n[M.L - 1] * M.n[M.L - 1];
  T* sx = reinterpret_cast<T*>(bottom_smem_raw);
  T* sf = sx + cells;
  T* sr = sf + cells;
  T* pcg = sr + cells;
  T* qcg = pcg + ncc;
  T* rcg = qcg + ncc;
  if (tid == 0) {
    int o = 0;
    for (int l = lb; l < M.L; ++l) { off[l] = o; o += M.n[l] * M.n[l]; }
  }
  __syncthreads();
  {
    const int n = M.n[lb];
    for (int t = tid; t < n * n; t += NT) {
      const long id = (long)(t / n) * M.pitch[lb] + (t % n);
      sf[off[lb] + t] = level_f(M, lb, id);
      sx[off[lb] + t] = x_zero ? (T)0 : M.x[lb][id];
    }
  }
  __syncthreads();
  auto smooth = [&](int l, int cfirst) {
    const int n = M.n[l];
    const T ihx = M.ih[l][0], ihy = M.ih[l][1];
    T* x = sx + off[l];
    const T* f = sf + off[l];
    for (int s = 0; s < 4; ++s) {
      const int color = (cfirst + s) & 1;
      for (int t = tid; t < n * n; t += NT) {
        const int a = t % n, b = t / n;
        if (((a + b) & 1) != color) continue;
        const bool we = px || a + 1 < n, ww = px || a > 0;
        const bool wn = py || b + 1 < n, wsn = py || b > 0;
        const T xe = x[b * n + wrapi(a + 1, n)], xw = x[b * n + wrapi(a - 1, n)];
        const T xn = x[wrapi(b + 1, n) * n + a], xs = x[wrapi(b - 1, n) * n + a];
        x[t] = gs_update<T>(xe, xw, xn, xs, we, ww, wn, wsn, ihx, ihy, f[t], M.idg[l]);
      }
      __syncthreads();
    }
  };
  auto apply_negL = [&](int l, const T* in, T* out) {  // out = -L in
    const int n = M.n[l];
    const T ihx = M.ih[l][0], ihy = M.ih[l][1];
    for (int t = tid; t < n * n; t += NT) {
      const int a = t % n, b = t / n;
      const T c = in[t];
      T lap = (T)0;
      if (px || a + 1 < n) lap += (in[b * n + wrapi(a + 1, n)] - c) * ihx;
      if (px || a > 0) lap += (in[b * n + wrapi(a - 1, n)] - c) * ihx;
      if (py || b + 1 < n) lap += (in[wrapi(b + 1, n) * n + a] - c) * ihy;
      if (py || b > 0) lap += (in[wrapi(b - 1, n) * n + a] - c) * ihy;
      out[t] = -lap;
    }
  };
  const int Lc = M.L - 1;
  for (int l = lb; l < Lc; ++l) {
    smooth(l, 0);
    // residual -> restrict
    const int n = M.n[l];
    apply_negL(l, sx + off[l], sr + off[l]);
    __syncthreads();
    const int nc = M.n[l + 1];
    for (int t = tid; t < nc * nc; t += NT) {
      const int I = t % nc, J = t / nc;
      T s = (T)0;
      for (int q = 0; q < 4; ++q) {
        const int c = (2 * J + (q >> 1)) * n + 2 * I + (q & 1);
        s += sf[off[l] + c] + sr[off[l] + c];  // f - L x = f + (-L x)
      }
      sf[off[l + 1] + t] = (T)0.25 * s;
      sx[off[l + 1] + t] = (T)0;
    }
    __syncthreads();
  }
  // coarsest level: CG on -L x = -f with the constant mode removed
  {
    const int n = M.n[Lc], nn = n * n;
    T* x = sx + off[Lc];
    T* b = sf + off[Lc];
    T mean = block_sum<T>([&] { T s = 0; for (int t = tid; t < nn; t += NT) s += b[t]; return s; }(), red) / (T)nn;
    for (int t = tid; t < nn; t += NT) { rcg[t] = -(b[t] - mean); x[t] = (T)0; pcg[t] = rcg[t]; }
    __syncthreads();
    T rr = block_sum<T>([&] { T s = 0; for (int t = tid; t < nn; t += NT) s += rcg[t] * rcg[t]; return s; }(), red);
    const T rr0 = rr;
    const T eps = sizeof(T) == 8 ? (T)1e-28 : (T)1e-12;
    for (int it = 0; it < 4 * nn && rr > eps * rr0 && rr > (T)0; ++it) {
      apply_negL(Lc, pcg, qcg);
      __syncthreads();
      const T pq = block_sum<T>([&] { T s = 0; for (int t = tid; t < nn; t += NT) s += pcg[t] * qcg[t]; return s; }(), red);
      if (!(pq > (T)0)) break;
      const T alpha = rr / pq;
      for (int t = tid; t < nn; t += NT) { x[t] += alpha * pcg[t]; rcg[t] -= alpha * qcg[t]; }
      __syncthreads();
      const T rr2 = block_sum<T>([&] { T s = 0; for (int t = tid; t < nn; t += NT) s += rcg[t] * rcg[t]; return s; }(), red);
      const T beta = rr2 / rr;
      rr = rr2;
      for (int t = tid; t < nn; t += NT) pcg[t] = rcg[t] + beta * pcg[t];
      __syncthreads();
    }
  }
  for (int l = Lc - 1; l >= lb; --l) {
    const int n = M.n[l], nc = M.n[l + 1];
    const T* xc = sx + off[l + 1];
    T* x = sx + off[l];
    for (int t = tid; t < n * n; t += NT) {
      const int a = t % n, b = t / n;
      const int I = a >> 1, J = b >> 1;
      int I2 = I + ((a & 1) ? 1 : -1), J2 = J + ((b & 1) ? 1 : -1);
      I2 = px ? wrapi(I2, nc) : min(max(I2, 0), nc - 1);
      J2 = py ? wrapi(J2, nc) : min(max(J2, 0), nc - 1);
      x[t] += (T)0.5625 * xc[J * nc + I] + (T)0.1875 * (xc[J * nc + I2] + xc[J2 * nc + I]) + (T)0.0625 * xc[J2 * nc + I2];
    }
    __syncthreads();
    smooth(l, 1);
  }
  {
    const int n = M.n[lb];
    for (int t = tid; t < n * n; t += NT) M.x[lb][(long)(t / n) * M.pitch[lb] + (t % n)] = sx[off[lb] + t];
  }
}

}  // namespace ns
