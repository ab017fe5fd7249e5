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
#include "ns_common.cuh"

namespace ns {

constexpr int kMaxLevels = 16;
constexpr int kBottomN = 32;       // levels with n <= kBottomN live in the bottom CTA
constexpr int kBottomCells = 1400; // >= 32^2 + 16^2 + 8^2 + 4^2

template <typename T>
struct MGLevels {
  int L;                          // number of levels
  int n[kMaxLevels];
  long pitch[kMaxLevels];
  T* x[kMaxLevels];
  T* f[kMaxLevels];
  double invh2[kMaxLevels][2];
  // 1/diagonal for the (east+west, north+south) neighbour counts: index a + 3 b
  double invdiag[kMaxLevels][9];
  // the same constants in T, so that no conversion runs per update
  T ih[kMaxLevels][2];
  T idg[kMaxLevels][9];
  int periodic[2];
  const double* fmean;            // subtracted from f at level 0 when non-null
};

// Gauss-Seidel update of one cell from its four neighbours; w* = 0 removes an
// absent (Neumann) neighbour from both the sum and the diagonal.
template <typename T>
__device__ __forceinline__ T gs_update(T xe, T xw, T xn, T xs, bool we, bool ww, bool wn, bool wsn, T ihx, T ihy, T f,
                                       const T* idg) {
  const T zero = (T)0;
  const T sum = ((we ? xe : zero) + (ww ? xw : zero)) * ihx + ((wn ? xn : zero) + (wsn ? xs : zero)) * ihy;
  const int k = (int)we + (int)ww + 3 * ((int)wn + (int)wsn);
  return (sum - f) * idg[k];
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
  for (int t = tid; t < SM::W * SM::HH; t += NT) {
    const int lx = t % SM::W, ly = t / SM::W;
    const int a = x0 - H + lx, b = y0 - H + ly;
    const bool in = (px || (a >= 0 && a < n)) && (py || (b >= 0 && b < n));
    T xv = (T)0, fv = (T)0;
    if (in) {
      const int aa = wrapi(a, n), bb = wrapi(b, n);
      const long id = (long)bb * P + aa;
      if (!x_zero) xv = M.x[l][id];
      fv = level_f(M, l, id);
      if (mode == 1) {
        // bilinear cell-centred prolongation of the coarse correction
        const int nc = M.n[l + 1];
        const long Pc = M.pitch[l + 1];
        const int I = aa >> 1, J = bb >> 1;
        int I2 = I + ((aa & 1) ? 1 : -1), J2 = J + ((bb & 1) ? 1 : -1);
        I2 = px ? wrapi(I2, nc) : min(max(I2, 0), nc - 1);
        J2 = py ? wrapi(J2, nc) : min(max(J2, 0), nc - 1);
        const T* xc = M.x[l + 1];
        const T c00 = xc[(long)J * Pc + I], c10 = xc[(long)J * Pc + I2];
        const T c01 = xc[(long)J2 * Pc + I], c11 = xc[(long)J2 * Pc + I2];
        xv = xv + ((T)0.5625 * c00 + (T)0.1875 * (c10 + c01) + (T)0.0625 * c11);
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
      if (!px && (a < 0 || a >= n)) continue;
      if (!py && (b < 0 || b >= n)) continue;
      const int lx = a - (x0 - H), ly = b - (y0 - H);
      const bool we = px || a + 1 < n, ww = px || a > 0;
      const bool wn = py || b + 1 < n, wsn = py || b > 0;
      sm.x[ly][lx] = gs_update<T>(sm.x[ly][lx + 1], sm.x[ly][lx - 1], sm.x[ly + 1][lx], sm.x[ly - 1][lx],
                                  we, ww, wn, wsn, ihx, ihy, sm.f[ly][lx], M.idg[l]);
    }
    __syncthreads();
  }
  for (int t = tid; t < TX * TY; t += NT) {
    const int a = x0 + t % TX, b = y0 + t / TX;
    if (a < n && b < n) M.x[l][(long)b * P + a] = sm.x[b - (y0 - H)][a - (x0 - H)];
  }
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
  T s = (T)0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int a = 2 * I + (q & 1), b = 2 * J + (q >> 1);
    const long id = (long)b * P + a;
    const T xc = x[id];
    T lap = (T)0;
    if (px || a + 1 < n) lap += (x[(long)b * P + wrapi(a + 1, n)] - xc) * ihx;
    if (px || a > 0) lap += (x[(long)b * P + wrapi(a - 1, n)] - xc) * ihx;
    if (py || b + 1 < n) lap += (x[(long)wrapi(b + 1, n) * P + a] - xc) * ihy;
    if (py || b > 0) lap += (x[(long)wrapi(b - 1, n) * P + a] - xc) * ihy;
    s += level_f(M, l, id) - lap;
  }
  M.f[l + 1][(long)J * M.pitch[l + 1] + I] = (T)0.25 * s;
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
