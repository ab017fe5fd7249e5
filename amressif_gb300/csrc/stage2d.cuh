// Fused predictor stage of the dual-time BDF2 momentum solve (2D, FP64).
//
// One launch = one RK pseudo-stage of main.cpp:931-1017 for the whole grid:
// the tile of face velocities u* is staged in shared memory, the cell-centred
// velocity (cont2cart, utilities.cpp:16-350) and its wall/lid ghosts are
// rebuilt there, the QUICK half-node fluxes (fn_flux_calc.cpp:11-202), the
// viscous term (fn_flux_calc.cpp:695-766), the flux ghost rule
// (main.cpp:939-1014), the face RHS (fn_rhs.cpp:8-68) and the BDF2 stage
// update (momentum.cpp:68-88) are evaluated without touching HBM, and only
// the new u* is written. The fourth stage also reduces the pseudo-increment
// norm (utilities.cpp:421-493).
//
// MODE selects what is written:
//   kExactRK   reference operation order (use with -fmad=false): bit-exact
//              against the oracle.
//   kFastRK    same algebra with the step-constant source S = -grad p +
//              (0.5/dt) du^n + (1.5/dt) u^n and reciprocal multiplies.
//   kAnchor    stage 0 of the mixed-precision iteration: u_base = u_prev +
//              e4, and G0 = G(u_base) is written in FP32 with an FP32 copy of
//              u_base for the FP32 increment stages.
//   kExplicit  PSEUDO_TIMESTEPPING = 0 (momentum.cpp:96-192).
//
// Geom::conv_scheme selects the convective routine: QUICK as above; the
// cell term of convective_flux_calc_quick read from StageArgs::conv
// (conv_alt2d.cuh forms it); or none (convective_flux_calc leaves the total
// flux at the 0 of its setVal, so total = 0 - 0 + visc keeps the bits).
#pragma once
#include "ns_common.cuh"

namespace ns {

enum StageMode : int { kExactRK = 0, kFastRK = 1, kAnchor = 2, kExplicit = 3 };

struct StageArgs {
  Geom g;
  const double* us[2];    // u* entering the stage (velStar)
  const double* ub[2];    // u_base (velCont)
  const double* un[2];    // u^n (velContPrev)
  const double* du[2];    // du^n = u^n - u^{n-1} (velContDiff)
  const double* p;        // pressure, cells
  const double* S[2];     // step-constant source (fast / anchor)
  const double* cart[2];  // optional cell velocity override (first stage of a run), cells
  const float* e4[2];     // anchor: increment added to us to form u_base
  double* conv[2];        // conv_scheme 1: cell convective term, cells
  double* out[2];         // new u* (or u_base for the anchor)
  float* g0[2];           // anchor: G(u_base) in FP32
  float* shadow[2];       // anchor: FP32 copy of u_base
  double rk;              // rk[sub]
  int do_norm;
  double* part;           // 2 * nblocks partial sums
  unsigned* counter;
  double* norm_out;       // pseudo-increment norm (max over directions)
};

template <int TX, int TY>
struct StageSmem {
  static constexpr int CW = TX + 6, CH = TY + 6;   // cell velocity, origin (x0-3, y0-3)
  static constexpr int FXW = TX + 3, FXH = TY + 2; // x-face fluxes, origin (x0-1, y0-1)
  static constexpr int FYW = TX + 2, FYH = TY + 3; // y-face fluxes, origin (x0-1, y0-1)
  static constexpr int TW = TX + 2, TH = TY + 2;   // total flux, origin (x0-1, y0-1)
  double c[2][CH][CW];
  double fx[2][FXH][FXW];
  double fy[2][FYH][FYW];
  double t[2][TH][TW];
};

struct ArithExact {
  static __device__ __forceinline__ double div(double a, double d, double) { return a / d; }
};
struct ArithFast {
  static __device__ __forceinline__ double div(double a, double, double inv) { return a * inv; }
};

template <int MODE>
__device__ __forceinline__ double load_us(const StageArgs& A, int comp, long idx) {
  double v = A.us[comp][idx];
  if (MODE == kAnchor && A.e4[comp] != nullptr) v = v + (double)A.e4[comp][idx];
  return v;
}

// QUICK half-node flux of fn_flux_calc.cpp:71-76 with the operation order of
// the reference: a = q(i+1), b = q(i), c = q(i-1), e = q(i-2).
__device__ __forceinline__ double quick_flux(double ucon_face, double a, double b, double c, double e) {
  const double ucon = 0.5 * ucon_face;
  const double ud = ucon + fabs(ucon);
  const double up = ucon - fabs(ucon);
  return up * (0.125 * (-a - 2 * b + 3 * c) + b) + ud * (0.125 * (-e - 2 * c + 3 * b) + c);
}

template <class AR, int MODE, int TX, int TY>
__global__ void __launch_bounds__(256) k_stage2d(StageArgs A) {
  using SM = StageSmem<TX, TY>;
  __shared__ SM sm;
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int tid = threadIdx.x, NT = blockDim.x;
  const bool perx = g.periodic[0], pery = g.periodic[1];
  const double dx = g.dx[0], dy = g.dx[1];
  const double idx_ = g.inv_dx[0], idy_ = g.inv_dx[1];

  // ---- 1. cell-centred velocity of the tile + 3-cell halo -----------------
  for (int t = tid; t < SM::CW * SM::CH; t += NT) {
    const int lx = t % SM::CW, ly = t / SM::CW;
    const int a = x0 - 3 + lx, b = y0 - 3 + ly;
    const bool inx = (a >= 0 && a < N), iny = (b >= 0 && b < N);
    double cu = 0.0, cv = 0.0;
    if ((inx || perx) && (iny || pery)) {
      const int aa = wrapi(a, N), bb = wrapi(b, N);
      if (A.cart[0] != nullptr) {
        cu = A.cart[0][bb * P + aa];
        cv = A.cart[1][bb * P + aa];
      } else {
        cu = 0.5 * (load_us<MODE>(A, 0, bb * P + aa) + load_us<MODE>(A, 0, bb * P + aa + 1));
        cv = 0.5 * (load_us<MODE>(A, 1, bb * P + aa) + load_us<MODE>(A, 1, (bb + 1) * P + aa));
      }
    }
    sm.c[0][ly][lx] = cu;
    sm.c[1][ly][lx] = cv;
  }
  __syncthreads();
  // x ghosts first, then y ghosts (the later direction wins at corners)
  if (!perx) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int a = x0 - 3 + lx, b = y0 - 3 + ly;
      if (!(b >= 0 && b < N) && !pery) continue;
      if (a >= -3 && a < 0) {
        const int ml = (-a - 1) - (x0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost(g.bc[0], m, sm.c[m][ly][ml]);
      } else if (a >= N && a < N + 3) {
        const int ml = (2 * N - 1 - a) - (x0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost(g.bc[1], m, sm.c[m][ly][ml]);
      }
    }
    __syncthreads();
  }
  if (!pery) {
    for (int t = tid; t < SM::CW * SM::CH; t += NT) {
      const int lx = t % SM::CW, ly = t / SM::CW;
      const int b = y0 - 3 + ly;
      if (b >= -3 && b < 0) {
        const int ml = (-b - 1) - (y0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost(g.bc[2], m, sm.c[m][ml][lx]);
      } else if (b >= N && b < N + 3) {
        const int ml = (2 * N - 1 - b) - (y0 - 3);
        for (int m = 0; m < 2; ++m) sm.c[m][ly][lx] = cart_ghost_north(g, m, sm.c[m][ml][lx], x0 - 3 + lx);
      }
    }
    __syncthreads();
  }

  const bool wx = (g.flux_ghost[0] == kWrap), wy = (g.flux_ghost[1] == kWrap);

  // ---- 2. half-node fluxes ----------------------------------------------
  // x-faces a in [x0-1, x0+TX+1], rows b in [y0-1, y0+TY]
  if (g.conv_scheme == 0) {
  for (int t = tid; t < SM::FXW * SM::FXH; t += NT) {
    const int fx = t % SM::FXW, fyy = t / SM::FXW;
    const int a = x0 - 1 + fx, b = y0 - 1 + fyy;
    // u component: rows [y0, y0+TY), faces [x0-1, x0+TX+1]
    // v component: rows [y0-1, y0+TY], faces [x0, x0+TX]
    const bool rowin = (b >= 0 && b < N);
    const bool facein = (a >= 0 && a <= N);
    const bool need_u = (fyy >= 1 && fyy <= TY) && rowin && (facein || wx);
    const bool need_v = (fx >= 1 && fx <= TX + 1) && (rowin || wy) && (a >= 0 && a <= N);
    if (!need_u && !need_v) continue;
    const int aa = facein ? a : wrapi(a, N);
    const int bb = wrapi(b, N);
    const double ucf = load_us<MODE>(A, 0, (long)bb * P + aa);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    if (need_u)
      sm.fx[0][fyy][fx] = quick_flux(ucf, sm.c[0][ly][lx + 1], sm.c[0][ly][lx], sm.c[0][ly][lx - 1], sm.c[0][ly][lx - 2]);
    if (need_v)
      sm.fx[1][fyy][fx] = quick_flux(ucf, sm.c[1][ly][lx + 1], sm.c[1][ly][lx], sm.c[1][ly][lx - 1], sm.c[1][ly][lx - 2]);
  }
  // y-faces: cols a in [x0-1, x0+TX], faces b in [y0-1, y0+TY+1]
  for (int t = tid; t < SM::FYW * SM::FYH; t += NT) {
    const int fx = t % SM::FYW, fyy = t / SM::FYW;
    const int a = x0 - 1 + fx, b = y0 - 1 + fyy;
    const bool colin = (a >= 0 && a < N);
    const bool facein = (b >= 0 && b <= N);
    // u component: cols [x0-1, x0+TX], faces [y0, y0+TY]
    // v component: cols [x0, x0+TX), faces [y0-1, y0+TY+1]
    const bool need_u = (fyy >= 1 && fyy <= TY + 1) && (colin || wx) && (b >= 0 && b <= N);
    const bool need_v = (fx >= 1 && fx <= TX) && colin && (facein || wy);
    if (!need_u && !need_v) continue;
    const int aa = wrapi(a, N);
    const int bb = facein ? b : wrapi(b, N);
    const double vcf = load_us<MODE>(A, 1, (long)bb * P + aa);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
    if (need_u)
      sm.fy[0][fyy][fx] = quick_flux(vcf, sm.c[0][ly + 1][lx], sm.c[0][ly][lx], sm.c[0][ly - 1][lx], sm.c[0][ly - 2][lx]);
    if (need_v)
      sm.fy[1][fyy][fx] = quick_flux(vcf, sm.c[1][ly + 1][lx], sm.c[1][ly][lx], sm.c[1][ly - 1][lx], sm.c[1][ly - 2][lx]);
  }
  }
  __syncthreads();

  // ---- 3. total = -conv + visc at cells ----------------------------------
  const double dx2 = g.dx2[0], dy2 = g.dx2[1];
  const double idx2 = g.inv_dx2[0], idy2 = g.inv_dx2[1], iren = g.inv_ren;
  for (int t = tid; t < SM::TW * SM::TH; t += NT) {
    const int tx = t % SM::TW, ty = t / SM::TW;
    const int a = x0 - 1 + tx, b = y0 - 1 + ty;
    const bool need_u = (ty >= 1 && ty <= TY) && (b < N) && ((a >= 0 && a < N) || wx);
    const bool need_v = (tx >= 1 && tx <= TX) && (a < N) && ((b >= 0 && b < N) || wy);
    const int ly = b - (y0 - 3), lx = a - (x0 - 3);
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if (m == 0 ? !need_u : !need_v) continue;
      double conv = 0.0;
      if (g.conv_scheme == 0)
        conv = AR::div(sm.fx[m][ty][tx + 1] - sm.fx[m][ty][tx], dx, idx_) +
               AR::div(sm.fy[m][ty + 1][tx] - sm.fy[m][ty][tx], dy, idy_);
      else if (g.conv_scheme == 1)  // the wrapped cell in periodic directions: FillBoundary's copy
        conv = A.conv[m][(long)wrapi(b, N) * P + wrapi(a, N)];
      const double ce = sm.c[m][ly][lx];
      const double s = sm.c[m][ly - 1][lx], n = sm.c[m][ly + 1][lx];
      const double w = sm.c[m][ly][lx - 1], e = sm.c[m][ly][lx + 1];
      const double visc = AR::div(AR::div(e - 2 * ce + w, dx2, idx2) + AR::div(n - 2 * ce + s, dy2, idy2), g.ren, iren);
      double tot = 0.0 - conv;
      tot = tot + visc;
      sm.t[m][ty][tx] = tot;
    }
  }
  __syncthreads();
  // ghost totals of the normal component (reflection / zero)
  if (tid < 2 * (TY + TX)) {
    if (tid < TY) {
      const int ty = tid + 1;
      if (x0 == 0 && !wx) sm.t[0][ty][0] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][1] : 0.0;
    } else if (tid < 2 * TY) {
      const int ty = tid - TY + 1;
      const int tx = N - (x0 - 1);  // cell a = N
      if (tx >= 1 && tx < SM::TW && !wx)
        sm.t[0][ty][tx] = (g.flux_ghost[0] == kReflect) ? -sm.t[0][ty][tx - 1] : 0.0;
    } else if (tid < 2 * TY + TX) {
      const int tx = tid - 2 * TY + 1;
      if (y0 == 0 && !wy) sm.t[1][0][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][1][tx] : 0.0;
    } else {
      const int tx = tid - 2 * TY - TX + 1;
      const int ty = N - (y0 - 1);
      if (ty >= 1 && ty < SM::TH && !wy)
        sm.t[1][ty][tx] = (g.flux_ghost[1] == kReflect) ? -sm.t[1][ty - 1][tx] : 0.0;
    }
  }
  __syncthreads();

  // ---- 4. face RHS and stage update ----------------------------------------
  const double c15 = g.c15, c05 = g.c05, rk = A.rk;
  double nrm[2] = {0.0, 0.0};
  // u faces: a in [x0, x0+TX) (+ a = N on the last tile column), b in [y0, y0+TY)
  const int nfx = (x0 + TX >= N) ? (N - x0 + 1) : TX;
  const int nfy = (y0 + TY >= N) ? (N - y0 + 1) : TY;
  const int ncx = min(TX, N - x0), ncy = min(TY, N - y0);
  for (int t = tid; t < nfx * ncy + ncx * nfy; t += NT) {
    int m, a, b;
    if (t < nfx * ncy) { m = 0; a = x0 + t % nfx; b = y0 + t / nfx; }
    else { const int q = t - nfx * ncy; m = 1; a = x0 + q % ncx; b = y0 + q / ncx; }
    const long id = (long)b * P + a;
    const int tx = a - (x0 - 1), ty = b - (y0 - 1);
    double tm, tc;
    int face, nf;
    if (m == 0) { tm = sm.t[0][ty][tx - 1]; tc = sm.t[0][ty][tx]; face = a; nf = N; }
    else { tm = sm.t[1][ty - 1][tx]; tc = sm.t[1][ty][tx]; face = b; nf = N; }
    double out;
    if (MODE == kExactRK || MODE == kExplicit) {
      // gradient_calc_approach2 with mirrored / wrapped p ghosts
      int ca = a, cb = b, pa = a, pb = b;
      if (m == 0) pa = a - 1; else pb = b - 1;
      const int d = m;
      int cidx = (d == 0) ? ca : cb, pidx = (d == 0) ? pa : pb;
      if (cidx == nf) cidx = g.ctx_mirror[d] ? nf - 1 : 0;
      if (pidx < 0) pidx = g.ctx_mirror[d] ? 0 : nf - 1;
      const double pc = (d == 0) ? A.p[(long)cb * P + cidx] : A.p[(long)cidx * P + ca];
      const double pm = (d == 0) ? A.p[(long)cb * P + pidx] : A.p[(long)pidx * P + ca];
      const double gp = AR::div(pc - pm, g.dx[d], g.inv_dx[d]);
      double r = -gp + 0.5 * (tm + tc);
      if (MODE == kExactRK) {
        r = r - c15 * (A.us[m][id] - A.un[m][id]) + c05 * A.du[m][id];
        out = A.ub[m][id] + (rk * r);
      } else {
        r = r + g.c2dt * A.du[m][id];
        out = A.us[m][id] + (g.dt15 * r);
      }
      A.out[m][id] = out;
    } else if (MODE == kFastRK) {
      const double G = (A.S[m][id] - c15 * A.us[m][id]) + 0.5 * (tm + tc);
      out = A.ub[m][id] + rk * G;
      A.out[m][id] = out;
    } else {  // kAnchor
      const double ubase = load_us<MODE>(A, m, id);
      const double G = (A.S[m][id] - c15 * ubase) + 0.5 * (tm + tc);
      A.out[m][id] = ubase;
      A.g0[m][id] = (float)G;
      A.shadow[m][id] = (float)ubase;
      out = ubase;
    }
    if (A.do_norm) {
      const double w = (face == 0 || face == nf) ? 0.5 : 1.0;
      const double q = A.ub[m][id] - out;
      nrm[m] += fabs((q * q) * w);
    }
  }
  if (A.do_norm) {
    if (grid_reduce_last<2>(nrm, A.part, A.counter, 0u) && threadIdx.x == 0) {
      const double npts = (double)N * (double)N;
      const double ex = sqrt(nrm[0]) / sqrt(npts), ey = sqrt(nrm[1]) / sqrt(npts);
      *A.norm_out = max_keep_nan(ex, ey);
    }
  }
}

}  // namespace ns
