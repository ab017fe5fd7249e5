// Mixed-precision 3D predictor (NS_PREC_MIXED): each pseudo-iteration
// evaluates the BDF2 residual G at u_b, u_b + e1, u_b + e2, u_b + e3
// (main.cpp:945-1014). The anchor G0 = G(u_b) is computed in float-float
// arithmetic (ff.cuh, about 48 bits, on the FP32 pipes) by four passes that
// mirror the FP64 ones of ns3d.cuh: cell velocity with ghosts, QUICK fluxes,
// cell totals, face residual; it rounds G0 and u_b to FP32. The three other
// stages evaluate only the increment dG(u_b; e) = G(u_b + e) - G0 in FP32:
//   dF = (un+ - ub+) Q+(phi_b) + (un- - ub-) Q-(phi_b) + un Q_sign(un)(phi_e)
// for the QUICK flux F = u+ Q+(phi) + u- Q-(phi) (fn_flux_calc.cpp:66-76),
// with un = ub + e and the positive-part difference un+ - ub+ taken from the
// signs (e, -ub or max(un, 0)), so no term subtracts nearly equal FP32
// numbers; the viscous term, the ghost rules (homogeneous for the increment)
// and the flux-ghost rule of the faces are linear. Every FP32 rounding error
// is proportional to the increment, so the fixed point is the float-float
// one, within a few units of 1e-15 of the FP64 one. The last stage writes
// u_b + e4 and the pseudo-norm of e4 (the Error_Computation norm,
// utilities.cpp:421-493, reduced in float-float). Between pseudo-iterations
// u_b is carried as float-float pairs; it is read from the FP64 u^n in the
// first iteration and stored to FP64 once, when the iteration stops, so no
// pass but that store issues an FP64 arithmetic instruction (GB300 runs FP64
// at 1/73 of the FP32 rate).
#pragma once
#include "bounds.cuh"
#include "ff.cuh"
#include "ns3d.cuh"

namespace ns {

struct Inc3 {
  Geom g;
  const float* ub[3];      // FP32 copy of u_b (faces)
  const float* g0[3];      // G(u_b) rounded to FP32 (faces)
  const float* ein[3];     // stage input increment; nullptr: rk_prev * g0
  float* eout[3];          // stage output increment (not written by the last stage)
  const float* phb[3];     // ghosted FP32 cell velocity of u_b, (N+4)^3
  float* phe[3];           // ghosted cell velocity of the increment, (N+4)^3
  float* dfl[3][3];        // flux increments dfl[d][m] at the faces along d
  float* dt[3];            // cell total increments
  const double* base64[3]; // u_b in FP64 (last stage of the first iteration) ...
  const float2* baseff[3]; // ... or as float-float pairs (later iterations)
  float2* outff[3];        // u_b + e4 (last stage)
  float* ubout[3];         // u_b + e4 rounded to FP32 (last stage; nullptr: not written)
  float rk_prev, rk, c15;
  float inv_dx[3], vcoef[3];  // 1/dx, 1/(Re dx^2)
  int last;
  int keep_e;              // last stage: also store e4 in eout (the next incremental anchor reads it)
  double* part;
  unsigned* counter;
  double* norm_out;
};

// float-float anchor: values are (hi, lo) float pairs
struct AncFF {
  Geom g;
  const double* u[3];  // u_b in FP64 (first iteration) ...
  const float2* uff[3];  // ... or as float-float pairs (faces)
  const double* S[3];  // step source (faces)
  float2* ph[3];       // ghosted cell velocity, (N+4)^3
  float* ph32[3];      // the same rounded to FP32: the base cell velocity of the increments
  float2* fl[3][3];    // fluxes fl[d][m] at the faces along d
  float2* t[3];        // cell totals
  float* g0[3];        // G(u_b) rounded to FP32
  float* ub[3];        // u_b rounded to FP32
  float inv_dx[3][2], vcoef[3][2], c15[2];  // constants as (hi, lo)
};

// float-float defect correction of the mixed-precision 3D Poisson solve:
// phi is carried as (hi, lo) pairs; each sweep adds the FP32 V-cycle
// correction e and recomputes r = (f - mean f) - L phi (the 7-point operator
// of mg3_lap_terms) in float-float, with max |r| reduced on the FP32 pipes
struct DCff3 {
  int n;
  long pitch, plane;
  int periodic[3];
  float ih[3][2];      // 1/h^2 per direction as (hi, lo)
  const float2* phin;  // phi (input; ignored when first)
  float2* phout;       // phi + e (output)
  const float* e;      // FP32 correction (nullable)
  float* r32;          // FP32 residual: the right-hand side of the next V-cycle
  const float2* f;     // f - mean f
  int first;           // phi = 0
  double* part;
  unsigned* counter;
  double* red_out;     // max |r|
  // dc_residual = 1 (k3_dc64): phi and the residual in FP64
  const double* phin64;
  double* phout64;
  const double* f64;   // f; the kernel subtracts *fmean
  const double* fmean;
  double ih64[3];      // the FP64 level-0 1/h^2
};

#ifndef NS_3D_ARGS_ONLY

// Every input of these kernels is read-only for the launch (outputs go to other
// buffers), so loads use the non-coherent path: the compiler may then issue
// them ahead of the stores, which keeps many loads in flight per thread.
__device__ __forceinline__ float ldf(const float* p, long i) { return __ldg(p + i); }
__device__ __forceinline__ ff ld_ff(const double* p, long i) { return ff_from_double(__ldg(p + i)); }
__device__ __forceinline__ ff ld2(const float2* p, long i) {
  const float2 v = __ldg(p + i);
  return ff_make(v.x, v.y);
}
__device__ __forceinline__ void st2(float2* p, long i, ff v) { p[i] = make_float2(v.hi, v.lo); }
__device__ __forceinline__ ff ffc(const float (&c)[2]) { return ff_make(c[0], c[1]); }
__device__ __forceinline__ float ff_round(ff v) { return v.hi + v.lo; }
__device__ __forceinline__ ff ld_base(const AncFF& A, int m, long i) { return A.uff[m] ? ld2(A.uff[m], i) : ld_ff(A.u[m], i); }

// ---- float-float anchor ----------------------------------------------------------------
// ghosted cell velocity of u_b (the rules of k3_cart)
__global__ void __launch_bounds__(256) k3f_cart(AncFF A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(2, 2, 2)
  if (i > N + 1 || j > N + 1 || k > N + 1) return;
  const int c[3] = {i, j, k};
  int out_d = -1, nout = 0;
  for (int d = 0; d < 3; ++d)
    if (c[d] < 0 || c[d] >= N) { out_d = d; ++nout; }
  int cm[3] = {i, j, k};
  int side = 0;
  if (nout == 1) {
    const int d = out_d;
    side = c[d] < 0 ? 0 : 1;
    cm[d] = g.periodic[d] ? wrapi(c[d], N) : (c[d] < 0 ? -c[d] - 1 : 2 * N - 1 - c[d]);
  }
  const bool mirror = nout == 1 && !g.periodic[out_d];
  const long gi = gid3(N, i, j, k);
  for (int m = 0; m < 3; ++m) {
    ff v = ff_make(0.f, 0.f);
    if (nout <= 1) {
      const long a = id3(g, cm[0], cm[1], cm[2]);
      const long b = a + (m == 0 ? 1 : (m == 1 ? g.pitch : g.plane));
      v = ff_scale2(ld_base(A, m, a) + ld_base(A, m, b), 0.5f);
      if (mirror) {
        const CartBC& bc = g.bc[2 * out_d + side];
        const int r = bc.rule[m];
        if (r == kInlet) v = ff_from_double(bc.add[m]) - v;
        else if (r == kNeg) v = -v;
      }
    }
    if (A.ph[m] != nullptr) st2(A.ph[m], gi, v);
    A.ph32[m][gi] = ff_round(v);
  }
}



// u > 0: 3/4 x(-1) + 3/8 x(0) - 1/8 x(-2); u <= 0: 3/8 x(-1) + 3/4 x(0) - 1/8 x(+1)
__device__ __forceinline__ ff q3p_ff(ff x2, ff x1, ff x0) { return (0.75f * x1 + 0.375f * x0) + ff_scale2(x2, -0.125f); }
__device__ __forceinline__ ff q3m_ff(ff x1, ff x0, ff xa) { return (0.375f * x1 + 0.75f * x0) + ff_scale2(xa, -0.125f); }

// QUICK fluxes of the three components at every face along the three
// directions, each face once (the faces of k3_flux)
__global__ void __launch_bounds__(256) k3f_flux(AncFF A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  if (i > N || j > N || k > N) return;
  const long G1[3] = {1, N + 4, (long)(N + 4) * (N + 4)};
  const long gc = gid3(N, i, j, k);
  const long fc = id3(g, i, j, k);
  const int c[3] = {i, j, k};
  // every face thread loads all its stencils (indices stay inside the ghosted
  // array), selects the upwind one and stores only the faces that exist, so
  // the loads of the three directions are independent of any branch
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const bool ok = (d == 0 || c[0] < N) && (d == 1 || c[1] < N) && (d == 2 || c[2] < N);
    const long s = G1[d];
    const ff ud = ld_base(A, d, fc);
    const bool pos = ud.hi > 0.f;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const float2* ph = A.ph[m];
      const ff x2 = ld2(ph, gc - 2 * s), x1 = ld2(ph, gc - s), x0 = ld2(ph, gc), xa = ld2(ph, gc + s);
      const ff q = pos ? q3p_ff(x2, x1, x0) : q3m_ff(x1, x0, xa);
      const ff F = ud.hi != 0.f ? ud * q : ff_make(0.f, 0.f);
      if (ok) st2(A.fl[d][m], fc, F);
    }
  }
}

// t_m = nu lap(phi_m) - div F_m at the cells
__global__ void __launch_bounds__(256) k3f_total(AncFF A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  if (i >= N || j >= N || k >= N) return;
  const long G1[3] = {1, N + 4, (long)(N + 4) * (N + 4)};
  const long gc = gid3(N, i, j, k);
  const long fc = id3(g, i, j, k);
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const float2* ph = A.ph[m];
    const ff p2 = ff_scale2(ld2(ph, gc), 2.f);
    ff acc = ff_make(0.f, 0.f);
    for (int d = 0; d < 3; ++d) {
      const long s = G1[d];
      const float2* F = A.fl[d][m];
      const ff lap = (ld2(ph, gc + s) + ld2(ph, gc - s)) - p2;
      acc = acc + (ffc(A.vcoef[d]) * lap - ffc(A.inv_dx[d]) * (ld2(F, fc + fstride[d]) - ld2(F, fc)));
    }
    st2(A.t[m], fc, acc);
  }
}

__device__ __forceinline__ ff t_along_ff(const AncFF& A, int m, int a, long base, long st) {
  const int N = A.g.N;
  if (a >= 0 && a < N) return ld2(A.t[m], base + a * st);
  const int fg = A.g.flux_ghost[m];
  if (fg == kWrap) return ld2(A.t[m], base + (long)wrapi(a, N) * st);
  if (fg == kZero) return ff_make(0.f, 0.f);
  const int am = a < 0 ? 0 : N - 1;
  return -ld2(A.t[m], base + (long)am * st);
}

// G0 = S - (1.5/dt) u_b + avg(t) with the flux-ghost rule (k3_face with
// u = u_b), rounded to FP32 together with u_b
__global__ void __launch_bounds__(256) k3f_face(AncFF A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int m = 0; m < 3; ++m) {
    const int lim[3] = {N + (m == 0), N + (m == 1), N + (m == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    const int c[3] = {i, j, k};
    const int a = c[m];
    const long id = id3(g, i, j, k);
    const long st = fstride[m];
    const long base = id - (long)a * st;
    const ff tl = t_along_ff(A, m, a - 1, base, st), tr = t_along_ff(A, m, a, base, st);
    const ff u = ld_base(A, m, id);
    const ff G = (ld_ff(A.S[m], id) - ffc(A.c15) * u) + ff_scale2(tl + tr, 0.5f);
    A.g0[m][id] = ff_round(G);
    A.ub[m][id] = ff_round(u);
  }
}

// ---- FP32 increment stages ----------------------------------------------------------------
__device__ __forceinline__ float inc_e(const Inc3& A, int m, long id) {
  return A.ein[m] ? ldf(A.ein[m], id) : A.rk_prev * ldf(A.g0[m], id);
}

// ghosted cell velocity of the increment (homogeneous ghosts); cells with
// more than one index outside [0, N) are 0
__global__ void __launch_bounds__(256) k3i_cart(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  NS3_IJK(2, 2, 2)
  if (i > N + 1 || j > N + 1 || k > N + 1) return;
  const int c[3] = {i, j, k};
  int out_d = -1, nout = 0;
  for (int d = 0; d < 3; ++d)
    if (c[d] < 0 || c[d] >= N) { out_d = d; ++nout; }
  int cm[3] = {i, j, k};
  int side = 0;
  if (nout == 1) {
    const int d = out_d;
    side = c[d] < 0 ? 0 : 1;
    cm[d] = g.periodic[d] ? wrapi(c[d], N) : (c[d] < 0 ? -c[d] - 1 : 2 * N - 1 - c[d]);
  }
  const bool mirror = nout == 1 && !g.periodic[out_d];
  const long gi = gid3(N, i, j, k);
  for (int m = 0; m < 3; ++m) {
    float ve = 0.f;
    if (nout <= 1) {
      const long a = id3(g, cm[0], cm[1], cm[2]);
      const long b = a + (m == 0 ? 1 : (m == 1 ? g.pitch : g.plane));
      ve = 0.5f * (inc_e(A, m, a) + inc_e(A, m, b));
      if (mirror) ve = cart_ghost_f(g.bc[2 * out_d + side], m, ve, true);
    }
    A.phe[m][gi] = ve;
  }
}

// QUICK interpolants: u > 0 from cells -2, -1, 0; u <= 0 from cells -1, 0, +1
__device__ __forceinline__ float q3p(float x2, float x1, float x0) { return -0.125f * x2 + 0.75f * x1 + 0.375f * x0; }
__device__ __forceinline__ float q3m(float x1, float x0, float xa) { return 0.375f * x1 + 0.75f * x0 - 0.125f * xa; }

// Flux increments and cell totals in one pass (dt_m = nu lap(phi_e,m) -
// div dF_m): the QUICK flux increments of the three components at every face
// along the three directions, then the cell totals, without the nine
// face-flux arrays between two passes (36 B/cell of stores and more of loads). A block owns a 32 x 8 tile of
// cells and climbs kFtKZ planes of it. Per plane it stages the ghosted cell
// velocities of the tile and a halo (x: -2..+33, y: -2..+9) in shared memory,
// forms the x and y face fluxes of the tile (33 x 8 and 32 x 9 faces) there,
// and each thread carries its column's z window (cells k-1 .. k+2) and its
// bottom z-face flux in registers, so every face flux is formed once.
constexpr int kFtKZ = 16;
struct FtSmem {
  float pb[3][12][36];  // phi_b (ghosted cell velocity of u_b), plane k, tile + halo
  float pe[3][12][36];  // phi_e (of the increment)
  float fx[3][8][33];   // x-face flux increments of the tile's rows
  float fy[3][9][32];   // y-face flux increments of the tile's columns
};

__device__ __forceinline__ float flux_inc(float ub, float e, float b2, float b1, float b0, float ba, float e2, float e1,
                                          float e0, float ea) {
  const float un = ub + e;
  const float dpos = fmaxf(e, -ub) + fminf(ub, 0.f);  // un+ - ub+ (quick_sign2 of stage_inc2d.cuh)
  const float dneg = e - dpos;                                            // un- - ub-
  const float qe = un > 0.f ? q3p(e2, e1, e0) : q3m(e1, e0, ea);
  return dpos * q3p(b2, b1, b0) + dneg * q3m(b1, b0, ba) + un * qe;
}

__global__ void __launch_bounds__(256) k3i_fluxtot(Inc3 A) {
  __shared__ FtSmem sm;
  const Geom& g = A.g;
  const int N = g.N;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 8, k0 = blockIdx.z * kFtKZ;
  const int k1 = min(k0 + kFtKZ, N);
  const int i = i0 + tx, j = j0 + ty;
  const bool cell = i < N && j < N;
  const long G1 = 1, G2 = N + 4, G3 = (long)(N + 4) * (N + 4);
  // the column's z window: zb[m][q] / ze[m][q] = phi at plane k - 1 + q
  float zb[3][4], ze[3][4], fzb[3];
  // bounds-check build: the ghosted arrays are (N + 4)^3, rows of N + 4; the
  // face arrays (N + 1) planes of N + 1 rows of pitch P
  const long GR = (long)(N + 4) * (N + 4), FR = (long)(N + 1) * (N + 1);
  auto zload = [&](int m, int kk, float& b, float& e) {
    const long gi = gid3(N, i, j, kk);
    if (!NS_BCHK(g.check, gi, N + 4, GR, N + 3, 71)) { b = e = 0.f; return; }
    b = ldf(A.phb[m], gi);
    e = ldf(A.phe[m], gi);
  };
  if (cell) {
    // the bottom z-face flux of the chunk's first plane (cells k0-2 .. k0+1)
    float b2[3], e2[3];
    for (int m = 0; m < 3; ++m) {
      zload(m, k0 - 2, b2[m], e2[m]);
      for (int q = 0; q < 3; ++q) zload(m, k0 - 1 + q, zb[m][q], ze[m][q]);
    }
    const long fz = id3(g, i, j, k0);
    const float ubz = ldf(A.ub[2], fz), ez = inc_e(A, 2, fz);
    for (int m = 0; m < 3; ++m)
      fzb[m] = flux_inc(ubz, ez, b2[m], zb[m][0], zb[m][1], zb[m][2], e2[m], ze[m][0], ze[m][1], ze[m][2]);
  }
  for (int k = k0; k < k1; ++k) {
    __syncthreads();  // the previous plane's shared values are consumed
    for (int t = threadIdx.x; t < 12 * 36; t += 256) {
      const int sx = t % 36, sy = t / 36;
      const int a = i0 - 2 + sx, b = j0 - 2 + sy;
      const bool in = a <= N + 1 && b <= N + 1 &&  // the ghosted array spans -2 .. N + 1
                      NS_BCHK(g.check, gid3(N, a, b, k), N + 4, GR, N + 3, 72);
      const long gi = in ? gid3(N, a, b, k) : 0;
      for (int m = 0; m < 3; ++m) {
        sm.pb[m][sy][sx] = in ? ldf(A.phb[m], gi) : 0.f;
        sm.pe[m][sy][sx] = in ? ldf(A.phe[m], gi) : 0.f;
      }
    }
    if (cell)
      for (int m = 0; m < 3; ++m) zload(m, k + 2, zb[m][3], ze[m][3]);
    __syncthreads();
    // x faces (i0 .. i0 + 32) x rows (j0 .. j0 + 7)
    for (int t = threadIdx.x; t < 33 * 8; t += 256) {
      const int ii = t % 33, jj = t / 33;
      const int a = i0 + ii, b = j0 + jj;
      if (a > N || b >= N) continue;
      const long fc = id3(g, a, b, k);
      if (!NS_BCHK(g.check, fc, g.pitch, FR, N, 73)) continue;
      const float ub = ldf(A.ub[0], fc), e = inc_e(A, 0, fc);
      const int sx = ii + 2, sy = jj + 2;
      for (int m = 0; m < 3; ++m) {
        const float(*pb)[36] = sm.pb[m];
        const float(*pe)[36] = sm.pe[m];
        sm.fx[m][jj][ii] = flux_inc(ub, e, pb[sy][sx - 2], pb[sy][sx - 1], pb[sy][sx], pb[sy][sx + 1], pe[sy][sx - 2],
                                    pe[sy][sx - 1], pe[sy][sx], pe[sy][sx + 1]);
      }
    }
    // y faces (j0 .. j0 + 8) x columns (i0 .. i0 + 31)
    for (int t = threadIdx.x; t < 32 * 9; t += 256) {
      const int ii = t % 32, jj = t / 32;
      const int a = i0 + ii, b = j0 + jj;
      if (a >= N || b > N) continue;
      const long fc = id3(g, a, b, k);
      if (!NS_BCHK(g.check, fc, g.pitch, FR, N, 73)) continue;
      const float ub = ldf(A.ub[1], fc), e = inc_e(A, 1, fc);
      const int sx = ii + 2, sy = jj + 2;
      for (int m = 0; m < 3; ++m) {
        const float(*pb)[36] = sm.pb[m];
        const float(*pe)[36] = sm.pe[m];
        sm.fy[m][jj][ii] = flux_inc(ub, e, pb[sy - 2][sx], pb[sy - 1][sx], pb[sy][sx], pb[sy + 1][sx], pe[sy - 2][sx],
                                    pe[sy - 1][sx], pe[sy][sx], pe[sy + 1][sx]);
      }
    }
    __syncthreads();
    if (cell) {
      // the top z-face flux (cells k-1 .. k+2) and the totals of cell (i, j, k)
      const long fz = id3(g, i, j, k + 1);
      const float ubz = ldf(A.ub[2], fz), ez = inc_e(A, 2, fz);
      const long fc = id3(g, i, j, k);
      const int sx = tx + 2, sy = ty + 2;
      for (int m = 0; m < 3; ++m) {
        const float fzt =
            flux_inc(ubz, ez, zb[m][0], zb[m][1], zb[m][2], zb[m][3], ze[m][0], ze[m][1], ze[m][2], ze[m][3]);
        const float(*pe)[36] = sm.pe[m];
        const float p0 = pe[sy][sx];
        float conv = 0.f, visc = 0.f;
        conv += (sm.fx[m][ty][tx + 1] - sm.fx[m][ty][tx]) * A.inv_dx[0];
        visc += (pe[sy][sx + 1] - 2.f * p0 + pe[sy][sx - 1]) * A.vcoef[0];
        conv += (sm.fy[m][ty + 1][tx] - sm.fy[m][ty][tx]) * A.inv_dx[1];
        visc += (pe[sy + 1][sx] - 2.f * p0 + pe[sy - 1][sx]) * A.vcoef[1];
        conv += (fzt - fzb[m]) * A.inv_dx[2];
        visc += (ze[m][2] - 2.f * p0 + ze[m][0]) * A.vcoef[2];
        A.dt[m][fc] = visc - conv;
        fzb[m] = fzt;
      }
      for (int m = 0; m < 3; ++m)
        for (int q = 0; q < 3; ++q) {
          zb[m][q] = zb[m][q + 1];
          ze[m][q] = ze[m][q + 1];
        }
    }
  }
  (void)G1;
  (void)G2;
  (void)G3;
  (void)GR;  // read by NS_BCHK in the bounds-check build only
  (void)FR;
}

__device__ __forceinline__ float t_along_inc(const Inc3& A, int m, int a, long base, long st) {
  const int N = A.g.N;
  if (a >= 0 && a < N) return ldf(A.dt[m], base + a * st);
  const int fg = A.g.flux_ghost[m];
  if (fg == kWrap) return ldf(A.dt[m], base + (long)wrapi(a, N) * st);
  if (fg == kZero) return 0.f;
  const int am = a < 0 ? 0 : N - 1;
  return -ldf(A.dt[m], base + (long)am * st);
}

// e_out = rk (G0 - (1.5/dt) e_in + avg(dt)); the last stage writes
// u_b + e_out (float-float) and the pseudo-norm of e_out. Each block walks
// kIncFaceKZ planes, so the reducing launch has few blocks (one partial and
// one counter update per block).
constexpr int kIncFaceKZ = 8;

__global__ void __launch_bounds__(256) k3i_face(Inc3 A) {
  const Geom& g = A.g;
  const int N = g.N;
  const int i = (int)(blockIdx.x * 32 + (threadIdx.x & 31));
  const int j = (int)(blockIdx.y * 8 + (threadIdx.x >> 5));
  float nrm[3] = {0.f, 0.f, 0.f};
  const long fstride[3] = {1, g.pitch, g.plane};
  for (int kk = 0; kk < kIncFaceKZ; ++kk) {
    const int k = (int)blockIdx.z * kIncFaceKZ + kk;
    if (k > N) break;
    for (int m = 0; m < 3; ++m) {
      const int lim[3] = {N + (m == 0), N + (m == 1), N + (m == 2)};
      if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
      const int c[3] = {i, j, k};
      const int a = c[m];
      const long id = id3(g, i, j, k);
      const long st = fstride[m];
      const long base = id - (long)a * st;
      const float tl = t_along_inc(A, m, a - 1, base, st), tr = t_along_inc(A, m, a, base, st);
      const float G = (ldf(A.g0[m], id) - A.c15 * inc_e(A, m, id)) + 0.5f * (tl + tr);
      const float eo = A.rk * G;
      if (A.last) {
        const ff b = A.baseff[m] ? ld2(A.baseff[m], id) : ld_ff(A.base64[m], id);
        const ff nb = ff_add_f(b, eo);
        st2(A.outff[m], id, nb);
        if (A.ubout[m] != nullptr) A.ubout[m][id] = ff_round(nb);
        if (A.keep_e) A.eout[m][id] = eo;
        const float w = (a == 0 || a == N) ? 0.5f : 1.f;
        nrm[m] += eo * eo * w;
      } else {
        A.eout[m][id] = eo;
      }
    }
  }
  double tot[3];
  if (A.last && grid_reduce_last_f<3, 256>(nrm, reinterpret_cast<float2*>(A.part), A.counter, 0u, tot) &&
      threadIdx.x == 0) {
    const double npts = (double)N * N * N;
    double e = 0.0;
    for (int m = 0; m < 3; ++m) e = max_keep_nan(e, sqrt(tot[m]) / sqrt(npts));
    *A.norm_out = e;
  }
}

// ---- float-float defect correction (Poisson) ------------------------------------------------
__device__ __forceinline__ ff dc3_val(const DCff3& A, long id) {
  if (A.first) return ff_make(0.f, 0.f);
  const ff v = ld2(A.phin, id);
  return A.e ? ff_add_f(v, ldf(A.e, id)) : v;
}

__global__ void __launch_bounds__(256) k3_dcff(DCff3 A) {
  const int n = A.n;
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  float v[1] = {0.f};
  if (i < n && j < n && k < n) {
    const long id = (long)k * A.plane + (long)j * A.pitch + i;
    const int c[3] = {i, j, k};
    const long st[3] = {1, A.pitch, A.plane};
    const ff xc = dc3_val(A, id);
    ff lap = ff_make(0.f, 0.f);
    for (int d = 0; d < 3; ++d) {
      ff s = ff_make(0.f, 0.f);
      if (A.periodic[d] || c[d] + 1 < n) s = s + (dc3_val(A, id + ((c[d] + 1 < n) ? st[d] : -(long)(n - 1) * st[d])) - xc);
      if (A.periodic[d] || c[d] > 0) s = s + (dc3_val(A, id + ((c[d] > 0) ? -st[d] : (long)(n - 1) * st[d])) - xc);
      lap = lap + ffc(A.ih[d]) * s;
    }
    const ff r = ld2(A.f, id) - lap;
    st2(A.phout, id, xc);
    const float r1 = ff_round(r);
    A.r32[id] = r1;
    v[0] = fabsf(r1);
  }
  double out[1];
  if (grid_reduce_last_f<1, 256>(v, reinterpret_cast<float2*>(A.part), A.counter, 1u, out) && threadIdx.x == 0)
    A.red_out[0] = out[0];
}

// ---- FP64 defect correction (dc_residual = 1) ---------------------------------------------
// phi_out = phi_in + e (FP64 + FP32), r = (f - mean f) - L phi_out in FP64,
// r32 = float(r), max |r|: the same sweep as k3_dcff with an FP64 phi
__device__ __forceinline__ double dc64_val(const DCff3& A, long id) {
  if (A.first) return 0.0;
  const double v = __ldg(A.phin64 + id);
  return A.e ? v + (double)ldf(A.e, id) : v;
}

__global__ void __launch_bounds__(256) k3_dc64(DCff3 A) {
  const int n = A.n;
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  float v[1] = {0.f};
  if (i < n && j < n && k < n) {
    const long id = (long)k * A.plane + (long)j * A.pitch + i;
    const int c[3] = {i, j, k};
    const long st[3] = {1, A.pitch, A.plane};
    const double xc = dc64_val(A, id);
    double lap = 0.0;
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      if (A.periodic[d] || c[d] + 1 < n) s += dc64_val(A, id + ((c[d] + 1 < n) ? st[d] : -(long)(n - 1) * st[d])) - xc;
      if (A.periodic[d] || c[d] > 0) s += dc64_val(A, id + ((c[d] > 0) ? -st[d] : (long)(n - 1) * st[d])) - xc;
      lap += A.ih64[d] * s;
    }
    const double r = (__ldg(A.f64 + id) - *A.fmean) - lap;
    A.phout64[id] = xc;
    const float r1 = (float)r;
    A.r32[id] = r1;
    v[0] = fabsf(r1);
  }
  double out[1];
  if (grid_reduce_last_f<1, 256>(v, reinterpret_cast<float2*>(A.part), A.counter, 1u, out) && threadIdx.x == 0)
    A.red_out[0] = out[0];
}

// f - mean f as (hi, lo) pairs (integer split, no FP64 instruction)
__global__ void __launch_bounds__(256) k3_rhs_ff(int n, long pitch, long plane, const double* f, const double* mean,
                                                 float2* out) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= n || j >= n || k >= n) return;
  const long id = (long)k * plane + (long)j * pitch + i;
  st2(out, id, ld_ff(f, id) - ff_from_double(*mean));
}

// phi (FP64) = hi + lo
__global__ void __launch_bounds__(256) k3_ff_cells(int n, long pitch, long plane, const float2* in, double* out) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5), k = blockIdx.z;
  if (i >= n || j >= n || k >= n) return;
  const long id = (long)k * plane + (long)j * pitch + i;
  const float2 v = in[id];
  out[id] = (double)v.x + (double)v.y;
}

// u* = hi + lo in FP64 on every face, once the pseudo-iterations stop
__global__ void __launch_bounds__(256) k3f_store(Geom g, const float2* in0, const float2* in1, const float2* in2,
                                                 double* o0, double* o1, double* o2) {
  const int N = g.N;
  NS3_IJK(0, 0, 0)
  const float2* in[3] = {in0, in1, in2};
  double* out[3] = {o0, o1, o2};
  for (int m = 0; m < 3; ++m) {
    const int lim[3] = {N + (m == 0), N + (m == 1), N + (m == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    const long id = id3(g, i, j, k);
    const float2 v = in[m][id];
    out[m][id] = (double)v.x + (double)v.y;
  }
}

#endif  // NS_3D_ARGS_ONLY

}  // namespace ns
