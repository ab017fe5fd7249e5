// Cell convective term of convective_flux_calc_quick (fn_flux_calc.cpp:204-393),
// the alternative routine that main_main does not call, on the one box of the
// 2D grid (FP64, the reference's operation order; instantiated in
// kernels_exact.cu, which is compiled with -fmad=false).
//
// One thread per cell writes conv_m(i, j) of both components into two cell
// arrays of pitch P; k_stage2d then forms total = 0 - conv + visc from them.
// As written, the routine computes:
//  - face values upwinded on the sign of u*, q_U + 0.0 * (QUICK correction):
//    the weight Real(1/8) is an integer division. The product is kept, since
//    it sets the sign of a zero result;
//  - faces over the cells only (face i is the west face of cell i); at the
//    last cell of the domain, face N takes face 0's value, along x and y;
//  - conv_u in conservative form (face velocity times face value), conv_v in
//    advective form (cell velocity times a face difference), both taking the
//    y differences at i+1 instead of j+1. The y-face fabs have no ghost cells,
//    so their element (i+1, j) at i = N-1 is (0, j+1) of the flat array.
#pragma once
#include "bounds.cuh"
#include "ns_common.cuh"
#include "stage2d.cuh"

namespace ns {

// Cell velocity of component m at (a, b), a and b in [-2, N+1], at most one
// of them outside [0, N): the periodic image, or the ghost rule of the side
// the index leaves by (utilities.cpp:62-349), applied to the mirrored cell.
__device__ __forceinline__ double alt_cell_vel(const StageArgs& A, int m, int a, int b) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  int aa = a, bb = b, side = -1;  // side: 0 xlo, 1 xhi, 2 ylo, 3 yhi
  if (a < 0 || a >= N) {
    if (g.periodic[0]) aa = wrapi(a, N);
    else { side = a < 0 ? 0 : 1; aa = a < 0 ? -a - 1 : 2 * N - 1 - a; }
  }
  if (b < 0 || b >= N) {
    if (g.periodic[1]) bb = wrapi(b, N);
    else { side = b < 0 ? 2 : 3; bb = b < 0 ? -b - 1 : 2 * N - 1 - b; }
  }
  const long id = (long)bb * P + aa;
  double q;
  if (A.cart[0] != nullptr) q = A.cart[m][id];
  else if (m == 0) q = 0.5 * (A.us[0][id] + A.us[0][id + 1]);
  else q = 0.5 * (A.us[1][id] + A.us[1][id + P]);
  if (side < 0) return q;
  if (side == 3) return cart_ghost_north(g, m, q, a);
  return cart_ghost(g.bc[side], m, q);
}

// Upwinded face value between the cells lo = (f-1) and hi = f along one
// direction: lo2, lo, hi, hi2 are the cells f-2 .. f+1.
__device__ __forceinline__ double alt_face(bool pos, double lo2, double lo, double hi, double hi2) {
  const double w = 0.0;  // Real(1/8)
  if (pos) return lo + w * (-lo2 - 2 * lo + 3 * hi);
  return hi + w * (3 * lo - 2 * hi - hi2);
}

// x-face value of component m at face f in [0, N] of row j (face N = face 0)
__device__ __forceinline__ double alt_xface(const StageArgs& A, int m, int f, int j) {
  if (f == A.g.N) f = 0;
  const bool pos = A.us[0][(long)j * A.g.pitch + f] > 0;
  return alt_face(pos, alt_cell_vel(A, m, f - 2, j), alt_cell_vel(A, m, f - 1, j), alt_cell_vel(A, m, f, j),
                  alt_cell_vel(A, m, f + 1, j));
}

// y-face value of component m at face f in [0, N] of column i (face N = face 0)
__device__ __forceinline__ double alt_yface(const StageArgs& A, int m, int i, int f) {
  if (f == A.g.N) f = 0;
  const bool pos = A.us[1][(long)f * A.g.pitch + i] > 0;
  return alt_face(pos, alt_cell_vel(A, m, i, f - 2), alt_cell_vel(A, m, i, f - 1), alt_cell_vel(A, m, i, f),
                  alt_cell_vel(A, m, i, f + 1));
}

// block 32 x 8 cells
__global__ void __launch_bounds__(256) k_conv_quick2d(StageArgs A) {
  const Geom& g = A.g;
  const int N = g.N;
  const long P = g.pitch;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= N || j >= N) return;
  // element (i+1, j) of a y-face fab (x extent N, N+1 rows)
  const int in = (i + 1 < N) ? i + 1 : 0, jn = (i + 1 < N) ? j : j + 1;
  const long id = (long)j * P + i, idn = (long)jn * P + in;
  if (!NS_BCHK(g.check, idn, P, N + 1, N - 1, 61)) return;
  const double u0 = A.us[0][id], u1 = A.us[0][id + 1];
  const double v0 = A.us[1][id], v1 = A.us[1][idn];
  const double dx = g.dx[0], dy = g.dx[1];
  {
    const double xa = alt_xface(A, 0, i, j), xb = alt_xface(A, 0, i + 1, j);
    const double ya = alt_yface(A, 0, i, j), yb = alt_yface(A, 0, in, jn);
    A.conv[0][id] = (u1 * xb - u0 * xa) / dx + (v1 * yb - v0 * ya) / dy;
  }
  {
    const double xa = alt_xface(A, 1, i, j), xb = alt_xface(A, 1, i + 1, j);
    const double ya = alt_yface(A, 1, i, j), yb = alt_yface(A, 1, in, jn);
    const double c0 = alt_cell_vel(A, 0, i, j), c1 = alt_cell_vel(A, 1, i, j);
    A.conv[1][id] = (c0 * (xb - xa)) / dx + (c1 * (yb - ya)) / dy;
  }
}

}  // namespace ns
