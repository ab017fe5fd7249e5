// Float-float defect correction of the mixed-precision Poisson solve (2D).
//
// phi is carried as hi + lo float arrays during the solve; each sweep adds the
// FP32 V-cycle correction e and recomputes r = (f - mean f) - L phi in
// float-float arithmetic, so no FP64 instruction runs inside the loop. The
// FP64 phi is assembled once at the end (k_ff_to_double2d).
#pragma once
#include <type_traits>
#include "ff.cuh"
#include "ns_common.cuh"

namespace ns {

struct DCffArgs {
  int n;
  long pitch;
  int periodic[2];
  float ih[2][2];        // 1/h^2 per direction as float-float
  const float* phin[2];  // phi hi, lo (input)
  float* phout[2];       // phi hi, lo (output)
  const float* e;        // FP32 correction
  float* r32;            // FP32 residual
  const float* f[2];     // (f - mean f) hi, lo
  int first;             // phi = 0, no correction
  double* part;
  unsigned* counter;
  double* red_out;       // {max |r|}
};

// Tile of 32 x kDcTY cells per block of 256 threads (each thread updates
// kDcTY / 8 rows), with a one-cell halo of phi + e in shared memory. At
// 4096^2 tiles of 16, 32, 64 and 128 rows took 0.191, 0.166, 0.156 and
// 0.182 ms a launch; the fast path of interior tiles then 0.148 ms.
constexpr int kDcTY = 64;

static __global__ void __launch_bounds__(256) k_dc_update_ff2d(DCffArgs A) {
  __shared__ ff sp[kDcTY + 2][34];
  const int n = A.n;
  const long P = A.pitch;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * kDcTY;
  const bool px = A.periodic[0], py = A.periodic[1];
  const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
  const ff ihx = ff_make(A.ih[0][0], A.ih[0][1]), ihy = ff_make(A.ih[1][0], A.ih[1][1]);
  float v[1] = {0.f};
  // FAST: the tile and its halo lie inside the domain (no wrap, no wall);
  // the same operations, and the same bits
  auto body = [&](auto fast_c) {
  constexpr bool FAST = decltype(fast_c)::value;
  for (int ly = wy; ly < kDcTY + 2; ly += 8)
    for (int lx = lane; lx < 34; lx += 32) {
      int a = x0 - 1 + lx, b = y0 - 1 + ly;
      ff v = ff_make(0.f, 0.f);
      if (!A.first && (FAST || ((px || (a >= 0 && a < n)) && (py || (b >= 0 && b < n))))) {
        const long id = (long)(FAST ? b : wrapi(b, n)) * P + (FAST ? a : wrapi(a, n));
        v = ff_add_f(ff_make(A.phin[0][id], A.phin[1][id]), A.e[id]);
      }
      sp[ly][lx] = v;
    }
  __syncthreads();
#pragma unroll
  for (int rr = 0; rr < kDcTY / 8; ++rr) {
    const int a = x0 + lane, b = y0 + wy + 8 * rr;
    if (FAST || (a < n && b < n)) {
      const int lx = lane + 1, ly = wy + 8 * rr + 1;
      const ff c = sp[ly][lx];
      ff sx = ff_make(0.f, 0.f), sy = sx;
      if (FAST || px || a + 1 < n) sx = sx + (sp[ly][lx + 1] - c);
      if (FAST || px || a > 0) sx = sx + (sp[ly][lx - 1] - c);
      if (FAST || py || b + 1 < n) sy = sy + (sp[ly + 1][lx] - c);
      if (FAST || py || b > 0) sy = sy + (sp[ly - 1][lx] - c);
      const ff lap = sx * ihx + sy * ihy;
      const long id = (long)b * P + a;
      const ff r = ff_make(A.f[0][id], A.f[1][id]) - lap;
      A.phout[0][id] = c.hi;
      A.phout[1][id] = c.lo;
      const float r1 = r.hi + r.lo;
      A.r32[id] = r1;
      v[0] = fmaxf(v[0], fabsf(r1));
    }
  }
  };
  if (x0 >= 1 && x0 + 33 <= n && y0 >= 1 && y0 + kDcTY + 1 <= n) body(std::true_type{});
  else body(std::false_type{});
  double out[1];
  if (grid_reduce_last_f<1, 256>(v, reinterpret_cast<float2*>(A.part), A.counter, 1u, out) && threadIdx.x == 0)
    A.red_out[0] = out[0];
}

// (f - mean) -> float-float, integer split of both (no FP64 instruction)
// grid ((n + 255) / 256, n): thread a of block row b takes cell (a, b)
static __global__ void __launch_bounds__(256) k_rhs_ff2d(int n, long P, const double* f, const double* mean, float* fh,
                                                         float* fl) {
  const int a = blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
  if (a >= n) return;
  const ff m = ff_from_double(*mean);
  const long id = (long)b * P + a;
  const ff r = ff_from_double(f[id]) - m;
  fh[id] = r.hi;
  fl[id] = r.lo;
}

// phi (FP64) = hi + lo
static __global__ void __launch_bounds__(256) k_ff_to_double2d(int n, long P, const float* h, const float* l, double* out) {
  const int a = blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
  if (a >= n) return;
  const long id = (long)b * P + a;
  out[id] = (double)h[id] + (double)l[id];
}

}  // namespace ns
