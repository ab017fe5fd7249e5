// Shared definitions of the GB300 fractional-step kernels (2D MAC grid).
//
// Layout in HBM: every level-0 field is a dense row-major array with one row
// pitch `pitch` (elements, a multiple of 32 so that rows start on 256-byte
// boundaries). x-face velocity u(i,j): i in [0,N], j in [0,N); y-face
// velocity v(i,j): i in [0,N), j in [0,N]; cell fields (p, phi, f): [0,N)^2.
// Element (i,j) lives at j*pitch + i. No ghost cells are stored: boundary
// rules are applied while a tile is staged in shared memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns {

// max of two pseudo-norm components that keeps a NaN (fmax drops it), so a
// non-finite field shows in the norm the host reads; equal to fmax otherwise
__device__ __forceinline__ double max_keep_nan(double a, double b) { return (a != a) ? a : ((b != b) ? b : fmax(a, b)); }


// Ghost rule of the cell-centred velocity on one domain side for one
// component (utilities.cpp:62-349): ghost = -q, +q, or add - q (inlets), with
// q the mirror cell value.
enum CartRule : int { kNeg = 0, kPos = 1, kInlet = 2 };

// Ghost rule of the cell-centred total flux across a domain side.
enum FluxGhost : int { kReflect = 0, kWrap = 1, kZero = 2 };

struct CartBC {
  int rule[3];
  double add[3];
};

struct Geom {
  int N;          // cells per side
  int dim;        // 2 (3D kernels use the same struct)
  long pitch;     // row pitch of level-0 arrays (elements)
  long plane;     // plane stride (3D); pitch * (N+1)
  double dx[3];
  double dt, ren;
  // host-computed constants (the same doubles the reference forms inline)
  double inv_dx[3];   // 1/dx
  double dx2[3];      // dx*dx
  double inv_dx2[3];  // 1/(dx*dx)
  double inv_ren;     // 1/ren
  double c15;         // 1.5/dt
  double c05;         // 0.5/dt
  double c2dt;        // 1/(2 dt)
  double dt15;        // dt/1.5
  int periodic[3];
  int flux_ghost[3];  // per direction: kReflect (quirk Q1), kWrap, kZero
  int ctx_mirror[3];  // 1: p/phi ghosts mirrored (quirk Q2), 0: periodic wrap
  int conv_scheme;    // NS_CONV_*: 0 QUICK, 1 convective_flux_calc_quick (CONV arrays), 2 no convective term
  CartBC bc[6];       // xlo, xhi, ylo, yhi, zlo, zhi
  // optional lid profile of the north inlet (u component, one value per cell
  // column, device memory): the ghost becomes 2*lid_u[i] - q instead of
  // 2*inflow_waveform[0] - q (the controlled lid of the adjoint problem)
  const double* lid_u;
  // bounds-check build only: the context's status words (failures, first
  // failing index, its site); null otherwise
  unsigned long long* check;
};

// periodic index in [0, n) for any a (tiles of small grids reach past one period)
__host__ __device__ __forceinline__ int wrapi(int a, int n) {
  if (a >= 0 && a < n) return a;
  const int r = a % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ double cart_ghost(const CartBC& b, int m, double q) {
  const int r = b.rule[m];
  return r == kInlet ? b.add[m] - q : (r == kNeg ? -q : q);
}

// north ghost of column a: the lid profile replaces the uniform inlet value
__device__ __forceinline__ double cart_ghost_north(const Geom& g, int m, double q, int a) {
  if (m == 0 && g.lid_u != nullptr && g.bc[3].rule[0] == kInlet) {
    const int aa = a < 0 ? 0 : (a >= g.N ? g.N - 1 : a);
    return 2 * g.lid_u[aa] - q;
  }
  return cart_ghost(g.bc[3], m, q);
}

__device__ __forceinline__ float cart_ghost_f(const CartBC& b, int m, float q, bool homogeneous) {
  const int r = b.rule[m];
  if (r == kInlet) return homogeneous ? -q : (float)b.add[m] - q;
  return r == kNeg ? -q : q;
}

// Deterministic grid reduction: every block writes its partials, the last
// block to finish reduces them in block order.
// max_mask: bit q set => entry q is reduced with max, else with +.
template <int NV>
__device__ __forceinline__ bool grid_reduce_last(double (&v)[NV], double* part, unsigned* counter, unsigned max_mask) {
  __shared__ double red[NV][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const bool is_max = (max_mask >> q) & 1u;
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) {
      double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[q][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    for (int q = 0; q < NV; ++q) {
      const bool is_max = (max_mask >> q) & 1u;
      double x = red[q][0];
      for (int w = 1; w < nwarps; ++w) x = is_max ? fmax(x, red[q][w]) : x + red[q][w];
      part[(long)q * nb + bid] = x;
    }
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    last = (done == (unsigned)(nb - 1));
  }
  __syncthreads();
  if (!last) return false;
  // The whole last block reduces the partials: thread t takes blocks
  // t, t+blockDim, ... in order, then a fixed shuffle/shared-memory tree.
  // The partials are read from L2 (__ldcg: other blocks' fenced stores are
  // visible there) eight at a time, so the loads overlap; they are combined
  // in the same order as one at a time.
  __threadfence();
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  const int stride = blockDim.x;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const bool is_max = (max_mask >> q) & 1u;
    const double* pv = part + (long)q * nb;
    double x = 0.0;
    bool first = true;
    int b = threadIdx.x;
    for (; b + 7 * stride < nb; b += 8 * stride) {
      double y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = __ldcg(pv + b + u * stride);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        x = first ? y[u] : (is_max ? fmax(x, y[u]) : x + y[u]);
        first = false;
      }
    }
    for (; b < nb; b += stride) {
      const double y = __ldcg(pv + b);
      x = first ? y : (is_max ? fmax(x, y) : x + y);
      first = false;
    }
    for (int o = 16; o > 0; o >>= 1) {
      double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max ? fmax(x, y) : x + y;
    }
    __syncthreads();
    if (lane == 0) red[q][warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = red[q][0];
      for (int w = 1; w < nwarps; ++w) s = is_max ? fmax(s, red[q][w]) : s + red[q][w];
      v[q] = s;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// Flattened walk over a W x H rectangle by all NT threads of the block
// (W, H compile-time, so the division is a multiply-shift).
#define NS_RECT_LOOP(W, H, NT, r, c)                                        \
  for (int _t = threadIdx.x, r = 0, c = 0; _t < (W) * (H) &&               \
       ((r = _t / (W)), (c = _t - r * (W)), true); _t += (NT))

// Block reduction on the FP32 pipes for the mixed-precision kernels: sums
// are accumulated as float-float pairs (error-free TwoSum), maxima in float.
// Each block writes (hi, lo) to part2; the last block reduces the partials in
// block order and returns the totals in v (as double) on thread 0.
template <int NV, int NT>
__device__ __forceinline__ bool grid_reduce_last_f(float (&v)[NV], float2* part2, unsigned* counter, unsigned max_mask,
                                                   double (&out)[NV]) {
  __shared__ float2 red[NV][NT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = NT / 32;
  auto ffadd = [](float2 a, float2 b) {
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb) + (a.y + b.y);
    const float h = s + e;
    return make_float2(h, e - (h - s));
  };
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const bool is_max = (max_mask >> q) & 1u;
    float2 x = make_float2(v[q], 0.f);
    for (int o = 16; o > 0; o >>= 1) {
      float2 y;
      y.x = __shfl_down_sync(0xffffffffu, x.x, o);
      y.y = __shfl_down_sync(0xffffffffu, x.y, o);
      x = is_max ? make_float2(fmaxf(x.x, y.x), 0.f) : ffadd(x, y);
    }
    if (lane == 0) red[q][warp] = x;
  }
  __syncthreads();
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (threadIdx.x == 0) {
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    for (int q = 0; q < NV; ++q) {
      const bool is_max = (max_mask >> q) & 1u;
      float2 x = red[q][0];
      for (int w = 1; w < NW; ++w) x = is_max ? make_float2(fmaxf(x.x, red[q][w].x), 0.f) : ffadd(x, red[q][w]);
      part2[(long)q * nb + bid] = x;
    }
    __threadfence();
    const unsigned done = atomicAdd(counter, 1u);
    last = (done == (unsigned)(nb - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const bool is_max = (max_mask >> q) & 1u;
    const float2* pv = part2 + (long)q * nb;
    float2 x = make_float2(0.f, 0.f);
    int b = threadIdx.x;
    for (; b + 7 * NT < nb; b += 8 * NT) {  // L2 loads, eight in flight, combined in order
      float2 y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = __ldcg(pv + b + u * NT);
#pragma unroll
      for (int u = 0; u < 8; ++u) x = is_max ? make_float2(fmaxf(x.x, y[u].x), 0.f) : ffadd(x, y[u]);
    }
    for (; b < nb; b += NT) {
      const float2 y = __ldcg(pv + b);
      x = is_max ? make_float2(fmaxf(x.x, y.x), 0.f) : ffadd(x, y);
    }
    for (int o = 16; o > 0; o >>= 1) {
      float2 y;
      y.x = __shfl_down_sync(0xffffffffu, x.x, o);
      y.y = __shfl_down_sync(0xffffffffu, x.y, o);
      x = is_max ? make_float2(fmaxf(x.x, y.x), 0.f) : ffadd(x, y);
    }
    __syncthreads();
    if (lane == 0) red[q][warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      float2 s = red[q][0];
      for (int w = 1; w < NW; ++w) s = is_max ? make_float2(fmaxf(s.x, red[q][w].x), 0.f) : ffadd(s, red[q][w]);
      out[q] = (double)s.x + (double)s.y;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

}  // namespace ns
