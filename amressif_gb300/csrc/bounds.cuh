// Bounds-check build (the reference's DEBUG=TRUE build, Exec/GNUmakefile:12).
//
// Compiled with -DNS_BOUNDS_CHECK (libamressif_gb300_check.so), the column-
// marching kernels and the 3D tiled flux pass test every global index they
// form by hand (cp.async sources, direct loads of face column / row N and of
// the periodic images, stores, the multigrid rows, the halo tiles and z
// windows) against the array it addresses: 0 <= index < pitch * (rows), with
// the column (index mod pitch) at most ncol. A failed
// test skips the access and records it in three status words the context
// owns (Geom::check): the number of failures, the first failing index and its
// site number. Nothing traps. In the normal build NS_BCHK is the constant
// true and the tests compile away.
//
// Sites: 1-12 k_inc_col2d, 21-32 k_anchor_col2d, 41-46 k_mg_smooth_col,
// 51-56 k_mg_smooth, 61 k_conv_quick2d, 71-73 k3i_fluxtot (3D).
#pragma once
#include <cuda_runtime.h>

namespace ns {

#ifdef NS_BOUNDS_CHECK
__device__ __forceinline__ bool bounds_ok(unsigned long long* st, long idx, long pitch, long rows, long ncol, int site) {
  const bool ok = idx >= 0 && idx < pitch * rows && (idx % pitch) <= ncol;
  if (!ok && st != nullptr) {
    if (atomicAdd(&st[0], 1ull) == 0ull) {
      st[1] = (unsigned long long)idx;
      st[2] = (unsigned long long)site;
    }
  }
  return ok;
}
#define NS_BCHK(st, idx, pitch, rows, ncol, site) ::ns::bounds_ok((st), (long)(idx), (long)(pitch), (long)(rows), (long)(ncol), (site))
#else
#define NS_BCHK(st, idx, pitch, rows, ncol, site) true
#endif

}  // namespace ns
