// ccs_bounds.cuh -- index checks of the bounds-checked build (-DCCS_BOUNDS).
//
// In a checked build, an index that a kernel passes to ccs_inb() outside [0, n)
// records the check's site and the index in this translation unit's device word
// (the first hit wins) and makes ccs_inb() return false, and the kernel skips the
// access: the build finds indexing mistakes on small cases without touching memory
// outside an array (ccs_debug_bounds reads the word).  In the normal build
// ccs_inb() is the constant `true` and the checks compile away.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ccs {
namespace {

#ifdef CCS_BOUNDS
__device__ unsigned long long g_bounds_hit = 0ull;

__device__ __forceinline__ bool ccs_inb(long long i, long long n, int site) {
  if (i >= 0 && i < n) return true;
  const unsigned long long code =
      ((unsigned long long)(site & 0xffff) << 48) | ((unsigned long long)i & 0xffffffffffffull);
  atomicCAS(&g_bounds_hit, 0ull, code);
  return false;
}

// the translation unit's first hit since the last call (0: none), cleared
inline unsigned long long bounds_take_tu() {
  unsigned long long v = 0ull;
  const unsigned long long z = 0ull;
  if (cudaMemcpyFromSymbol(&v, g_bounds_hit, sizeof(v)) != cudaSuccess) return 0ull;
  cudaMemcpyToSymbol(g_bounds_hit, &z, sizeof(z));
  return v;
}

// checks index i against [0, n) under `site` and accesses nothing: exercises the
// recording path of the checked build
__global__ void bounds_selftest_kernel(long long i, long long n, int site) {
  if (threadIdx.x == 0 && blockIdx.x == 0) (void)ccs_inb(i, n, site);
}
#else
__device__ __forceinline__ constexpr bool ccs_inb(long long, long long, int) { return true; }
inline unsigned long long bounds_take_tu() { return 0ull; }
#endif

}  // namespace
}  // namespace ccs
