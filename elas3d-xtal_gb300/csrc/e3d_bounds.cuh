// Bounds-checked debug build.  Compiled with -DE3D_BOUNDS, every index written
// as E3D_IDX(i, n) is compared with the length n of the buffer it addresses;
// an index outside [0, n) is counted, the first one's source line, value and
// limit are kept in a device record of this translation unit, and 0 is used in
// its place, so the access stays inside the buffer and nothing traps.  The
// host reads and clears the record with bounds_take (exported as
// e3d_debug_bounds).  Without E3D_BOUNDS, E3D_IDX(i, n) is i and the checks
// cost nothing.
#pragma once
#include <cuda_runtime.h>

namespace e3d {

struct BoundsRecord {
  unsigned long long count;
  long long line, index, limit;
};

#ifdef E3D_BOUNDS
static __device__ BoundsRecord g_bounds;

static __device__ __noinline__ long long bounds_fail(long long i, long long n, int line) {
  if (atomicAdd(&g_bounds.count, 1ull) == 0ull) {
    g_bounds.line = line;
    g_bounds.index = i;
    g_bounds.limit = n;
  }
  return 0;
}

__device__ __forceinline__ long long bounds_idx(long long i, long long n, int line) {
  return (i >= 0 && i < n) ? i : bounds_fail(i, n, line);
}

#define E3D_IDX(i, n) bounds_idx((long long)(i), (long long)(n), __LINE__)
#else
#define E3D_IDX(i, n) (i)
#endif

// Host: copies this translation unit's record to out = {count, line, index,
// limit} and clears it.  Returns 1 in a checked build, 0 in a plain one (out
// zeroed), -1 on a CUDA error.
static inline int bounds_take(long long out[4]) {
  out[0] = out[1] = out[2] = out[3] = 0;
#ifdef E3D_BOUNDS
  BoundsRecord r{};
  if (cudaMemcpyFromSymbol(&r, g_bounds, sizeof r) != cudaSuccess) return -1;
  const BoundsRecord zero{};
  if (cudaMemcpyToSymbol(g_bounds, &zero, sizeof zero) != cudaSuccess) return -1;
  out[0] = (long long)r.count;
  out[1] = r.line;
  out[2] = r.index;
  out[3] = r.limit;
  return 1;
#else
  return 0;
#endif
}

}  // namespace e3d
