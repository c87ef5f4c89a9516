// TMA (cp.async.bulk.tensor) + mbarrier helpers for the stencil's plane
// pipeline, as inline PTX for sm_103a.
//
// Each SoA vector (3 components of nx*ny*nz values, component-major) is
// described by a 4-D tensor map (x, y, z, component).  A tile plane needs the
// 32x8 main box, the halo column to its +x side, the halo row to its +y side and
// the corner: four boxes per vector and plane, each from its own map (a map
// fixes its box).  Periodic wrap is a choice of coordinates (the column after
// the last tile is x = 0), so no box starts at a negative coordinate and every
// x start is a multiple of 32 elements (16-byte aligned); boxes that run past
// the grid edge are zero-filled by the hardware and those lanes are unused.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace e3d {

// Box kinds of one vector: main, +x column, +y row, corner.
enum : int { BOX_MAIN = 0, BOX_COL = 1, BOX_ROW = 2, BOX_CORNER = 3 };

// Tensor maps of the fused FP32 apply: the two search-direction buffers (the
// one read as h_old alternates), z, and the phase ids (3-D, box 32x8x1).
struct PlaneMaps {
  CUtensorMap h0[4];
  CUtensorMap h1[4];
  CUtensorMap z[4];
  CUtensorMap pix;
};

// Box extents (elements) per kind: x, y (z and component boxes are 1 and 3).
constexpr int kBoxX[4] = {32, 4, 32, 4};
constexpr int kBoxY[4] = {8, 8, 1, 1};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// One bounded probe of the phase with parity `parity`; true when it completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done = 0;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the phase with a wall-clock limit; false on timeout or when
// *abort (if given) becomes non-zero.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long timeout_ns,
                                          const volatile int* abort = nullptr) {
  if (mbar_try_wait(bar, parity)) return true;
  unsigned long long t0 = 0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (unsigned long long spins = 0; spins < (1ull << 34); ++spins) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spins & 63ull) == 63ull) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > timeout_ns) return false;
      if (abort && *abort != 0) return false;
    }
  }
  return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (TMA) writes to it.
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders earlier generic-proxy accesses (global and shared) before later
// async-proxy accesses of this thread.
__device__ __forceinline__ void fence_proxy_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int c,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace e3d
