// Kernels of the sm_103a voxel-FE solver.  See e3d_device.cuh for the element
// arithmetic.  Layout in HBM (all component-major, node m = x + nx*(y + ny*z)):
//   u, g, b, z, h[2], Ah : 3*ns values each
//   minv                 : 6*ns (symmetric 3x3 block inverse: 00 11 22 01 02 12)
//   pix                  : ns int32, 0-based phase
//   cs                   : nphase*kCsStride FP64 stiffness tables (C/16 and the summed mode matrices)
//   cs32                 : nphase*24, FP32 upper triangle of C/16 (element_modal_f32)
//   dk                   : nphase*576, [p][a][i][b][j] (reference local order)
//   dkd                  : nphase*72 diagonal 3x3 blocks [p][a][i][j]
//   hx, hy, hd           : tile-edge force halos (see apply_tile)
#pragma once
#include <cstdint>
#include <type_traits>

#include "e3d_bounds.cuh"
#include "e3d_device.cuh"
#include "e3d_tma.cuh"

namespace e3d {

constexpr int TILE_X = 32;
constexpr int TILE_Y = 8;

// Tuning knobs of the persistent PCG kernel (set at build time).
#ifndef E3D_PB_UNROLL_F32
#define E3D_PB_UNROLL_F32 1  // phase-B nodes in flight per thread, FP32 form (2 spills under the 128-register cap)
#endif
#ifndef E3D_PB_UNROLL_F64
#define E3D_PB_UNROLL_F64 1  // phase-B nodes in flight per thread, FP64 form
#endif
#ifndef E3D_F32_BLOCKS_PER_SM
#define E3D_F32_BLOCKS_PER_SM 2  // resident 256-thread blocks per SM, FP32 form
#endif
// Planes per step of the ring-fed FP32 tile: each thread computes E3D_RING_ZS
// consecutive elements of its column between two barriers.  ZS = 1 runs two
// 128-register blocks per SM; ZS = 2 one 255-register block (two independent
// element computations per thread, no spills) -- measured slower at 500^3
// (13.3 vs 9.7 ms per inner iteration): occupancy matters more here.
#ifndef E3D_RING_ZS
#define E3D_RING_ZS 1
#endif
#ifndef E3D_TMA_STAGES
#define E3D_TMA_STAGES (E3D_RING_ZS + 4)  // ring stages per block (ZS + 1 in use, the rest in flight)
#endif
// FP32 tile state kept in shared memory instead of registers: the transformed
// lower node plane (rebuilt from the node buffer for each element) and the
// upper-plane forces carried to the next element (one slot per thread).  With
// the first, the FP32 persistent kernel no longer spills under its 128-register
// cap (500^3 inner iteration 6.9 ms, from 9.2); the second costs more shared
// memory traffic than it saves (6.9 ms either way) and stays off.
#ifndef E3D_F32_POLD_SMEM
#define E3D_F32_POLD_SMEM 1
#endif
#ifndef E3D_F32_CARRY_SMEM
#define E3D_F32_CARRY_SMEM 0
#endif
// FP32 persistent kernel (per-thread loads): the correction update du -= lam*h
// of iteration k is applied in phase A of iteration k+1, which loads h there
// anyway, so phase B reads neither h nor du; the update still pending when the
// launch ends is applied before it returns.
#ifndef E3D_F32_DEFER_U
#define E3D_F32_DEFER_U 1
#endif
// Phase-B planes in flight per thread through cp.async stages (a power of two;
// 0 keeps the one-node register form of pcg_update_tiles).
#ifndef E3D_PB_ASYNC_F32
#define E3D_PB_ASYNC_F32 4
#endif
#ifndef E3D_PB_ASYNC_F64
#define E3D_PB_ASYNC_F64 2
#endif
// FP32 stencil: each element's stiffness row staged in shared memory one plane
// ahead through cp.async (per-thread-load persistent kernel).  Measured slower:
// 500^3 inner iteration 8.41 ms against 5.68 ms with the rows read through the
// read-only path, where a warp whose elements share a grain gets its row in
// one broadcast access.
#ifndef E3D_F32_TAB_ASYNC
#define E3D_F32_TAB_ASYNC 0
#endif
constexpr int kTabAsyncBytes = 2 * 6 * 256 * 16;  // two slots of six float4 per thread (NT = 256)
// FP64 stencil: node sums share the adjoint butterflies between neighbouring
// elements (9 instead of 11 additions per component and node).
#ifndef E3D_F64_SHARED_ADJ
#define E3D_F64_SHARED_ADJ 1
#endif
#ifndef E3D_PB_UNROLL_RING
#define E3D_PB_UNROLL_RING (E3D_RING_ZS == 2 ? 4 : 1)  // phase-B nodes in flight per thread, ring kernel
#endif
constexpr int NT = TILE_X * TILE_Y;  // threads per block of the tile kernels

// Device status codes (host maps them to E3D_*).
enum : int { DEV_OK = 0, DEV_TIMEOUT = 1, DEV_BAD_INDEX = 2 };
// PCG status.
enum : int {
  PCG_RUNNING = 0,
  PCG_CONVERGED = 1,
  PCG_HAH = 2,
  PCG_MAXITER = 3,
  PCG_BREAKDOWN = 4,
  PCG_TIMEOUT = 5,
  PCG_REPLACE = 6  // mixed form: the FP32 residual has dropped far enough for an FP64 replacement
};

struct GridDims {
  int nx, ny, nz;
  long long ns;
  int ntx, nty, ntz;  // tiles per direction
  int tz;             // element planes per tile
  long long ntiles;
};

// Length of one tile-edge halo buffer (hx, hy, hd) with w values per plane row.
__host__ __device__ inline long long halo_len(const GridDims& G, int w) { return 3LL * G.ntiles * G.tz * w; }

// Periodic wrap of v into [0, n); the callers pass neighbours (v in [-n, 2n)),
// handled without an integer division.
__host__ __device__ inline int wrapi(int v, int n) {
  if (v >= 0 && v < n) return v;
  if (v < 0 && v >= -n) return v + n;
  if (v >= n && v < 2 * n) return v - n;
  v %= n;
  return v < 0 ? v + n : v;
}

// Node index -> (x, y, z); 32-bit division when the grid allows it (every grid
// up to 2^32 nodes), far cheaper than the 64-bit one.
__device__ __forceinline__ void node_xyz(const GridDims& G, long long m, int& x, int& y, int& z) {
  if (G.ns <= 0xffffffffLL) {
    const unsigned mm = (unsigned)m, nx = (unsigned)G.nx, ny = (unsigned)G.ny;
    const unsigned q = mm / nx;
    x = (int)(mm - q * nx);
    const unsigned r = q / ny;
    y = (int)(q - r * ny);
    z = (int)r;
  } else {
    x = (int)(m % G.nx);
    y = (int)((m / G.nx) % G.ny);
    z = (int)(m / ((long long)G.nx * G.ny));
  }
}

template <typename T>
struct ApplyArgs {
  GridDims g;
  const int32_t* __restrict__ pix;  // 0-based phase per voxel
  const T* __restrict__ cs;         // scaled stiffness table
  int ncs;                          // rows of cs (every phase id is below it)
  const T* __restrict__ x;          // input (or h_old when fused)
  const T* __restrict__ zv;         // z (fused Fletcher-Reeves update only)
  T gamma;                          // FR coefficient
  int reset;                        // 1: h_new = z
  T* __restrict__ hnew;             // fused: h_new written for owned nodes
  T* __restrict__ y;                // in-tile part of K x
  T* __restrict__ hx;               // [3][ntiles][tz][TILE_Y]
  T* __restrict__ hy;               // [3][ntiles][tz][TILE_X]
  T* __restrict__ hd;               // [3][ntiles][tz]
  T* __restrict__ du;               // deferred correction update (DEFER_U): du -= lam_prev * x, own nodes
  T lam_prev;
};

template <typename T, bool CARRY>
struct ApplySmemT {
  T node[2][3][(TILE_X + 1) * (TILE_Y + 1)];
  T r[9][NT];
};
template <typename T>
struct ApplySmemT<T, true> {
  T node[2][3][(TILE_X + 1) * (TILE_Y + 1)];
  T r[9][NT];
  T carry[12][NT];
};
template <typename T>
using ApplySmem = ApplySmemT<T, sizeof(T) == 4 && E3D_F32_CARRY_SMEM != 0>;

// ---------------------------------------------------------------------------
// TMA plane ring of the fused FP32 stencil.  One stage holds one node plane of
// a tile: for h_old and z the main 32x8 box, the +x column box (4x8), the +y
// row box (32x1) and the corner box (4x1), three components each, then the
// tile's 32x8 phase ids.  Warp 0 keeps the ring full (one lane per box),
// running ahead across the block's tiles; a stage is refilled once every
// thread has read it (after the block barrier of the step that last reads it),
// and consumers wait on the stage's mbarrier with a wall-clock limit.
constexpr int kRingMain = 3 * 32 * 8 * 4;
constexpr int kRingCol = 3 * 4 * 8 * 4;
constexpr int kRingRow = 3 * 32 * 1 * 4;
constexpr int kRingCorner = 3 * 4 * 1 * 4;
constexpr int kRingVec = kRingMain + kRingCol + kRingRow + 128;  // corner box padded to 128 B
constexpr int kRingPix = 32 * 8 * 4;
constexpr int kStageBytes = 2 * kRingVec + kRingPix;
constexpr unsigned kPlaneTx = 2u * (kRingMain + kRingCol + kRingRow + kRingCorner) + kRingPix;
constexpr int kRingSmemBytes = E3D_TMA_STAGES * kStageBytes + 128;  // + alignment slack
static_assert(kRingVec % 128 == 0 && kStageBytes % 128 == 0, "TMA destinations must stay 128-byte aligned");

// Producer state, written by lane 0 of warp 0 and read by warp 0; kept in
// shared memory so it does not occupy registers of every thread.
struct RingCursor {
  long long ptile, tstride, tend;
  const CUtensorMap* hmap;  // the four maps of the buffer read as h_old
  int pzl, pzend;
  unsigned int issued;
};

struct PlaneRing {
  unsigned char* stage;   // E3D_TMA_STAGES * kStageBytes, 128-byte aligned
  uint64_t* full;         // one mbarrier per stage
  RingCursor* cur;        // shared memory
  const PlaneMaps* maps;  // tensor maps in global memory
  int* err;
  unsigned long long timeout_ns;
  unsigned int q;  // planes consumed by this block (same in every thread)
  int failed;      // a wait ran out or an error is flagged: stop waiting and issuing
};

__device__ __forceinline__ void ring_tile_span(const GridDims& G, long long t, int& zl0, int& zl1) {
  const int tiz = (int)(t / ((long long)G.ntx * G.nty));
  const int z0 = tiz * G.tz;
  zl0 = z0 - 1;
  zl1 = z0 + min(G.tz, G.nz - z0);
}

// Warp 0: start the loads of the cursor's next plane into its stage; lane 0
// sets the expected bytes, lanes 0-8 issue one box each, lane 0 advances the
// cursor.
__device__ __forceinline__ void ring_issue(PlaneRing& R, const GridDims& G) {
  RingCursor& C = *R.cur;
  const int lane = threadIdx.x;  // warp 0 only
  // warp-uniform decisions (the cursor was published by the last __syncwarp);
  // the error flag in global memory is read only on the slow path of a wait
  const bool bad = __any_sync(0xffffffffu, R.failed);
  if (bad) R.failed = 1;
  if (bad || C.ptile >= C.tend) return;
  const long long t = C.ptile;
  const int tix = (int)(t % G.ntx);
  const int tiy = (int)((t / G.ntx) % G.nty);
  const int x0 = tix * TILE_X, y0 = tiy * TILE_Y;
  const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0);
  // +x column / +y row of the tile, wrapped; x starts are multiples of 32 or 0
  const int xc = (x0 + wx == G.nx) ? 0 : x0 + wx;
  const int yr = (y0 + wy == G.ny) ? 0 : y0 + wy;
  const int zp = wrapi(C.pzl, G.nz);
  const unsigned s = C.issued % E3D_TMA_STAGES;
  unsigned char* st = R.stage + (size_t)s * kStageBytes;
  uint64_t* bar = R.full + s;
  if (lane == 0) mbar_arrive_expect_tx(bar, kPlaneTx);
  __syncwarp();
  if (lane < 8) {
    const int v = lane >> 2, kind = lane & 3;  // vector (h_old, z) and box kind
    const CUtensorMap* m = (v ? R.maps->z : C.hmap) + kind;
    const int off = v * kRingVec + (kind == BOX_MAIN ? 0 : kind == BOX_COL ? kRingMain
                                                   : kind == BOX_ROW ? kRingMain + kRingCol
                                                                     : kRingMain + kRingCol + kRingRow);
    const int bx = (kind == BOX_COL || kind == BOX_CORNER) ? xc : x0;
    const int by = (kind == BOX_ROW || kind == BOX_CORNER) ? yr : y0;
    tma_load_4d(st + off, m, bx, by, zp, 0, bar);
  } else if (lane == 8) {
    tma_load_3d(st + 2 * kRingVec, &R.maps->pix, x0, y0, zp, bar);
  }
  __syncwarp();
  if (lane == 0) {
    C.issued += 1;
    if (++C.pzl > C.pzend) {
      C.ptile += C.tstride;
      if (C.ptile < C.tend) ring_tile_span(G, C.ptile, C.pzl, C.pzend);
    }
  }
  __syncwarp();
}

// Once per kernel: barriers, from thread 0; followed by __syncthreads.
__device__ __forceinline__ void ring_setup(PlaneRing& R, unsigned char* dyn, uint64_t* bars, RingCursor* cur,
                                           const PlaneMaps* maps, int* err, unsigned long long timeout_ns) {
  const uint32_t a = smem_u32(dyn);
  R.stage = dyn + ((128u - (a & 127u)) & 127u);
  R.full = bars;
  R.cur = cur;
  R.maps = maps;
  R.err = err;
  R.timeout_ns = timeout_ns;
  R.q = 0;
  R.failed = 0;
  if (threadIdx.x == 0) {
    cur->ptile = cur->tend = 0;
    cur->tstride = 1;
    cur->hmap = maps->h0;
    cur->pzl = cur->pzend = 0;
    cur->issued = 0;
    for (int i = 0; i < E3D_TMA_STAGES; ++i) mbar_init(bars + i, 1);
    fence_mbar_init();
  }
  // (the caller's __syncthreads publishes the cursor and the barriers)
}

// Start of one stencil pass over tiles first, first+stride, ... < tend, reading
// h_old through hmap.  Every plane of the previous pass has been consumed.
__device__ __forceinline__ void ring_begin(PlaneRing& R, const GridDims& G, const CUtensorMap* hmap,
                                           long long first, long long stride, long long tend) {
  if (threadIdx.x < 32) {
    if (threadIdx.x == 0) {
      fence_proxy_async_all();  // this block's and (after the grid barrier) the grid's writes before TMA reads
      RingCursor& C = *R.cur;
      C.hmap = hmap;
      C.ptile = first;
      C.tstride = stride;
      C.tend = tend;
      if (first < tend) ring_tile_span(G, first, C.pzl, C.pzend);
    }
    __syncwarp();
    for (int i = 0; i < E3D_TMA_STAGES; ++i) ring_issue(R, G);
  }
}

// All threads: wait until plane number n (n - R.q < E3D_TMA_STAGES) has
// landed; returns its stage.
__device__ __forceinline__ const unsigned char* ring_wait(PlaneRing& R, unsigned n) {
  const unsigned s = n % E3D_TMA_STAGES;
  // fast path: one probe; the slow path polls the error flag and the clock
  if (!R.failed && !mbar_try_wait(R.full + s, (n / E3D_TMA_STAGES) & 1u)) {
    if (!mbar_wait(R.full + s, (n / E3D_TMA_STAGES) & 1u, R.timeout_ns, R.err)) {
      if (*(volatile int*)R.err == DEV_OK) atomicExch(R.err, DEV_TIMEOUT);
      R.failed = 1;
    }
  }
  return R.stage + (size_t)s * kStageBytes;
}

// Stage address of plane number n (already waited for).
__device__ __forceinline__ const unsigned char* ring_stage(const PlaneRing& R, unsigned n) {
  return R.stage + (size_t)(n % E3D_TMA_STAGES) * kStageBytes;
}

// All threads, after a __syncthreads that follows every read of the oldest
// plane R.q: its stage is free (the barrier orders those reads before the
// refill); warp 0 refills it with the cursor's next plane.
__device__ __forceinline__ void ring_release(PlaneRing& R, const GridDims& G) {
  R.q += 1;
  if (threadIdx.x < 32) ring_issue(R, G);
}

// Thread 0, before the block exits: wait (bounded) for the last plane issued
// into each stage, so that no copy is still in flight after a failed pass.
// Phases complete in order, so the last one covers the earlier ones.
__device__ __forceinline__ void ring_drain(PlaneRing& R) {
  if (threadIdx.x != 0) return;
  const unsigned issued = R.cur->issued;
  for (unsigned s = 0; s < E3D_TMA_STAGES && s < issued; ++s) {
    const unsigned n = s + E3D_TMA_STAGES * ((issued - 1 - s) / E3D_TMA_STAGES);
    (void)mbar_wait(R.full + s, (n / E3D_TMA_STAGES) & 1u, 1000000000ull);
  }
}

// One tile: TILE_X x TILE_Y element columns marching through tz element planes
// (plus one redundant plane below).  Each thread owns node column (x0+tx,
// y0+ty) and the element whose lower corner it is.  Element forces are summed
// into the nodes inside the tile through shared memory; the contributions to
// the nodes just past the tile's high-x / high-y edges go to the halo buffers
// and are added by the consumer (apply_finish / the PCG update), which keeps
// every sum in a fixed order.  FUSED: the input is h_new = z + gamma*h_old (or
// z on reset) formed on load -- the Fletcher-Reeves update of the previous
// iteration (src/elas3dxtal_pcg.f90:1988-1995) folded into this pass -- and
// h_new is stored for the tile's own nodes.  Returns this thread's share of
// h_new . (K h_new) through hAh.
//
// TAB_ASYNC (FP32): each element's stiffness row is copied into a per-thread
// shared-memory slot one plane ahead (cp.async, two slots alternating by plane
// parity in `tab`, 2 x 6 x NT float4), so the gather's latency is off the
// element's critical path.
template <typename T, bool FUSED, bool POLD_SMEM = (sizeof(T) == 4 && E3D_F32_POLD_SMEM != 0), bool DEFER_U = false,
          bool TAB_ASYNC = false>
__device__ void apply_tile(const ApplyArgs<T>& A, long long tile, ApplySmem<T>& sm, double& hAh,
                           float4* __restrict__ tab = nullptr) {
  static_assert(!TAB_ASYNC || sizeof(T) == 4, "the staged table rows are the FP32 ones");
  const GridDims& G = A.g;
  const int tid = threadIdx.x;
  const int tx = tid % TILE_X, ty = tid / TILE_X;
  const int tix = (int)(tile % G.ntx);
  const int tiy = (int)((tile / G.ntx) % G.nty);
  const int tiz = (int)(tile / ((long long)G.ntx * G.nty));
  const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
  const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
  const bool active = (tx < wx) && (ty < wy);
  const int xg = x0 + tx, yg = y0 + ty;
  const long long ns = G.ns;
  const long long nxy = (long long)G.nx * G.ny;
  const int nhalo = wx + wy + 1;
  // halo node (lx, ly) for loader thread q = tid < nhalo
  int hlx = 0, hly = 0;
  if (tid < wy) {
    hlx = wx;
    hly = tid;
  } else if (tid < wy + wx) {
    hlx = tid - wy;
    hly = wy;
  } else {
    hlx = wx;
    hly = wy;
  }
  const int hgx = wrapi(x0 + hlx, G.nx), hgy = wrapi(y0 + hly, G.ny);

  // Raw loads of one node plane are issued a step ahead (prefetch) so they are
  // in flight while the previous element computes; commit forms h_new and
  // stores the plane into shared memory.
  T pz_own[3], px_own[3], pz_h[3], px_h[3], pu_own[3];
  const bool need_x = !FUSED || !A.reset;
  auto prefetch = [&](int zl) {
    const int zp = wrapi(zl, G.nz);
    if (active) {
      const long long m = E3D_IDX((long long)xg + (long long)G.nx * yg + nxy * zp, ns);
      const bool own = zl >= z0 && zl < z0 + wz;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (need_x || (DEFER_U && own)) px_own[c] = __ldcg(A.x + m + c * ns);
        if (FUSED) pz_own[c] = __ldcg(A.zv + m + c * ns);
        if (DEFER_U && own) pu_own[c] = A.du[m + c * ns];
      }
    }
    if (tid < nhalo) {
      const long long m = E3D_IDX((long long)hgx + (long long)G.nx * hgy + nxy * zp, ns);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (need_x) px_h[c] = __ldcg(A.x + m + c * ns);
        if (FUSED) pz_h[c] = __ldcg(A.zv + m + c * ns);
      }
    }
  };
  auto combine = [&](const T (&zz)[3], const T (&xx)[3], T (&v)[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (FUSED)
        v[c] = A.reset ? zz[c] : fma_(A.gamma, xx[c], zz[c]);
      else
        v[c] = xx[c];
    }
  };
  auto commit = [&](int zl, bool own) {
    const int zp = wrapi(zl, G.nz);
    T* buf0 = sm.node[(zl + 2) & 1][0];
    const int stride = (TILE_X + 1) * (TILE_Y + 1);
    if (active) {
      T v[3];
      combine(pz_own, px_own, v);
      if (FUSED && own) {
        const long long m = E3D_IDX((long long)xg + (long long)G.nx * yg + nxy * zp, ns);
#pragma unroll
        for (int c = 0; c < 3; ++c) A.hnew[m + c * ns] = v[c];
        if constexpr (DEFER_U) {
          // nothing pending at the first step of a launch (lam_prev = 0): h_old
          // may then hold another solve's direction and is not used
          if (A.lam_prev != T(0)) {
#pragma unroll
            for (int c = 0; c < 3; ++c) A.du[m + c * ns] = pu_own[c] - A.lam_prev * px_own[c];
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) buf0[c * stride + ty * (TILE_X + 1) + tx] = v[c];
    }
    if (tid < nhalo) {
      T v[3];
      combine(pz_h, px_h, v);
#pragma unroll
      for (int c = 0; c < 3; ++c) buf0[E3D_IDX(c * stride + hly * (TILE_X + 1) + hlx, 3 * stride)] = v[c];
    }
  };
  auto read_corners = [&](int zl, T (&v)[3][4]) {
    const T* buf0 = sm.node[(zl + 2) & 1][0];
    const int stride = (TILE_X + 1) * (TILE_Y + 1);
    const int o = ty * (TILE_X + 1) + tx;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[c][0] = buf0[c * stride + o];
      v[c][1] = buf0[c * stride + o + 1];
      v[c][2] = buf0[c * stride + o + TILE_X + 1];
      v[c][3] = buf0[c * stride + o + TILE_X + 2];
    }
  };

  constexpr bool kPoldSmem = POLD_SMEM;
  constexpr bool kCarrySmem = sizeof(T) == 4 && E3D_F32_CARRY_SMEM != 0;
  // FP64: the node sums share the adjoint's partial butterflies between
  // neighbouring elements (see the node-sum step below).
  constexpr bool kShareAdj = sizeof(T) == 8 && E3D_F64_SHARED_ADJ != 0;
  T Pold[3][4], carry[3][4];
  // FP32: the tile's share of h.Ah is summed in FP32 and added to the FP64
  // accumulator once per tile; FP64: every node's term goes straight into it.
  float dot32 = 0.f;
  auto add_dot = [&](T v) {
    if constexpr (sizeof(T) == 4)
      dot32 += v;
    else
      hAh += (double)v;
  };
  const long long ecol = (long long)xg + (long long)G.nx * yg;  // element column
  prefetch(z0 - 1);
  commit(z0 - 1, false);
  __syncthreads();
  if (!kPoldSmem && active) {
    T v0[3][4];
    read_corners(z0 - 1, v0);
#pragma unroll
    for (int c = 0; c < 3; ++c) had_xy(v0[c], Pold[c]);
  }
  prefetch(z0);
  int ph_cur = active ? __ldcs(A.pix + E3D_IDX(ecol + nxy * wrapi(z0 - 1, G.nz), ns)) : 0;
  // TAB_ASYNC: the row of element k sits in slot k & 1; ph_cur then holds the
  // phase of element k + 1 (its row is copied during step k)
  auto tab_issue = [&](int k, int ph) {
    if constexpr (TAB_ASYNC) {
      if (active) {
        float4* d = tab + (k & 1) * 6 * NT + tid;
        const float* src = reinterpret_cast<const float*>(A.cs) + E3D_IDX(ph, A.ncs) * kCs32Stride;
#pragma unroll
        for (int i = 0; i < 6; ++i)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(
                           (unsigned)__cvta_generic_to_shared(d + i * NT)),
                       "l"(src + 4 * i)
                       : "memory");
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
  };
  if constexpr (TAB_ASYNC) {
    tab_issue(z0 - 1, ph_cur);
    ph_cur = (active && z0 < z0 + wz) ? __ldcs(A.pix + E3D_IDX(ecol + nxy * wrapi(z0, G.nz), ns)) : 0;
  }
  const int htiles_stride = G.tz;  // per-tile plane stride in halo buffers
  for (int k = z0 - 1; k < z0 + wz; ++k) {
    const bool own_next = (k + 1 >= z0) && (k + 1 < z0 + wz);
    commit(k + 1, own_next);
    __syncthreads();
    if (k + 2 <= z0 + wz) prefetch(k + 2);
    int ph_nxt;
    if constexpr (TAB_ASYNC) {
      // row of element k + 1 now, phase of element k + 2 for the next step
      if (k + 1 < z0 + wz) tab_issue(k + 1, ph_cur);
      else asm volatile("cp.async.commit_group;\n" ::: "memory");
      ph_nxt = (active && k + 2 < z0 + wz) ? __ldcs(A.pix + E3D_IDX(ecol + nxy * wrapi(k + 2, G.nz), ns)) : 0;
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // element k's row has landed
    } else {
      ph_nxt = (active && k + 1 < z0 + wz) ? __ldcs(A.pix + E3D_IDX(ecol + nxy * wrapi(k + 1, G.nz), ns)) : 0;
    }
    T rr[3][4];
    if (active) {
      T nxt[3][4];
      read_corners(k + 1, nxt);
      if constexpr (kPoldSmem) {  // plane k, intact until the barrier that ends this step
        T v0[3][4];
        read_corners(k, v0);
#pragma unroll
        for (int c = 0; c < 3; ++c) had_xy(v0[c], Pold[c]);
      }
      T Pn[3][4];
      T h[3][8];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        had_xy(nxt[c], Pn[c]);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          h[c][b] = Pn[c][b] + Pold[c][b];
          h[c][b + 4] = Pn[c][b] - Pold[c][b];
        }
      }
      T f[3][8];
      if constexpr (TAB_ASYNC)
        element_modal_f32<NT>(reinterpret_cast<const float*>(tab + (k & 1) * 6 * NT + tid), h[0], h[1], h[2], f[0],
                              f[1], f[2]);
      else if constexpr (sizeof(T) == 4)
        element_modal_f32(A.cs + E3D_IDX(ph_cur, A.ncs) * kCs32Stride, h[0], h[1], h[2], f[0], f[1], f[2]);
      else
        element_modal<T>(A.cs + E3D_IDX(ph_cur, A.ncs) * kCsStride, h[0], h[1], h[2], f[0], f[1], f[2]);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        T lo[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          lo[b] = f[c][b] - f[c][b + 4];
          const T hi = f[c][b] + f[c][b + 4];
          if constexpr (kCarrySmem) {
            if (k >= z0) lo[b] += sm.carry[4 * c + b][tid];
            sm.carry[4 * c + b][tid] = hi;
          } else {
            if (k >= z0) lo[b] += carry[c][b];
            carry[c][b] = hi;
          }
        }
        if (k >= z0) {
          if constexpr (kShareAdj) {  // rr = e0, e1, g0, g1 of had_xy_adj; the butterfly's last step is shared
            rr[c][0] = lo[0] - lo[2];
            rr[c][1] = lo[0] + lo[2];
            rr[c][2] = lo[1] - lo[3];
            rr[c][3] = lo[1] + lo[3];
          } else {
            had_xy_adj(lo, rr[c]);
          }
        }
        if constexpr (!kPoldSmem) {
#pragma unroll
          for (int b = 0; b < 4; ++b) Pold[c][b] = Pn[c][b];
        }
      }
    }
    // plane k's values for the dot products, read before the barrier below
    // (after it, the next step may overwrite this buffer with plane k+2)
    T hk[3][4];
    if (k >= z0 && active) {
      const T* cb = sm.node[(k + 2) & 1][0];
      constexpr int cst = (TILE_X + 1) * (TILE_Y + 1);
      const int o = ty * (TILE_X + 1) + tx;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        hk[c][0] = cb[c * cst + o];
        hk[c][1] = tx == wx - 1 ? cb[c * cst + o + 1] : T(0);
        hk[c][2] = ty == wy - 1 ? cb[c * cst + o + TILE_X + 1] : T(0);
        hk[c][3] = (tx == wx - 1 && ty == wy - 1) ? cb[c * cst + o + TILE_X + 2] : T(0);
      }
    }
    if (kShareAdj && k >= z0) {
      // Node (x, y) collects r0(x,y) + r1(x-1,y) + r2(x,y-1) + r3(x-1,y-1) with
      // r0 = e0 - g0, r1 = e0 + g0, r2 = e1 - g1, r3 = e1 + g1.  Grouped as
      // E = e0(x,y) + e1(x,y-1), G = g0(x,y) + g1(x,y-1) (the element below
      // hands over e1, g1 through shared memory) and then
      // (E - G)(x,y) + (E + G)(x-1,y) (the lane to the left hands over E + G):
      // 9 additions per component and node instead of 11.  Contributions from
      // across the tile's low edges arrive through the halos, as before.
      if (active) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          sm.r[2 * c + 0][tid] = rr[c][1];  // e1: to the element at y+1
          sm.r[2 * c + 1][tid] = rr[c][3];  // g1
        }
      }
      __syncthreads();
      if (ty < wy) {  // warp-uniform: every lane of the row takes part in the shuffles
        const int lz = k - z0;
        T acc[3], pxv[3], hyv[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T E = T(0), Gs = T(0), e1 = T(0), g1 = T(0);
          if (active) {
            E = rr[c][0];
            Gs = rr[c][2];
            if (ty > 0) {
              E += sm.r[2 * c + 0][tid - TILE_X];
              Gs += sm.r[2 * c + 1][tid - TILE_X];
            }
            e1 = rr[c][1];
            g1 = rr[c][3];
          }
          const T P = E + Gs;  // r1 + r3 of this column: to node (x+1, y)
          const T R = e1 + g1;  // r3 alone: to node (x+1, y+1) of the next row
          const T Pl = __shfl_up_sync(0xffffffffu, P, 1);
          const T Rl = __shfl_up_sync(0xffffffffu, R, 1);
          acc[c] = tx > 0 ? (E - Gs) + Pl : (E - Gs);
          pxv[c] = P;
          hyv[c] = tx > 0 ? (e1 - g1) + Rl : (e1 - g1);
          rr[c][3] = R;
        }
        if (active) {
          const long long m = E3D_IDX((long long)xg + (long long)G.nx * yg + nxy * wrapi(k, G.nz), ns);
#pragma unroll
          for (int c = 0; c < 3; ++c) A.y[m + c * ns] = acc[c];
          add_dot(hk[0][0] * acc[0] + hk[1][0] * acc[1] + hk[2][0] * acc[2]);
          const long long hb = tile * htiles_stride + lz;
          if (tx == wx - 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) A.hx[E3D_IDX(((long long)c * G.ntiles * htiles_stride + hb) * TILE_Y + ty, halo_len(G, TILE_Y))] = pxv[c];
            add_dot(hk[0][1] * pxv[0] + hk[1][1] * pxv[1] + hk[2][1] * pxv[2]);
          }
          if (ty == wy - 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) A.hy[E3D_IDX(((long long)c * G.ntiles * htiles_stride + hb) * TILE_X + tx, halo_len(G, TILE_X))] = hyv[c];
            add_dot(hk[0][2] * hyv[0] + hk[1][2] * hyv[1] + hk[2][2] * hyv[2]);
          }
          if (tx == wx - 1 && ty == wy - 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c) A.hd[E3D_IDX((long long)c * G.ntiles * htiles_stride + hb, halo_len(G, 1))] = rr[c][3];
            add_dot(hk[0][3] * rr[0][3] + hk[1][3] * rr[1][3] + hk[2][3] * rr[2][3]);
          }
        }
      }
    } else if (k >= z0) {
      if (active) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          sm.r[3 * c + 0][tid] = rr[c][1];  // to node (x+1, y)
          sm.r[3 * c + 1][tid] = rr[c][2];  // to node (x, y+1)
          sm.r[3 * c + 2][tid] = rr[c][3];  // to node (x+1, y+1)
        }
      }
      __syncthreads();
      if (active) {
        const int lz = k - z0;
        const long long m = E3D_IDX((long long)xg + (long long)G.nx * yg + nxy * wrapi(k, G.nz), ns);
        T hxv[3], hyv[3], acc[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          acc[c] = rr[c][0];
          if (tx > 0) acc[c] += sm.r[3 * c + 0][tid - 1];
          if (ty > 0) acc[c] += sm.r[3 * c + 1][tid - TILE_X];
          if (tx > 0 && ty > 0) acc[c] += sm.r[3 * c + 2][tid - TILE_X - 1];
          A.y[m + c * ns] = acc[c];
          hxv[c] = rr[c][1] + (ty > 0 ? sm.r[3 * c + 2][tid - TILE_X] : T(0));
          hyv[c] = rr[c][2] + (tx > 0 ? sm.r[3 * c + 2][tid - 1] : T(0));
        }
        // per-node dot in T, accumulated in FP64
        add_dot(hk[0][0] * acc[0] + hk[1][0] * acc[1] + hk[2][0] * acc[2]);
        const long long hb = tile * htiles_stride + lz;
        if (tx == wx - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hx[E3D_IDX(((long long)c * G.ntiles * htiles_stride + hb) * TILE_Y + ty, halo_len(G, TILE_Y))] = hxv[c];
          add_dot(hk[0][1] * hxv[0] + hk[1][1] * hxv[1] + hk[2][1] * hxv[2]);
        }
        if (ty == wy - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hy[E3D_IDX(((long long)c * G.ntiles * htiles_stride + hb) * TILE_X + tx, halo_len(G, TILE_X))] = hyv[c];
          add_dot(hk[0][2] * hyv[0] + hk[1][2] * hyv[1] + hk[2][2] * hyv[2]);
        }
        if (tx == wx - 1 && ty == wy - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hd[E3D_IDX((long long)c * G.ntiles * htiles_stride + hb, halo_len(G, 1))] = rr[c][3];
          add_dot(hk[0][3] * rr[0][3] + hk[1][3] * rr[1][3] + hk[2][3] * rr[2][3]);
        }
      }
    } else if constexpr (kPoldSmem) {
      __syncthreads();  // plane z0-1 was re-read: the next step refills its buffer
    }
    ph_cur = ph_nxt;
  }
  if constexpr (TAB_ASYNC) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  if constexpr (sizeof(T) == 4) hAh += (double)dot32;
}

// Shared memory of apply_tile_ring: the in-plane force exchange of the ZS
// planes of a step, double-buffered by step parity so one barrier per step
// suffices.
template <int ZS>
struct RingApplySmem {
  float r[2][9 * ZS][NT];
};

// The fused FP32 tile fed by the plane ring (TMA).  Same element arithmetic,
// values and summation order as apply_tile<float, true>, but every thread reads
// its element's four corners of the next plane straight from the ring stage
// (main box, or the +x column / +y row / corner box at the tile edge) and forms
// h_new = z + gamma*h_old there, so no node buffer and no copy barrier are
// needed.  A step computes ZS consecutive elements of the thread's column
// (ZS = 2: two independent element computations between barriers, the shared
// middle plane transformed once); with the force exchange double-buffered one
// __syncthreads per step orders the steps, and the step's oldest stages are
// refilled right after it.  At a step for element planes k .. k+ZS-1 the ring
// holds plane k at R.q.
template <int ZS>
static __device__ void apply_tile_ring(const ApplyArgs<float>& A, long long tile, RingApplySmem<ZS>& sm, double& hAh,
                                       PlaneRing& R) {
  const GridDims& G = A.g;
  const int tid = threadIdx.x;
  const int tx = tid % TILE_X, ty = tid / TILE_X;
  const int tix = (int)(tile % G.ntx);
  const int tiy = (int)((tile / G.ntx) % G.nty);
  const int tiz = (int)(tile / ((long long)G.ntx * G.nty));
  const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
  const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
  const bool active = (tx < wx) && (ty < wy);
  const long long ns = G.ns;
  const long long nxy = (long long)G.nx * G.ny;
  const long long ncol = (long long)(x0 + tx) + (long long)G.nx * (y0 + ty);
  // stage offset (floats within one vector) and component stride of corner d
  // = dx + 2*dy of this thread's element
  auto corner_at = [&](int d, int& off, int& str) {
    const int lx = tx + (d & 1), ly = ty + (d >> 1);
    if (lx < wx) {
      if (ly < wy) {
        off = ly * TILE_X + lx;
        str = NT;
      } else {
        off = (kRingMain + kRingCol) / 4 + lx;
        str = TILE_X;
      }
    } else {
      if (ly < wy) {
        off = kRingMain / 4 + ly * 4;
        str = TILE_X;
      } else {
        off = (kRingMain + kRingCol + kRingRow) / 4;
        str = 4;
      }
    }
  };
  auto hval = [&](const unsigned char* st, int off) -> float {
    const float x = reinterpret_cast<const float*>(st)[E3D_IDX(off, kRingVec / 4)];
    const float z = reinterpret_cast<const float*>(st + kRingVec)[E3D_IDX(off, kRingVec / 4)];
    return A.reset ? z : fmaf(A.gamma, x, z);
  };
  auto corners = [&](const unsigned char* st, float (&v)[3][4]) {
#pragma unroll
    for (int d = 0; d < 4; ++d) {
      int off, str;
      corner_at(d, off, str);
#pragma unroll
      for (int c = 0; c < 3; ++c) v[c][d] = hval(st, off + c * str);
    }
  };
  auto phase_of = [&](const unsigned char* st) { return reinterpret_cast<const int*>(st + 2 * kRingVec)[tid]; };

  float Pold[3][4], carry[3][4];
  float dot32 = 0.f;
  int ph_cur = 0;
  {
    const unsigned char* st = ring_wait(R, R.q);  // plane z0-1
    if (active) {
      float v0[3][4];
      corners(st, v0);
#pragma unroll
      for (int c = 0; c < 3; ++c) had_xy(v0[c], Pold[c]);
      ph_cur = phase_of(st);
    }
  }
  const int hstride = G.tz;
  int step = 0;
  for (int k = z0 - 1; k < z0 + wz; k += ZS, ++step) {
    const int ne = min(ZS, z0 + wz - k);  // elements k .. k+ne-1 in this step
    float rr[ZS][3][4];
    float hk[ZS][3][4];
#pragma unroll
    for (int j = 0; j < ZS; ++j) {
      if (j < ne) {
        const int kk = k + j;
        const unsigned char* st1 = ring_wait(R, R.q + 1 + j);  // plane kk+1
        int ph_nxt = 0;
        if (active) {
          float nxt[3][4];
          corners(st1, nxt);
          if (kk + 1 >= z0 && kk + 1 < z0 + wz) {
            const long long m = E3D_IDX(ncol + nxy * (kk + 1), ns);
#pragma unroll
            for (int c = 0; c < 3; ++c) A.hnew[m + c * ns] = nxt[c][0];
          }
          ph_nxt = phase_of(st1);
          float Pn[3][4], h[3][8];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            had_xy(nxt[c], Pn[c]);
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              h[c][b] = Pn[c][b] + Pold[c][b];
              h[c][b + 4] = Pn[c][b] - Pold[c][b];
            }
          }
          float f[3][8];
          element_modal_f32(A.cs + E3D_IDX(ph_cur, A.ncs) * kCs32Stride, h[0], h[1], h[2], f[0], f[1], f[2]);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float lo[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              lo[b] = f[c][b] - f[c][b + 4];
              const float hi = f[c][b] + f[c][b + 4];
              if (kk >= z0) lo[b] += carry[c][b];
              carry[c][b] = hi;
            }
            if (kk >= z0) had_xy_adj(lo, rr[j][c]);
#pragma unroll
            for (int b = 0; b < 4; ++b) Pold[c][b] = Pn[c][b];
          }
        }
        // plane kk's h_new for the dot products, read before the barrier (the
        // stage is refilled after it)
        if (kk >= z0 && active) {
          const unsigned char* st0 = ring_stage(R, R.q + j);
#pragma unroll
          for (int d = 0; d < 4; ++d) {
            const bool need = d == 0 || (d == 1 && tx == wx - 1) || (d == 2 && ty == wy - 1) ||
                              (d == 3 && tx == wx - 1 && ty == wy - 1);
            int off, str;
            corner_at(d, off, str);
#pragma unroll
            for (int c = 0; c < 3; ++c) hk[j][c][d] = need ? hval(st0, off + c * str) : 0.f;
          }
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            sm.r[step & 1][9 * j + 3 * c + 0][tid] = rr[j][c][1];  // to node (x+1, y)
            sm.r[step & 1][9 * j + 3 * c + 1][tid] = rr[j][c][2];  // to node (x, y+1)
            sm.r[step & 1][9 * j + 3 * c + 2][tid] = rr[j][c][3];  // to node (x+1, y+1)
          }
        }
        ph_cur = ph_nxt;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < ZS; ++j)
      if (j < ne) ring_release(R, G);  // planes k .. k+ne-1
#pragma unroll
    for (int j = 0; j < ZS; ++j) {
      const int kk = k + j;
      if (j < ne && kk >= z0 && active) {
        const float(*r)[NT] = sm.r[step & 1] + 9 * j;
        const int lz = kk - z0;
        const long long m = E3D_IDX(ncol + nxy * kk, ns);
        float hxv[3], hyv[3], acc[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          acc[c] = rr[j][c][0];
          if (tx > 0) acc[c] += r[3 * c + 0][tid - 1];
          if (ty > 0) acc[c] += r[3 * c + 1][tid - TILE_X];
          if (tx > 0 && ty > 0) acc[c] += r[3 * c + 2][tid - TILE_X - 1];
          A.y[m + c * ns] = acc[c];
          hxv[c] = rr[j][c][1] + (ty > 0 ? r[3 * c + 2][tid - TILE_X] : 0.f);
          hyv[c] = rr[j][c][2] + (tx > 0 ? r[3 * c + 2][tid - 1] : 0.f);
        }
        dot32 += hk[j][0][0] * acc[0] + hk[j][1][0] * acc[1] + hk[j][2][0] * acc[2];
        const long long hb = tile * hstride + lz;
        if (tx == wx - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hx[E3D_IDX(((long long)c * G.ntiles * hstride + hb) * TILE_Y + ty, halo_len(G, TILE_Y))] = hxv[c];
          dot32 += hk[j][0][1] * hxv[0] + hk[j][1][1] * hxv[1] + hk[j][2][1] * hxv[2];
        }
        if (ty == wy - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hy[E3D_IDX(((long long)c * G.ntiles * hstride + hb) * TILE_X + tx, halo_len(G, TILE_X))] = hyv[c];
          dot32 += hk[j][0][2] * hyv[0] + hk[j][1][2] * hyv[1] + hk[j][2][2] * hyv[2];
        }
        if (tx == wx - 1 && ty == wy - 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) A.hd[E3D_IDX((long long)c * G.ntiles * hstride + hb, halo_len(G, 1))] = rr[j][c][3];
          dot32 += hk[j][0][3] * rr[j][0][3] + hk[j][1][3] * rr[j][1][3] + hk[j][2][3] * rr[j][2][3];
        }
      }
    }
  }
  ring_release(R, G);  // plane z0+wz, last read before the final step's barrier
  hAh += (double)dot32;
}

// Halo contribution for node (x, y, z) from the neighbouring tiles.
template <typename T>
__device__ __forceinline__ void halo_add(const GridDims& G, const T* __restrict__ hx,
                                         const T* __restrict__ hy, const T* __restrict__ hd,
                                         int x, int y, int z, T (&v)[3]) {
  const int tix = x / TILE_X, lx = x - tix * TILE_X;
  const int tiy = y / TILE_Y, ly = y - tiy * TILE_Y;
  const int tiz = z / G.tz, lz = z - tiz * G.tz;
  if (lx != 0 && ly != 0) return;
  const int txl = tix == 0 ? G.ntx - 1 : tix - 1;
  const int tyd = tiy == 0 ? G.nty - 1 : tiy - 1;
  const long long plane = (long long)tiz * G.nty;
  const long long per_c = G.ntiles * G.tz;
  if (lx == 0) {
    const long long t = (long long)txl + (long long)G.ntx * (tiy + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hx + E3D_IDX((c * per_c + t * G.tz + lz) * TILE_Y + ly, 3 * per_c * TILE_Y));
  }
  if (ly == 0) {
    const long long t = (long long)tix + (long long)G.ntx * (tyd + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hy + E3D_IDX((c * per_c + t * G.tz + lz) * TILE_X + lx, 3 * per_c * TILE_X));
  }
  if (lx == 0 && ly == 0) {
    const long long t = (long long)txl + (long long)G.ntx * (tyd + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hd + E3D_IDX(c * per_c + t * G.tz + lz, 3 * per_c));
  }
}

// halo_add for a node whose tile coordinates are known (no integer division);
// same additions in the same order.
template <typename T>
__device__ __forceinline__ void halo_add_tile(const GridDims& G, const T* __restrict__ hx,
                                              const T* __restrict__ hy, const T* __restrict__ hd,
                                              int tix, int tiy, int tiz, int lx, int ly, int lz, T (&v)[3]) {
  if (lx != 0 && ly != 0) return;
  const int txl = tix == 0 ? G.ntx - 1 : tix - 1;
  const int tyd = tiy == 0 ? G.nty - 1 : tiy - 1;
  const long long plane = (long long)tiz * G.nty;
  const long long per_c = G.ntiles * G.tz;
  if (lx == 0) {
    const long long t = (long long)txl + (long long)G.ntx * (tiy + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hx + E3D_IDX((c * per_c + t * G.tz + lz) * TILE_Y + ly, 3 * per_c * TILE_Y));
  }
  if (ly == 0) {
    const long long t = (long long)tix + (long long)G.ntx * (tyd + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hy + E3D_IDX((c * per_c + t * G.tz + lz) * TILE_X + lx, 3 * per_c * TILE_X));
  }
  if (lx == 0 && ly == 0) {
    const long long t = (long long)txl + (long long)G.ntx * (tyd + plane);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += __ldcg(hd + E3D_IDX(c * per_c + t * G.tz + lz, 3 * per_c));
  }
}

// ---------------------------------------------------------------------------
// Stand-alone apply: one tile per block, then apply_finish adds the halos.
template <typename T>
__global__ void __launch_bounds__(NT, 1) apply_tiles_kernel(ApplyArgs<T> A, double* partial) {
  __shared__ ApplySmem<T> sm;
  __shared__ double red[NT / 32];
  double hAh = 0.0;
  apply_tile<T, false>(A, blockIdx.x, sm, hAh);
  const double s = block_sum<NT>(hAh, red);
  if (partial && threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <typename T>
__global__ void apply_finish_kernel(GridDims G, const T* __restrict__ yin, const T* __restrict__ hx,
                                    const T* __restrict__ hy, const T* __restrict__ hd,
                                    T* __restrict__ yout) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= G.ns) return;
  int x, y, z;
  node_xyz(G, m, x, y, z);
  T v[3] = {yin[m], yin[m + G.ns], yin[m + 2 * G.ns]};
  halo_add<T>(G, hx, hy, hd, x, y, z, v);
  yout[m] = v[0];
  yout[m + G.ns] = v[1];
  yout[m + 2 * G.ns] = v[2];
}

// energy_OpenMP tail (src/elas3dxtal_pcg.f90:1332-1340): g = Ku + b,
// partial sums of (u.Ku/2 + b.u) and of g.g (gg0, :452).
static __global__ void __launch_bounds__(256) energy_finish_kernel(GridDims G, const double* __restrict__ ku,
                                                            const double* __restrict__ hx,
                                                            const double* __restrict__ hy,
                                                            const double* __restrict__ hd,
                                                            const double* __restrict__ u,
                                                            const double* __restrict__ b,
                                                            double* __restrict__ g, double* partial) {
  __shared__ double red[8];
  double eu = 0.0, gg = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < G.ns;
       m += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    node_xyz(G, m, x, y, z);
    double v[3] = {ku[m], ku[m + G.ns], ku[m + 2 * G.ns]};
    halo_add<double>(G, hx, hy, hd, x, y, z, v);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long i = m + c * G.ns;
      eu += 0.5 * u[i] * v[c] + b[i] * u[i];
      const double gv = v[c] + b[i];
      g[i] = gv;
      gg += gv * gv;
    }
  }
  const double s1 = block_sum<256>(eu, red);
  const double s2 = block_sum<256>(gg, red);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s1;
    partial[2 * blockIdx.x + 1] = s2;
  }
}

// Sums n partials of stride `stride` in a fixed order (single block).
static __global__ void reduce_partials_kernel(const double* __restrict__ partial, int n, int stride,
                                       int nfields, double* __restrict__ out) {
  __shared__ double red[8];
  for (int f = 0; f < nfields; ++f) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[(long long)i * stride + f];
    const double t = block_sum<256>(s, red);
    if (threadIdx.x == 0) out[f] = t;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// femat.  One block of 32 threads per phase.
struct FematParams {
  int nphase, flag_m;
  double c11, c12, c44, K1, G1, Km, Gm;
};

// rotatestiffnessby (src/elas3dxtal_pcg.f90:2535-2633) for one grain.
static __device__ void bond_rotate(const double r[3], double c11, double c12, double c44, double out[6][6]) {
  double Cc[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Cc[i][j] = 0.0;
  Cc[0][0] = Cc[1][1] = Cc[2][2] = c11;
  Cc[0][1] = Cc[0][2] = Cc[1][2] = Cc[1][0] = Cc[2][0] = Cc[2][1] = c12;
  Cc[3][3] = Cc[4][4] = Cc[5][5] = c44;
  const double rdotr = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double term1 = 1.0 - rdotr;
  double term2 = 1.0 + rdotr;
  double Q[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Q[i][j] = (i == j ? term1 : 0.0) + 2.0 * r[i] * r[j];
  Q[0][1] -= 2.0 * r[2];
  Q[0][2] += 2.0 * r[1];
  Q[1][2] -= 2.0 * r[0];
  Q[1][0] += 2.0 * r[2];
  Q[2][0] -= 2.0 * r[1];
  Q[2][1] += 2.0 * r[0];
  if (term2 > 1.0e-12) {
    term2 = 1.0 / term2;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Q[i][j] *= term2;
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Q[i][j] = (i == j) ? 1.0 : 0.0;
  }
  double N[6][6];
  for (int row = 0; row < 3; ++row) {
    N[row][0] = Q[row][0] * Q[row][0];
    N[row][1] = Q[row][1] * Q[row][1];
    N[row][2] = Q[row][2] * Q[row][2];
    N[row][3] = Q[row][1] * Q[row][2];
    N[row][4] = Q[row][2] * Q[row][0];
    N[row][5] = Q[row][0] * Q[row][1];
  }
  N[3][0] = 2.0 * Q[2][0] * Q[0][0];
  N[3][1] = 2.0 * Q[2][1] * Q[0][1];
  N[3][2] = 2.0 * Q[2][2] * Q[0][2];
  N[3][3] = Q[0][1] * Q[2][2] + Q[0][2] * Q[2][1];
  N[3][4] = Q[0][2] * Q[2][0] + Q[0][0] * Q[2][2];
  N[3][5] = Q[0][0] * Q[2][1] + Q[0][1] * Q[2][0];
  N[4][0] = 2.0 * Q[1][0] * Q[2][0];
  N[4][1] = 2.0 * Q[1][1] * Q[2][1];
  N[4][2] = 2.0 * Q[1][2] * Q[2][2];
  N[4][3] = Q[1][1] * Q[2][2] + Q[1][2] * Q[2][1];
  N[4][4] = Q[1][0] * Q[2][2] + Q[1][2] * Q[2][0];
  N[4][5] = Q[1][1] * Q[2][0] + Q[1][0] * Q[2][1];
  N[5][0] = 2.0 * Q[0][0] * Q[1][0];
  N[5][1] = 2.0 * Q[0][1] * Q[1][1];
  N[5][2] = 2.0 * Q[0][2] * Q[1][2];
  N[5][3] = Q[0][1] * Q[1][2] + Q[0][2] * Q[1][1];
  N[5][4] = Q[0][2] * Q[1][0] + Q[0][0] * Q[1][2];
  N[5][5] = Q[0][0] * Q[1][1] + Q[0][1] * Q[1][0];
  double Tm[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += N[k][i] * Cc[k][j];
      Tm[i][j] = s;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += Tm[i][k] * N[k][j];
      out[i][j] = s;
    }
}

// Phase ids from device memory: 1-based with the range check of ppixel_hdf5
// (src/elas3dxtal_pcg.f90:2986-2989) -> 0-based; flags DEV_BAD_INDEX.
static __global__ void pix_from_device_kernel(long long ns, const int32_t* __restrict__ in, int nphase,
                                              int32_t* __restrict__ out, int* err) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (long long)gridDim.x * blockDim.x) {
    const int32_t v = in[m];
    if (v < 1 || v > nphase) {
      atomicExch(err, DEV_BAD_INDEX);
      out[m] = 0;
    } else {
      out[m] = v - 1;
    }
  }
}

// The same check and conversion in place: the 1-based ids were copied into
// the phase map as they came from the host (err may be null when the host has
// checked the ids already).
static __global__ void pix_to_zero_based_kernel(long long ns, int nphase, int32_t* pix, int* err) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (long long)gridDim.x * blockDim.x) {
    const int32_t v = pix[m];
    if (v < 1 || v > nphase) {
      if (err) atomicExch(err, DEV_BAD_INDEX);
      pix[m] = 0;
    } else {
      pix[m] = v - 1;
    }
  }
}

// Reference local node r (1..8 -> 0..7) to corner index a = ox + 2oy + 4oz.
static __constant__ int kRefToCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};

static __global__ void femat_phase_kernel(FematParams P, const double* __restrict__ rod, double* __restrict__ cmod,
                                   double* __restrict__ cs, float* __restrict__ cs32,
                                   double* __restrict__ dk, double* __restrict__ dkd) {
  const int p = blockIdx.x;
  __shared__ double csh[kCsStride];
  __shared__ double col[24][24];  // col[c][r] = (K e_c)[r], c/r = refnode*3 + dof
  if (threadIdx.x == 0) {
    double C6[6][6];
    const bool iso_phase = (p == P.nphase - 1) || (P.flag_m == 0);
    if (iso_phase) {
      // K*ck + G*cmu (src/elas3dxtal_pcg.f90:655-664, 680-682, 701-705)
      const double K = (p == P.nphase - 1) ? P.K1 : P.Km;
      const double Gs = (p == P.nphase - 1) ? P.G1 : P.Gm;
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
          const double ck = (i < 3 && j < 3) ? 1.0 : 0.0;
          double cmu = 0.0;
          if (i < 3 && j < 3) cmu = (i == j) ? 4.0 / 3.0 : -2.0 / 3.0;
          if (i >= 3 && i == j) cmu = 1.0;
          C6[i][j] = K * ck + Gs * cmu;
        }
    } else {
      const double r[3] = {rod[3 * p], rod[3 * p + 1], rod[3 * p + 2]};
      bond_rotate(r, P.c11, P.c12, P.c44, C6);
    }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) cmod[p + (long long)P.nphase * (i + 6 * j)] = C6[i][j];
    modal_table(C6, csh);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kCsStride; i += blockDim.x) cs[(long long)p * kCsStride + i] = csh[i];
  for (int r = threadIdx.x; r < 6; r += blockDim.x)  // FP32: upper triangle of C/16
    for (int c = r; c < 6; ++c) cs32[(long long)p * kCs32Stride + sym6(r, c)] = (float)csh[6 * r + c];
  for (int i = 21 + threadIdx.x; i < kCs32Stride; i += blockDim.x) cs32[(long long)p * kCs32Stride + i] = 0.f;
  // dk columns: K applied to unit nodal vectors with the same element routine
  // as the stencil, so the preconditioner and b see exactly that matrix.
  if (threadIdx.x < 24) {
    const int cidx = threadIdx.x;
    const int rb = cidx / 3, j = cidx % 3;
    double u[3][8], r[3][8];
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 8; ++a) u[c][a] = 0.0;
    u[j][kRefToCorner[rb]] = 1.0;
    element_apply<double>(csh, u, r);
    for (int ra = 0; ra < 8; ++ra)
      for (int i = 0; i < 3; ++i) col[cidx][ra * 3 + i] = r[i][kRefToCorner[ra]];
  }
  __syncthreads();
  // symmetric dk: entry (r, c) taken from the column with the larger index
  for (int e = threadIdx.x; e < 576; e += blockDim.x) {
    const int r = e / 24, c = e % 24;
    const double v = (r <= c) ? col[c][r] : col[r][c];
    dk[(long long)p * 576 + e] = v;
    const int ra = r / 3, i = r % 3, cb = c / 3, j = c % 3;
    if (ra == cb) dkd[(long long)p * 72 + ra * 9 + i * 3 + j] = v;
  }
}

// Periodic-jump force b (src/elas3dxtal_pcg.f90:815-1100), node-centric so
// the sum over a node's boundary elements has a fixed order.  An element with
// lower corner (i,j,k) on the high face of any direction d has nodal jumps
// delta(a, :) = sum_d [wrap_d] [o_d(a)] E(:, d) n_d.
struct JumpParams {
  double E[3][3];  // symmetric strain tensor
};

__device__ __forceinline__ void element_delta(const GridDims& G, const JumpParams& J, int i, int j, int k,
                                              double (&d)[8][3], bool& any) {
  const bool wx = (i == G.nx - 1), wy = (j == G.ny - 1), wz = (k == G.nz - 1);
  any = wx || wy || wz;
  for (int ra = 0; ra < 8; ++ra) {
    const int a = kRefToCorner[ra];
    const int ox = a & 1, oy = (a >> 1) & 1, oz = (a >> 2) & 1;
    for (int c = 0; c < 3; ++c) {
      double v = 0.0;
      if (wx && ox) v += J.E[c][0] * (double)G.nx;
      if (wy && oy) v += J.E[c][1] * (double)G.ny;
      if (wz && oz) v += J.E[c][2] * (double)G.nz;
      d[ra][c] = v;
    }
  }
}

// Boundary nodes (x, y or z on a face of the box), each once: the two x faces
// whole, then the y faces at interior x, then the z faces at interior x and y.
// Consecutive indices are consecutive x where the set allows, so a warp's
// lanes share the boundary work instead of idling beside one boundary lane.
__host__ __device__ inline long long boundary_node_count(const GridDims& G) {
  const long long fx = G.nx > 1 ? 2 : 1, fy = G.ny > 1 ? 2 : 1, fz = G.nz > 1 ? 2 : 1;
  const long long ix = G.nx > 2 ? G.nx - 2 : 0, iy = G.ny > 2 ? G.ny - 2 : 0;
  return fx * G.ny * G.nz + ix * fy * G.nz + ix * iy * fz;
}

__device__ __forceinline__ void boundary_node(const GridDims& G, long long t, int& x, int& y, int& z) {
  const long long fx = G.nx > 1 ? 2 : 1, fy = G.ny > 1 ? 2 : 1;
  const long long ix = G.nx > 2 ? G.nx - 2 : 0, iy = G.ny > 2 ? G.ny - 2 : 0;
  const long long na = fx * G.ny * G.nz, nb = ix * fy * G.nz;
  if (t < na) {
    const long long r = t / fx;
    x = (t % fx) == 0 ? 0 : G.nx - 1;
    y = (int)(r % G.ny);
    z = (int)(r / G.ny);
  } else if (t < na + nb) {
    const long long s = t - na, r = s / ix;
    x = 1 + (int)(s % ix);
    y = (r % fy) == 0 ? 0 : G.ny - 1;
    z = (int)(r / fy);
  } else {
    const long long s = t - na - nb, r = s / ix;
    x = 1 + (int)(s % ix);
    y = 1 + (int)(r % iy);
    z = (r / iy) == 0 ? 0 : G.nz - 1;
  }
}

// b over the boundary nodes listed by boundary_node (b is zero elsewhere and
// cleared beforehand): one thread per boundary node.
static __global__ void femat_b_kernel(GridDims G, JumpParams J, const int32_t* __restrict__ pix,
                               const double* __restrict__ dk, double* __restrict__ b) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= boundary_node_count(G)) return;
  int x, y, z;
  boundary_node(G, t, x, y, z);
  const long long m = E3D_IDX((long long)x + (long long)G.nx * y + (long long)G.nx * G.ny * z, G.ns);
  double acc[3] = {0.0, 0.0, 0.0};
  // elements containing m in reference order 27,7,6,5,25,15,14,13 (local node ra)
  for (int ra = 0; ra < 8; ++ra) {
    const int a = kRefToCorner[ra];
    const int ex = wrapi(x - (a & 1), G.nx), ey = wrapi(y - ((a >> 1) & 1), G.ny),
              ez = wrapi(z - ((a >> 2) & 1), G.nz);
    double d[8][3];
    bool any;
    element_delta(G, J, ex, ey, ez, d, any);
    if (!any) continue;
    const int ph = pix[E3D_IDX((long long)ex + (long long)G.nx * ey + (long long)G.nx * G.ny * ez, G.ns)];
    const double* D = dk + (long long)ph * 576;
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int rb = 0; rb < 8; ++rb)
        for (int jj = 0; jj < 3; ++jj) s += D[(ra * 3 + i) * 24 + rb * 3 + jj] * d[rb][jj];
      acc[i] += s;
    }
  }
  b[m] = acc[0];
  b[m + G.ns] = acc[1];
  b[m + 2 * G.ns] = acc[2];
}

// Constant C = 1/2 sum_e delta_e^T K_e delta_e over boundary elements.
static __global__ void __launch_bounds__(256) femat_c_kernel(GridDims G, JumpParams J, const int32_t* __restrict__ pix,
                                                      const double* __restrict__ dk, double* partial) {
  __shared__ double red[8];
  double acc = 0.0;
  // boundary elements: enumerate the three high faces without double counting
  const long long nfx = (long long)G.ny * G.nz;                        // i = nx-1
  const long long nfy = (long long)(G.nx - 1) * G.nz;                  // j = ny-1, i < nx-1
  const long long nfz = (long long)(G.nx - 1) * (G.ny - 1);            // k = nz-1, i < nx-1, j < ny-1
  const long long total = nfx + nfy + nfz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    if (t < nfx) {
      i = G.nx - 1;
      j = (int)(t % G.ny);
      k = (int)(t / G.ny);
    } else if (t < nfx + nfy) {
      const long long s = t - nfx;
      j = G.ny - 1;
      i = (int)(s % (G.nx - 1));
      k = (int)(s / (G.nx - 1));
    } else {
      const long long s = t - nfx - nfy;
      k = G.nz - 1;
      i = (int)(s % (G.nx - 1));
      j = (int)(s / (G.nx - 1));
    }
    double d[8][3];
    bool any;
    element_delta(G, J, i, j, k, d, any);
    const int ph = pix[E3D_IDX((long long)i + (long long)G.nx * j + (long long)G.nx * G.ny * k, G.ns)];
    const double* D = dk + (long long)ph * 576;
    double e = 0.0;
    for (int r = 0; r < 24; ++r) {
      double s = 0.0;
      for (int c = 0; c < 24; ++c) s += D[r * 24 + c] * d[c / 3][c % 3];
      e += d[r / 3][r % 3] * s;
    }
    acc += 0.5 * e;
  }
  const double s = block_sum<256>(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Affine initial guess (src/elas3dxtal_pcg.f90:423-438).
static __global__ void affine_kernel(GridDims G, JumpParams J, double* __restrict__ u) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= G.ns) return;
  int xi, yi, zi;
  node_xyz(G, m, xi, yi, zi);
  const double x = xi, y = yi, z = zi;
  const double exx = J.E[0][0], eyy = J.E[1][1], ezz = J.E[2][2];
  const double exy = J.E[0][1], exz = J.E[0][2], eyz = J.E[1][2];
  u[m] = x * exx + y * exy + z * exz;
  u[m + G.ns] = x * exy + y * eyy + z * eyz;
  u[m + 2 * G.ns] = x * exz + y * eyz + z * ezz;
}

// invert3x3 (src/elas3dxtal_pcg.f90:2046-2147); a is row-major a[i][j].
__device__ __forceinline__ void invert3x3(const double a[3][3], double ai[3][3]) {
  const double c11 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  const double c21 = -a[1][0] * a[2][2] + a[1][2] * a[2][0];
  const double c31 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  const double det = a[0][0] * c11 + a[0][1] * c21 + a[0][2] * c31;
  if (fabs(det) < 1e-14) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ai[i][j] = 0.0;
    return;
  }
  const double inv_det = 1.0 / det;
  const double c12 = -a[0][1] * a[2][2] + a[0][2] * a[2][1];
  const double c22 = a[0][0] * a[2][2] - a[0][2] * a[2][0];
  const double c32 = -a[0][0] * a[2][1] + a[0][1] * a[2][0];
  const double c13 = a[0][1] * a[1][2] - a[0][2] * a[1][1];
  const double c23 = -a[0][0] * a[1][2] + a[0][2] * a[1][0];
  const double c33 = a[0][0] * a[1][1] - a[0][1] * a[1][0];
  ai[0][0] = c11 * inv_det;
  ai[1][0] = c21 * inv_det;
  ai[2][0] = c31 * inv_det;
  ai[0][1] = c12 * inv_det;
  ai[1][1] = c22 * inv_det;
  ai[2][1] = c32 * inv_det;
  ai[0][2] = c13 * inv_det;
  ai[1][2] = c23 * inv_det;
  ai[2][2] = c33 * inv_det;
}

// Block-Jacobi (src/elas3dxtal_pcg.f90:1498-1520): sum of the node's diagonal
// 3x3 blocks over its 8 elements (reference order), inverted.  Stores the
// symmetric inverse as 6 SoA planes (00 11 22 01 02 12) in FP64 and FP32.
static __global__ void bjacobi_kernel(GridDims G, const int32_t* __restrict__ pix, const double* __restrict__ dkd,
                               double* __restrict__ minv, float* __restrict__ minv32, int identity = 0) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= G.ns) return;
  if (identity) {  // plain CG: z = g
    for (int q = 0; q < 6; ++q) {
      const double v = q < 3 ? 1.0 : 0.0;
      if (minv) minv[m + q * G.ns] = v;
      if (minv32) minv32[m + q * G.ns] = (float)v;
    }
    return;
  }
  int x, y, z;
  node_xyz(G, m, x, y, z);
  double M[3][3];
  for (int ra = 0; ra < 8; ++ra) {
    const int a = kRefToCorner[ra];
    const int ex = wrapi(x - (a & 1), G.nx), ey = wrapi(y - ((a >> 1) & 1), G.ny),
              ez = wrapi(z - ((a >> 2) & 1), G.nz);
    const int ph = pix[E3D_IDX((long long)ex + (long long)G.nx * ey + (long long)G.nx * G.ny * ez, G.ns)];
    const double* D = dkd + (long long)ph * 72 + ra * 9;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M[i][j] = (ra == 0) ? D[i * 3 + j] : M[i][j] + D[i * 3 + j];
  }
  double Mi[3][3];
  invert3x3(M, Mi);
  const double s[6] = {Mi[0][0], Mi[1][1], Mi[2][2], Mi[0][1], Mi[0][2], Mi[1][2]};
  for (int q = 0; q < 6; ++q) {
    if (minv) minv[m + q * G.ns] = s[q];
    if (minv32) minv32[m + q * G.ns] = (float)s[q];
  }
}

template <typename T>
__device__ __forceinline__ void precond3(const T* __restrict__ mi, long long m, long long ns, const T (&g)[3],
                                         T (&z)[3]) {
  const T a00 = mi[m], a11 = mi[m + ns], a22 = mi[m + 2 * ns];
  const T a01 = mi[m + 3 * ns], a02 = mi[m + 4 * ns], a12 = mi[m + 5 * ns];
  // z(i) = Minv(i,1) g1 + Minv(i,2) g2 + Minv(i,3) g3 (src/elas3dxtal_pcg.f90:1930-1932)
  z[0] = a00 * g[0] + a01 * g[1] + a02 * g[2];
  z[1] = a01 * g[0] + a11 * g[1] + a12 * g[2];
  z[2] = a02 * g[0] + a12 * g[1] + a22 * g[2];
}

// ---------------------------------------------------------------------------
// Stress (stress_OpenMP :2149-2408, stress_fullfield_OpenMP :2723-2833).
__device__ __forceinline__ void voxel_strain(const GridDims& G, const JumpParams& J, const double* __restrict__ u,
                                             int x, int y, int z, double (&eps)[6]) {
  double v[3][8];
  for (int a = 0; a < 8; ++a) {
    const int ox = a & 1, oy = (a >> 1) & 1, oz = (a >> 2) & 1;
    const int xx = x + ox >= G.nx ? 0 : x + ox, yy = y + oy >= G.ny ? 0 : y + oy,
              zz = z + oz >= G.nz ? 0 : z + oz;
    const long long mm = E3D_IDX((long long)xx + (long long)G.nx * yy + (long long)G.nx * G.ny * zz, G.ns);
    for (int c = 0; c < 3; ++c) v[c][a] = u[mm + c * G.ns];
  }
  // periodic jump, x then y then z as at :2282-2323
  if (x == G.nx - 1)
    for (int a = 0; a < 8; ++a)
      if (a & 1)
        for (int c = 0; c < 3; ++c) v[c][a] += J.E[c][0] * (double)G.nx;
  if (y == G.ny - 1)
    for (int a = 0; a < 8; ++a)
      if (a & 2)
        for (int c = 0; c < 3; ++c) v[c][a] += J.E[c][1] * (double)G.ny;
  if (z == G.nz - 1)
    for (int a = 0; a < 8; ++a)
      if (a & 4)
        for (int c = 0; c < 3; ++c) v[c][a] += J.E[c][2] * (double)G.nz;
  // centre strain = (1/4) x first-order Hadamard differences (engineering shear)
  double dX[3], dY[3], dZ[3];
  for (int c = 0; c < 3; ++c) {
    double sx = 0, sy = 0, sz = 0;
    for (int a = 0; a < 8; ++a) {
      sx += (a & 1) ? v[c][a] : -v[c][a];
      sy += (a & 2) ? v[c][a] : -v[c][a];
      sz += (a & 4) ? v[c][a] : -v[c][a];
    }
    dX[c] = 0.25 * sx;
    dY[c] = 0.25 * sy;
    dZ[c] = 0.25 * sz;
  }
  eps[0] = dX[0];
  eps[1] = dY[1];
  eps[2] = dZ[2];
  eps[3] = dZ[0] + dX[2];
  eps[4] = dZ[1] + dY[2];
  eps[5] = dY[0] + dX[1];
}

static __global__ void __launch_bounds__(256) stress_avg_kernel(GridDims G, JumpParams J, const int32_t* __restrict__ pix,
                                                         const double* __restrict__ cmod, int nphase,
                                                         const double* __restrict__ u, double* partial) {
  __shared__ double red[8];
  double acc[12];
  for (int t = 0; t < 12; ++t) acc[t] = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < G.ns;
       m += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    node_xyz(G, m, x, y, z);
    double eps[6];
    voxel_strain(G, J, u, x, y, z, eps);
    const int ph = pix[m];
    for (int r = 0; r < 6; ++r) {
      double s = 0.0;
      for (int c = 0; c < 6; ++c) s += cmod[E3D_IDX(ph, nphase) + (long long)nphase * (r + 6 * c)] * eps[c];
      acc[r] += s;
      acc[6 + r] += eps[r];
    }
  }
  for (int t = 0; t < 12; ++t) {
    const double s = block_sum<256>(acc[t], red);
    if (threadIdx.x == 0) partial[12 * (long long)blockIdx.x + t] = s;
  }
}

static __global__ void stress_field_kernel(GridDims G, JumpParams J, const int32_t* __restrict__ pix,
                                    const double* __restrict__ cmod, int nphase, const double* __restrict__ u,
                                    double* __restrict__ sigma, double* __restrict__ vm) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= G.ns) return;
  int x, y, z;
  node_xyz(G, m, x, y, z);
  double eps[6];
  voxel_strain(G, J, u, x, y, z, eps);
  const int ph = pix[m];
  double s6[6];
  for (int r = 0; r < 6; ++r) {
    double s = 0.0;
    for (int c = 0; c < 6; ++c) s += cmod[E3D_IDX(ph, nphase) + (long long)nphase * (r + 6 * c)] * eps[c];
    s6[r] = s;
    if (sigma) sigma[m + r * G.ns] = s;
  }
  if (vm) {
    const double a = s6[0] - s6[1], bq = s6[1] - s6[2], c = s6[2] - s6[0];
    vm[m] = sqrt(0.5 * (a * a + bq * bq + c * c + 6.0 * (s6[3] * s6[3] + s6[4] * s6[4] + s6[5] * s6[5])));
  }
}

// Phase B of a PCG iteration over tiles first, first + stride, ... < ntiles,
// node loop in tile order (no index division), U nodes of a column per thread
// in flight (the defaults keep one: more spill under the register cap):
// u -= lam h (unless UPD_U is false: the FP32 persistent kernel applies it in
// the next phase A), g -= lam Ah (+ tile-edge halos), z = Minv g
// (src/elas3dxtal_pcg.f90:1913-1932, symmetric Minv); returns this thread's
// share of z.g (FP32: summed per tile column in FP32, then in FP64).
template <typename T, int U = (sizeof(T) == 4 ? E3D_PB_UNROLL_F32 : E3D_PB_UNROLL_F64), bool UPD_U = true>
__device__ __forceinline__ double pcg_update_tiles(const GridDims& G, long long first, long long stride, T lam,
                                                   const T* __restrict__ hc, const T* __restrict__ Ah,
                                                   const T* __restrict__ hx, const T* __restrict__ hy,
                                                   const T* __restrict__ hd, const T* __restrict__ minv,
                                                   T* __restrict__ u, T* __restrict__ g, T* __restrict__ z) {
  const long long ns = G.ns;
  double zg_t = 0.0;
  const int tx = threadIdx.x % TILE_X, ty = threadIdx.x / TILE_X;
  const long long nxy = (long long)G.nx * G.ny;
  for (long long t = first; t < G.ntiles; t += stride) {
    const int tix = (int)(t % G.ntx);
    const int tiy = (int)((t / G.ntx) % G.nty);
    const int tiz = (int)(t / ((long long)G.ntx * G.nty));
    const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
    const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
    if (tx >= wx || ty >= wy) continue;
    const long long col = (long long)(x0 + tx) + (long long)G.nx * (y0 + ty);
    float zg32 = 0.f;  // FP32: this column's z.g, added to the FP64 sum once per tile
    for (int lz0 = 0; lz0 < wz; lz0 += U) {
      T ah[U][3], hv[U][3], uv[U][3], gv[U][3], mi[U][6];
#pragma unroll
      for (int j = 0; j < U; ++j) {
        if (lz0 + j < wz) {
          const long long m = E3D_IDX(col + nxy * (z0 + lz0 + j), ns);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            ah[j][c] = __ldcg(Ah + m + c * ns);
            if constexpr (UPD_U) {
              hv[j][c] = __ldcg(hc + m + c * ns);
              uv[j][c] = u[m + c * ns];
            }
            gv[j][c] = g[m + c * ns];
          }
#pragma unroll
          for (int q = 0; q < 6; ++q) mi[j][q] = __ldg(minv + m + q * ns);
        }
      }
#pragma unroll
      for (int j = 0; j < U; ++j) {
        if (lz0 + j < wz) {
          const long long m = E3D_IDX(col + nxy * (z0 + lz0 + j), ns);
          halo_add_tile<T>(G, hx, hy, hd, tix, tiy, tiz, tx, ty, lz0 + j, ah[j]);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            if constexpr (UPD_U) u[m + c * ns] = uv[j][c] - lam * hv[j][c];
            gv[j][c] = gv[j][c] - lam * ah[j][c];
            g[m + c * ns] = gv[j][c];
          }
          const T z0v = mi[j][0] * gv[j][0] + mi[j][3] * gv[j][1] + mi[j][4] * gv[j][2];
          const T z1v = mi[j][3] * gv[j][0] + mi[j][1] * gv[j][1] + mi[j][5] * gv[j][2];
          const T z2v = mi[j][4] * gv[j][0] + mi[j][5] * gv[j][1] + mi[j][2] * gv[j][2];
          z[m] = z0v;
          z[m + ns] = z1v;
          z[m + 2 * ns] = z2v;
          if constexpr (sizeof(T) == 4)
            zg32 += z0v * gv[j][0] + z1v * gv[j][1] + z2v * gv[j][2];
          else
            zg_t += (double)(z0v * gv[j][0] + z1v * gv[j][1] + z2v * gv[j][2]);
        }
      }
    }
    if constexpr (sizeof(T) == 4) zg_t += (double)zg32;
  }
  return zg_t;
}

// ---------------------------------------------------------------------------
// Phase B with its loads in flight through cp.async.  pcg_update_tiles keeps
// one node's loads in registers at a time (the register cap set by the stencil
// leaves nothing for more), so each thread waits a full memory latency per
// node.  Here every thread streams its node column through S shared-memory
// stages: the loads of plane lz + S - 1 are issued (cp.async, no registers held)
// before plane lz is consumed, so S planes' worth of bytes stay in flight per
// thread.  Each thread reads back only the slots it filled itself, so no block
// barrier is needed: cp.async.wait_group orders a thread's own copies.  The
// tile-edge halos (hx for lane 0 of each row, hy for row 0, hd for the corner
// node) travel in the same stages.  Same additions in the same order as
// pcg_update_tiles: the results are bitwise the same.
__device__ __forceinline__ void cp_async_4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
template <typename T>
__device__ __forceinline__ void cp_async_t(T* dst, const T* src) {
  if constexpr (sizeof(T) == 4)
    cp_async_4(dst, src);
  else
    cp_async_8(dst, src);
}

// Values of one stage: per thread Ah 3, g 3, Minv 6 (and h 3, u 3 when u is
// updated here), then the halo slots hx[3][TILE_Y], hy[3][TILE_X], hd[3].
template <bool UPD_U>
__host__ __device__ constexpr int pb_fields() {
  return UPD_U ? 18 : 12;
}
template <bool UPD_U>
__host__ __device__ constexpr int pb_stage_len() {
  return pb_fields<UPD_U>() * NT + 3 * TILE_Y + 3 * TILE_X + 3;
}
template <typename T, int S, bool UPD_U>
__host__ __device__ constexpr int pb_async_bytes() {
  return S * pb_stage_len<UPD_U>() * (int)sizeof(T);
}

template <typename T, int S, bool UPD_U = true>
__device__ __forceinline__ double pcg_update_tiles_async(const GridDims& G, long long first, long long stride, T lam,
                                                         const T* __restrict__ hc, const T* __restrict__ Ah,
                                                         const T* __restrict__ hx, const T* __restrict__ hy,
                                                         const T* __restrict__ hd, const T* __restrict__ minv,
                                                         T* __restrict__ u, T* __restrict__ g, T* __restrict__ z,
                                                         T* __restrict__ stages) {
  static_assert(S >= 2 && (S & (S - 1)) == 0, "stage count: a power of two");
  constexpr int F = pb_fields<UPD_U>();
  constexpr int SL = pb_stage_len<UPD_U>();
  const long long ns = G.ns;
  double zg_t = 0.0;
  const int tid = threadIdx.x;
  const int tx = tid % TILE_X, ty = tid / TILE_X;
  const long long nxy = (long long)G.nx * G.ny;
  const long long per_c = G.ntiles * G.tz;
  for (long long t = first; t < G.ntiles; t += stride) {
    const int tix = (int)(t % G.ntx);
    const int tiy = (int)((t / G.ntx) % G.nty);
    const int tiz = (int)(t / ((long long)G.ntx * G.nty));
    const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
    const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
    if (tx >= wx || ty >= wy) continue;
    const long long col = (long long)(x0 + tx) + (long long)G.nx * (y0 + ty);
    // halo sources (the tiles at -x, -y and -x-y), as in halo_add_tile
    const bool hxn = tx == 0, hyn = ty == 0;
    const int txl = tix == 0 ? G.ntx - 1 : tix - 1;
    const int tyd = tiy == 0 ? G.nty - 1 : tiy - 1;
    const long long plane = (long long)tiz * G.nty;
    const long long tX = (long long)txl + (long long)G.ntx * (tiy + plane);
    const long long tY = (long long)tix + (long long)G.ntx * (tyd + plane);
    const long long tD = (long long)txl + (long long)G.ntx * (tyd + plane);
    auto issue = [&](int lz) {
      T* d = stages + (lz & (S - 1)) * SL;
      const long long m = E3D_IDX(col + nxy * (z0 + lz), ns);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cp_async_t<T>(d + c * NT + tid, Ah + m + c * ns);
        cp_async_t<T>(d + (3 + c) * NT + tid, g + m + c * ns);
      }
#pragma unroll
      for (int q = 0; q < 6; ++q) cp_async_t<T>(d + (6 + q) * NT + tid, minv + m + q * ns);
      if constexpr (UPD_U) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          cp_async_t<T>(d + (12 + c) * NT + tid, hc + m + c * ns);
          cp_async_t<T>(d + (15 + c) * NT + tid, u + m + c * ns);
        }
      }
      T* hs = d + F * NT;
      if (hxn) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          cp_async_t<T>(hs + c * TILE_Y + ty, hx + E3D_IDX((c * per_c + tX * G.tz + lz) * TILE_Y + ty, 3 * per_c * TILE_Y));
      }
      if (hyn) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          cp_async_t<T>(hs + 3 * TILE_Y + c * TILE_X + tx,
                        hy + E3D_IDX((c * per_c + tY * G.tz + lz) * TILE_X + tx, 3 * per_c * TILE_X));
      }
      if (hxn && hyn) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          cp_async_t<T>(hs + 3 * TILE_Y + 3 * TILE_X + c, hd + E3D_IDX(c * per_c + tD * G.tz + lz, 3 * per_c));
      }
    };
#pragma unroll
    for (int j = 0; j < S - 1; ++j) {
      if (j < wz) issue(j);
      cp_async_commit();
    }
    float zg32 = 0.f;  // FP32: this column's z.g, added to the FP64 sum once per tile
    for (int lz = 0; lz < wz; ++lz) {
      if (lz + S - 1 < wz) issue(lz + S - 1);
      cp_async_commit();
      cp_async_wait<S - 1>();  // plane lz has landed
      const T* d = stages + (lz & (S - 1)) * SL;
      const T* hs = d + F * NT;
      T ah[3], gv[3], mi[6];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ah[c] = d[c * NT + tid];
        gv[c] = d[(3 + c) * NT + tid];
      }
#pragma unroll
      for (int q = 0; q < 6; ++q) mi[q] = d[(6 + q) * NT + tid];
      if (hxn) {
#pragma unroll
        for (int c = 0; c < 3; ++c) ah[c] += hs[c * TILE_Y + ty];
      }
      if (hyn) {
#pragma unroll
        for (int c = 0; c < 3; ++c) ah[c] += hs[3 * TILE_Y + c * TILE_X + tx];
      }
      if (hxn && hyn) {
#pragma unroll
        for (int c = 0; c < 3; ++c) ah[c] += hs[3 * TILE_Y + 3 * TILE_X + c];
      }
      const long long m = E3D_IDX(col + nxy * (z0 + lz), ns);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if constexpr (UPD_U) u[m + c * ns] = d[(15 + c) * NT + tid] - lam * d[(12 + c) * NT + tid];
        gv[c] = gv[c] - lam * ah[c];
        g[m + c * ns] = gv[c];
      }
      const T z0v = mi[0] * gv[0] + mi[3] * gv[1] + mi[4] * gv[2];
      const T z1v = mi[3] * gv[0] + mi[1] * gv[1] + mi[5] * gv[2];
      const T z2v = mi[4] * gv[0] + mi[5] * gv[1] + mi[2] * gv[2];
      z[m] = z0v;
      z[m + ns] = z1v;
      z[m + 2 * ns] = z2v;
      if constexpr (sizeof(T) == 4)
        zg32 += z0v * gv[0] + z1v * gv[1] + z2v * gv[2];
      else
        zg_t += (double)(z0v * gv[0] + z1v * gv[1] + z2v * gv[2]);
    }
    if constexpr (sizeof(T) == 4) zg_t += (double)zg32;
  }
  cp_async_wait<0>();
  return zg_t;
}

// u -= lam h over the owned nodes of tiles first, first + stride, ... (the same
// tile and column ownership as apply_tile and pcg_update_tiles).
template <typename T>
__device__ void flush_u_tiles(const GridDims& G, long long first, long long stride, T lam, const T* __restrict__ h,
                              T* __restrict__ u) {
  const long long ns = G.ns;
  const int tx = threadIdx.x % TILE_X, ty = threadIdx.x / TILE_X;
  const long long nxy = (long long)G.nx * G.ny;
  for (long long t = first; t < G.ntiles; t += stride) {
    const int tix = (int)(t % G.ntx);
    const int tiy = (int)((t / G.ntx) % G.nty);
    const int tiz = (int)(t / ((long long)G.ntx * G.nty));
    const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
    const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
    if (tx >= wx || ty >= wy) continue;
    const long long col = (long long)(x0 + tx) + (long long)G.nx * (y0 + ty);
    for (int lz = 0; lz < wz; ++lz) {
      const long long m = E3D_IDX(col + nxy * (z0 + lz), ns);
#pragma unroll
      for (int c = 0; c < 3; ++c) u[m + c * ns] = u[m + c * ns] - lam * __ldcg(h + m + c * ns);
    }
  }
}

// ---------------------------------------------------------------------------
// Persistent PCG (dembx_OpenMP main loop, src/elas3dxtal_pcg.f90:1574-2012).
// One cooperative launch runs up to it_limit iterations; every block keeps an
// identical copy of the scalars (each reduces the same partials in the same
// order), so only two grid barriers per iteration are needed:
//   A: h_new = z + gamma*h_old (or z), Ah = K h_new, partial h.Ah   | barrier
//      lambda = gg/hAh (guards :1899-1907)
//   B: u -= lambda h ; g -= lambda Ah ; z = Minv g ; partial z.g     | barrier
//      (FP32 per-thread-load form: u -= lambda h moves into the next A)
//      rel_res, divergence reset (:1961-1981), gamma (:1988), stop test (:2007)
struct PcgState {
  double gg, gg0, rel_res_prev, gamma, rel_res, tol, hAh, gglast;
  double rel_at_replace;  // mixed form: rel_res of the last FP64 residual (set-up or replacement)
  double refine_drop;     // mixed form: replace once rel_res < refine_drop * rel_at_replace (0: never)
  int it, status, reset, resets, cur, max_iter, divergence_reset, refinements;
  int since_replace, final_ready;  // final_ready: the job engine ended on a converged FP64 replacement
};

struct GridBarrier {
  unsigned int count;
  unsigned int gen;
};

// Grid-wide barrier for a cooperative launch.  Waits are bounded by a
// wall-clock limit (globaltimer) and an iteration cap; on expiry, or when
// another block has flagged an error, it returns false and the caller exits.
static __device__ bool grid_barrier(GridBarrier* gb, int* err, unsigned long long timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int* vgen = &gb->gen;
    const unsigned int g0 = *vgen;
    __threadfence();
    const unsigned int prev = atomicAdd(&gb->count, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      const unsigned long long t0 = global_timer_ns();
      unsigned long long spins = 0;
      while (*vgen == g0) {
        if (*(volatile int*)err != DEV_OK) {
          ok = 0;
          break;
        }
        __nanosleep(128);
        if (((++spins) & 255ull) == 0ull) {
          if (global_timer_ns() - t0 > timeout_ns || spins > (1ull << 34)) {
            atomicExch(err, DEV_TIMEOUT);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of n per-block partials in a fixed order, returned to every thread.
static __device__ double reduce_broadcast(const double* partial, int n, double* red) {
  __shared__ double s_val;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(partial + i);
  const double t = block_sum<NT>(s, red);
  if (threadIdx.x == 0) s_val = t;
  __syncthreads();
  return s_val;
}

// Dynamic shared memory of the per-thread-load persistent kernel: the phase-B
// cp.async stages (0 when phase B keeps its loads in registers).
template <typename T>
constexpr int pcg_dyn_smem_bytes() {
  constexpr bool defer_u = sizeof(T) == 4 && E3D_F32_DEFER_U != 0;
  constexpr int S = sizeof(T) == 4 ? E3D_PB_ASYNC_F32 : E3D_PB_ASYNC_F64;
  constexpr int pb = S > 0 ? pb_async_bytes<T, (S > 0 ? S : 2), !defer_u>() : 0;
  // phase A's staged table rows use the same bytes (the phases never overlap)
  constexpr int tab = (sizeof(T) == 4 && E3D_F32_TAB_ASYNC != 0) ? kTabAsyncBytes : 0;
  return pb > tab ? pb : tab;
}

// T = double: the plain FP64 solve (u is the solution).  T = float: the inner
// loop of the mixed-precision solve (u is the FP32 correction since the last
// FP64 residual replacement; stencil, preconditioner and vectors in FP32, dot
// products and scalar recurrences in FP64).
template <typename T>
struct PcgArgs {
  ApplyArgs<T> A;  // x / hnew / zv / gamma / reset set per iteration
  T* h0;
  T* h1;
  T* u;
  T* g;
  T* z;
  T* Ah;
  const T* minv;
  double* partA;  // [gridDim.x]
  double* partB;  // [gridDim.x]
  PcgState* st;
  double* history;
  GridBarrier* bar;
  int* err;
  int it_limit;
  unsigned long long timeout_ns;
  const PlaneMaps* maps;  // TMA form only
};

// TMA (FP32 only): phase A reads its node planes through the block's plane
// ring (dynamic shared memory of kRingSmemBytes).
template <typename T, bool TMA = false>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? (TMA && E3D_RING_ZS == 2 ? 1 : E3D_F32_BLOCKS_PER_SM) : 1)
    pcg_persistent_kernel(PcgArgs<T> P) {
  static_assert(!TMA || sizeof(T) == 4, "the plane ring feeds the FP32 stencil");
  using Smem = std::conditional_t<TMA, RingApplySmem<E3D_RING_ZS>, ApplySmem<T>>;
  __shared__ Smem sm;
  __shared__ double red[NT / 32];
  __shared__ PcgState S0;
  __shared__ uint64_t ring_bars[E3D_TMA_STAGES];
  __shared__ RingCursor ring_cur;
  PlaneRing ring;
  // per-thread-load form: phase B streams through cp.async stages in the
  // dynamic shared memory (pcg_update_tiles_async)
  constexpr int kPbStages = TMA ? 0 : (sizeof(T) == 4 ? E3D_PB_ASYNC_F32 : E3D_PB_ASYNC_F64);
  constexpr bool kTabAsync = sizeof(T) == 4 && !TMA && E3D_F32_TAB_ASYNC != 0;
  T* pb_stages = nullptr;
  float4* tab_slots = nullptr;
  {
    extern __shared__ __align__(128) unsigned char e3d_ring_smem[];
    if constexpr (TMA) ring_setup(ring, e3d_ring_smem, ring_bars, &ring_cur, P.maps, P.err, P.timeout_ns);
    if constexpr (kPbStages > 0) pb_stages = reinterpret_cast<T*>(e3d_ring_smem);
    if constexpr (kTabAsync) tab_slots = reinterpret_cast<float4*>(e3d_ring_smem);
  }
  // The PCG scalars live in shared memory: every thread reads them after a
  // barrier, thread 0 alone updates them (all blocks compute the same values
  // from the same partials), so they hold no registers during the sweeps.
  PcgState& s = S0;
  if (threadIdx.x == 0) s = *P.st;
  __syncthreads();
  if (s.status != PCG_RUNNING) return;
  const bool lead = threadIdx.x == 0;
  const GridDims& G = P.A.g;
  const int it_end = min(s.it + P.it_limit, s.max_iter);
  constexpr bool kDeferU = sizeof(T) == 4 && !TMA && E3D_F32_DEFER_U != 0;
  T lam_pending = T(0);  // kDeferU: du -= lam_pending * h_pending not yet applied
  const T* h_pending = nullptr;
  while (s.it < it_end) {
    // ---- phase A: fused direction update + stencil + h.Ah
    ApplyArgs<T> A = P.A;
    const int cur = s.cur;
    A.x = cur ? P.h1 : P.h0;
    A.hnew = cur ? P.h0 : P.h1;
    A.zv = P.z;
    A.y = P.Ah;
    A.gamma = (T)s.gamma;
    A.reset = s.reset;
    if constexpr (kDeferU) {
      A.du = P.u;
      A.lam_prev = lam_pending;
    }
    double hAh_t = 0.0;
    if constexpr (TMA) ring_begin(ring, G, cur ? P.maps->h1 : P.maps->h0, blockIdx.x, gridDim.x, G.ntiles);
    for (long long t = blockIdx.x; t < G.ntiles; t += gridDim.x) {
      if constexpr (TMA)
        apply_tile_ring<E3D_RING_ZS>(A, t, sm, hAh_t, ring);
      else
        apply_tile<T, true, (sizeof(T) == 4 && E3D_F32_POLD_SMEM != 0), kDeferU, kTabAsync>(A, t, sm, hAh_t,
                                                                                           tab_slots);
      __syncthreads();
    }
    {
      const double bs = block_sum<NT>(hAh_t, red);
      if (threadIdx.x == 0) P.partA[blockIdx.x] = bs;
    }
    if constexpr (TMA) fence_proxy_async_all();  // h_new stores before the next pass's TMA reads
    if (!grid_barrier(P.bar, P.err, P.timeout_ns)) {
      if (lead) s.status = PCG_TIMEOUT;
      break;
    }
    lam_pending = T(0);  // applied by this phase A
    const double hAh = reduce_broadcast(P.partA, gridDim.x, red);
    if (lead) {
      s.it += 1;
      s.cur ^= 1;
      s.hAh = hAh;
      if (!isfinite(hAh))
        s.status = PCG_BREAKDOWN;
      else if (fabs(hAh) < 1e-14)  // src/elas3dxtal_pcg.f90:1899-1902
        s.status = PCG_HAH;
    }
    __syncthreads();
    if (s.status != PCG_RUNNING) break;
    const double lambda = s.gg / hAh;
    const T lam = (T)lambda;
    // ---- phase B: u, g update, preconditioner, z.g -- node loop in tile order
    // (no index division); with kDeferU the u update waits for the next phase A.
    const T* hc = cur ? P.h0 : P.h1;  // the h_new of phase A
    constexpr int U = TMA ? E3D_PB_UNROLL_RING : (sizeof(T) == 4 ? E3D_PB_UNROLL_F32 : E3D_PB_UNROLL_F64);
    double zg_t;
    if constexpr (kPbStages > 0)
      zg_t = pcg_update_tiles_async<T, kPbStages, !kDeferU>(G, blockIdx.x, gridDim.x, lam, hc, P.Ah, P.A.hx, P.A.hy,
                                                            P.A.hd, P.minv, P.u, P.g, P.z, pb_stages);
    else
      zg_t = pcg_update_tiles<T, U, !kDeferU>(G, blockIdx.x, gridDim.x, lam, hc, P.Ah, P.A.hx, P.A.hy, P.A.hd,
                                              P.minv, P.u, P.g, P.z);
    if constexpr (kDeferU) {
      lam_pending = lam;
      h_pending = hc;
    }
    {
      const double bs = block_sum<NT>(zg_t, red);
      if (threadIdx.x == 0) P.partB[blockIdx.x] = bs;
    }
    if constexpr (TMA) fence_proxy_async_all();  // z stores before the next pass's TMA reads
    if (!grid_barrier(P.bar, P.err, P.timeout_ns)) {
      if (lead) s.status = PCG_TIMEOUT;
      break;
    }
    const double gg_new = reduce_broadcast(P.partB, gridDim.x, red);
    if (lead) {
      const double gglast = s.gg;
      s.gg = gg_new;
      s.gglast = gglast;
      if (!isfinite(gg_new)) {
        s.status = PCG_BREAKDOWN;
      } else {
        const double rel_res = sqrt(gg_new / s.gg0);
        s.rel_res = rel_res;
        if (blockIdx.x == 0 && P.history) P.history[E3D_IDX(s.it - 1, s.max_iter)] = rel_res;
        if (s.divergence_reset && rel_res > 10.0 * s.rel_res_prev && s.it > 1) {  // :1961-1981
          s.reset = 1;
          s.resets += 1;
        } else {
          s.gamma = gg_new / gglast;
          s.reset = 0;
        }
        s.rel_res_prev = rel_res;
        if (rel_res < s.tol)
          s.status = PCG_CONVERGED;
        else if (sizeof(T) == 4 && s.refine_drop > 0.0 && rel_res < s.refine_drop * s.rel_at_replace)
          s.status = PCG_REPLACE;  // the host replaces the residual in FP64 and relaunches
      }
    }
    __syncthreads();
    if (s.status != PCG_RUNNING) break;
  }
  __syncthreads();
  if (lead && s.status == PCG_RUNNING && s.it >= s.max_iter) s.status = PCG_MAXITER;
  // The last update is applied by the threads whose phase A wrote those du and
  // h values (same tile and column ownership), so no barrier is needed.
  if constexpr (kDeferU)
    if (lam_pending != T(0)) flush_u_tiles<T>(G, blockIdx.x, gridDim.x, lam_pending, h_pending, P.u);
  if constexpr (TMA) ring_drain(ring);
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.st = s;
}

// PCG set-up (src/elas3dxtal_pcg.f90:1527-1567): z = Minv g, partial z.g.
template <typename T>
__global__ void __launch_bounds__(256) pcg_init_kernel(GridDims G, const T* __restrict__ minv,
                                                       const T* __restrict__ g, T* __restrict__ z,
                                                       double* partial) {
  __shared__ double red[8];
  double acc = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < G.ns;
       m += (long long)gridDim.x * blockDim.x) {
    const T gv[3] = {g[m], g[m + G.ns], g[m + 2 * G.ns]};
    T zv[3];
    precond3<T>(minv, m, G.ns, gv, zv);
    for (int c = 0; c < 3; ++c) {
      z[m + c * G.ns] = zv[c];
      acc += (double)zv[c] * (double)gv[c];
    }
  }
  const double s = block_sum<256>(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

static __global__ void pcg_init_scalars_kernel(const double* __restrict__ partial, int n, double gg0_ref,
                                        int criterion, float tol, int max_iter, int divergence_reset,
                                        double refine_drop, PcgState* st) {
  __shared__ double red[8];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  const double gg = block_sum<256>(s, red);
  if (threadIdx.x == 0) {
    PcgState S;
    S.gg = gg;
    S.gg0 = (criterion == 1) ? gg : gg0_ref;
    S.rel_res_prev = sqrt(gg / S.gg0);
    S.rel_res = S.rel_res_prev;
    S.gamma = 0.0;
    S.tol = (double)tol;
    S.hAh = 0.0;
    S.gglast = gg;
    S.it = 0;
    S.status = PCG_RUNNING;
    S.reset = 1;  // h = z on the first step (:1554-1562)
    S.resets = 0;
    S.cur = 0;
    S.max_iter = max_iter;
    S.divergence_reset = divergence_reset;
    S.refinements = 0;
    S.since_replace = 0;
    S.final_ready = 0;
    S.rel_at_replace = S.rel_res_prev;
    S.refine_drop = refine_drop;
    *st = S;
  }
}

// ---------------------------------------------------------------------------
// Mixed precision: FP64 residual replacement between FP32 inner chunks.
// u64 += du32 ; du32 = 0 (the inner loop restarts its correction at zero).
static __global__ void fold_correction_kernel(long long n3, const float* __restrict__ du, double* __restrict__ u,
                                       float* __restrict__ du_zero) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  u[i] += (double)du[i];
  du_zero[i] = 0.0f;
}

// g = K u + b from the FP64 stencil (in-tile part + halos), stored in FP64 and
// FP32; then z32 = Minv32 g32 and partial z.g for the replaced residual.
static __global__ void __launch_bounds__(256) true_residual_kernel(GridDims G, const double* __restrict__ ku,
                                                            const double* __restrict__ hx,
                                                            const double* __restrict__ hy,
                                                            const double* __restrict__ hd,
                                                            const double* __restrict__ b, const float* __restrict__ minv32,
                                                            double* __restrict__ g64, float* __restrict__ g32,
                                                            float* __restrict__ z32, double* partial) {
  __shared__ double red[8];
  double acc = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < G.ns;
       m += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    node_xyz(G, m, x, y, z);
    double v[3] = {ku[m], ku[m + G.ns], ku[m + 2 * G.ns]};
    halo_add<double>(G, hx, hy, hd, x, y, z, v);
    float gv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long i = m + c * G.ns;
      const double gd = v[c] + b[i];
      g64[i] = gd;
      gv[c] = (float)gd;
      g32[i] = gv[c];
    }
    float zv[3];
    precond3<float>(minv32, m, G.ns, gv, zv);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      z32[m + c * G.ns] = zv[c];
      acc += (double)zv[c] * (double)gv[c];
    }
  }
  const double s = block_sum<256>(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Scalars after a residual replacement: gg from the true residual, gamma
// re-derived from it (the direction h is kept), and a convergence flag that
// only stands if the true residual also meets the tolerance.
static __global__ void replace_scalars_kernel(const double* __restrict__ partial, int n, PcgState* st,
                                       double* history) {
  __shared__ double red[8];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  const double gg = block_sum<256>(s, red);
  if (threadIdx.x == 0) {
    PcgState S = *st;
    S.gg = gg;
    S.refinements += 1;
    if (S.status == PCG_REPLACE) S.status = PCG_RUNNING;
    if (!isfinite(gg)) {
      S.status = PCG_BREAKDOWN;
    } else {
      const double rel = sqrt(gg / S.gg0);
      S.rel_res = rel;
      S.rel_res_prev = rel;
      S.rel_at_replace = rel;
      if (!S.reset) S.gamma = gg / S.gglast;
      if (history && S.it > 0) history[E3D_IDX(S.it - 1, S.max_iter)] = rel;
      if (S.status == PCG_CONVERGED && !(rel < S.tol)) S.status = PCG_RUNNING;
      if (S.status == PCG_RUNNING && rel < S.tol) S.status = PCG_CONVERGED;
    }
    *st = S;
  }
}

// g32 = (float) g64 at the start of a mixed solve.
static __global__ void to_float_kernel(long long n, const double* __restrict__ a, float* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

}  // namespace e3d
