// Job engine: many independent solves in one persistent launch.
//
// A job is one complete voxel-FE solve (one RVE under one macro-strain load
// case): periodic-jump force b and constant C (femat, src/elas3dxtal_pcg.f90:
// 815-1100), affine guess (:423-438), energy (:1107-1353), PCG (:1356-2043) with
// an FP32 inner loop and FP64 residual replacement, final energy and averaged
// stress (:2149-2408).  A job is executed by k "parts" (thread blocks): part p
// takes tiles p, p+k, ...; parts meet at job-local barriers and reduce through
// per-job partial slots, exactly as the single-problem kernel does across the
// whole grid.
//
// Scheduling: blocks pull parts from a global counter in order, so every part
// of a job is handed out before any part of the next job; with k <= the number
// of resident blocks no job can wait for a part that is never started.  Every
// wait is bounded (globaltimer limit); on expiry the job reports a timeout.
//
// Jobs are resumable: each keeps its stage and PCG scalars in global memory and
// a launch advances every unfinished job by at most `it_limit` iterations, so
// a host scheduler can run the engine in rounds and admit new jobs between
// rounds (continuous batching).
#pragma once
#include "e3d_kernels.cuh"

namespace e3d {

enum : int { JOB_NEW = 0, JOB_ITER = 1, JOB_DONE = 2 };

struct JobResult {
  int status;       // PCG_* at exit
  int iterations;
  int refinements;
  int resets;
  double utot0, utot, gg0, rel_res, true_rel, C;
  double strav[6], epsav[6];
};

struct JobDesc {
  GridDims G;
  JumpParams J;
  // shared per RVE (read only)
  const int32_t* pix;  // global phase ids, 0-based into the batch tables
  const float* cs32;   // [phase][24] packed upper triangle of C/16
  const double* cs64;  // [phase][kCsStride], modal_table
  const double* dk;    // [phase][576]
  const double* cmod;  // cmod(nphase_total,6,6), Fortran layout
  int nphase_total;
  const float* minv32;  // [6][ns] of the RVE
  // per job
  double* sig;  // [nphase_total][6]: each phase's stress under the job's macro strain (set-up scratch)
  double* u;
  double* g;
  double* b;
  float* du;
  float* g32;
  float* z32;
  float* h0;
  float* h1;
  float* Ah;
  double* hx;
  double* hy;
  double* hd;
  double* partial;  // [kJobSlots][nparts]
  GridBarrier* bar;
  PcgState* st;
  int* stage;
  JobResult* out;
  int nparts;
  int it_round;  // iterations per engine launch for this solve (0: the launch's it_limit)
  int max_iter;
  int refine_every;
  int criterion;
  int divergence_reset;
  float tol;
};

struct EngineArgs {
  const JobDesc* jobs;
  const int* part_job;   // part index -> job
  const int* part_rank;  // part index -> rank within its job
  int nparts_total;
  int njobs;
  unsigned int* head;    // dispenser
  int* err;
  int it_limit;          // iterations per job per launch
  unsigned long long timeout_ns;
};

// Barrier among the k parts of one job (same protocol as grid_barrier).
static __device__ bool job_barrier(GridBarrier* gb, unsigned int k, int* err, unsigned long long timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int* vgen = &gb->gen;
    const unsigned int g0 = *vgen;
    __threadfence();
    const unsigned int prev = atomicAdd(&gb->count, 1u);
    if (prev == k - 1) {
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

// Slots of the per-job partial array.
enum : int { SL_A = 0, SL_B = 1, SL_C = 2, SL_U = 3, SL_GG = 4, SL_ZG = 5, SL_S = 6 /* 6..17 */ };
constexpr int kJobSlots = 18;

// Sum of the k partials of slot `slot`, same value in every part.
static __device__ double job_reduce(const JobDesc& J, int slot, double* red) {
  return reduce_broadcast(J.partial + E3D_IDX((long long)slot * J.nparts, kJobSlots * (long long)J.nparts), J.nparts,
                          red);
}

static __device__ void job_put(const JobDesc& J, int slot, int part, double v, double* red) {
  const double s = block_sum<NT>(v, red);
  if (threadIdx.x == 0) J.partial[E3D_IDX((long long)slot * J.nparts + part, kJobSlots * (long long)J.nparts)] = s;
}

// Visits every node of the part's tiles in tile order: f(m, x, y, z, tix, tiy, tiz, lx, ly, lz).
template <typename F>
__device__ __forceinline__ void for_part_nodes(const JobDesc& J, int part, F&& f) {
  const GridDims& G = J.G;
  const int tx = threadIdx.x % TILE_X, ty = threadIdx.x / TILE_X;
  const long long nxy = (long long)G.nx * G.ny;
  for (long long t = part; t < G.ntiles; t += J.nparts) {
    const int tix = (int)(t % G.ntx);
    const int tiy = (int)((t / G.ntx) % G.nty);
    const int tiz = (int)(t / ((long long)G.ntx * G.nty));
    const int x0 = tix * TILE_X, y0 = tiy * TILE_Y, z0 = tiz * G.tz;
    const int wx = min(TILE_X, G.nx - x0), wy = min(TILE_Y, G.ny - y0), wz = min(G.tz, G.nz - z0);
    if (tx >= wx || ty >= wy) continue;
    const long long col = (long long)(x0 + tx) + (long long)G.nx * (y0 + ty);
    for (int lz = 0; lz < wz; ++lz)
      f(E3D_IDX(col + nxy * (z0 + lz), G.ns), x0 + tx, y0 + ty, z0 + lz, tix, tiy, tiz, tx, ty, lz);
  }
}

// b at node m: sum over its boundary elements of the row of K_e delta_e.
static __device__ __noinline__ void job_b_node(const JobDesc& J, int x, int y, int z, double (&acc)[3]) {
  const GridDims& G = J.G;
  acc[0] = acc[1] = acc[2] = 0.0;
  if (!(x == 0 || x == G.nx - 1 || y == 0 || y == G.ny - 1 || z == 0 || z == G.nz - 1)) return;
  for (int ra = 0; ra < 8; ++ra) {
    const int a = kRefToCorner[ra];
    const int ex = wrapi(x - (a & 1), G.nx), ey = wrapi(y - ((a >> 1) & 1), G.ny),
              ez = wrapi(z - ((a >> 2) & 1), G.nz);
    double d[8][3];
    bool any;
    element_delta(G, J.J, ex, ey, ez, d, any);
    if (!any) continue;
    const int ph = J.pix[E3D_IDX((long long)ex + (long long)G.nx * ey + (long long)G.nx * G.ny * ez, G.ns)];
    const double* D = J.dk + E3D_IDX(ph, J.nphase_total) * 576;
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int rb = 0; rb < 8; ++rb)
        for (int jj = 0; jj < 3; ++jj) s += D[(ra * 3 + i) * 24 + rb * 3 + jj] * d[rb][jj];
      acc[i] += s;
    }
  }
}

static __device__ __noinline__ double job_c_elem(const JobDesc& J, int x, int y, int z) {
  const GridDims& G = J.G;
  if (!(x == G.nx - 1 || y == G.ny - 1 || z == G.nz - 1)) return 0.0;
  double d[8][3];
  bool any;
  element_delta(G, J.J, x, y, z, d, any);
  const int ph = J.pix[E3D_IDX((long long)x + (long long)G.nx * y + (long long)G.nx * G.ny * z, G.ns)];
  const double* D = J.dk + E3D_IDX(ph, J.nphase_total) * 576;
  double e = 0.0;
  for (int r = 0; r < 24; ++r) {
    double s = 0.0;
    for (int c = 0; c < 24; ++c) s += D[r * 24 + c] * d[c / 3][c % 3];
    e += d[r / 3][r % 3] * s;
  }
  return 0.5 * e;
}

// Elements with a corner across a high face (i = nx-1, j = ny-1 or k = nz-1),
// each once, as femat_c_kernel enumerates them.
__device__ __forceinline__ long long boundary_element_count(const GridDims& G) {
  return (long long)G.ny * G.nz + (long long)(G.nx - 1) * G.nz + (long long)(G.nx - 1) * (G.ny - 1);
}

__device__ __forceinline__ void boundary_element(const GridDims& G, long long t, int& i, int& j, int& k) {
  const long long nfx = (long long)G.ny * G.nz, nfy = (long long)(G.nx - 1) * G.nz;
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
}

// Stress of every phase under the job's macro strain, sigma = cmod . eps
// (engineering shear), for the start gradient below.
static __device__ __noinline__ void job_phase_stress(const JobDesc& J, int part) {
  const double e[6] = {J.J.E[0][0], J.J.E[1][1], J.J.E[2][2], 2.0 * J.J.E[0][2], 2.0 * J.J.E[1][2], 2.0 * J.J.E[0][1]};
  const int np = J.nphase_total;
  for (long long ph = (long long)part * NT + threadIdx.x; ph < np; ph += (long long)J.nparts * NT) {
    for (int r = 0; r < 6; ++r) {
      double v = 0.0;
      for (int c = 0; c < 6; ++c) v += J.cmod[ph + (long long)np * (r + 6 * c)] * e[c];
      J.sig[E3D_IDX(6 * ph + r, 6LL * np)] = v;
    }
  }
}

// Start gradient g0 = K u_affine + b at node (x, y, z), in closed form.  The
// affine field E.x, continued across the periodic jumps, is E.x_e on every
// element e, whose first-order Walsh-Hadamard components are 4 eps and whose
// modal force is then the constant mode's sigma_e / 4 alone; back at the
// corners that is sigma_e . s / 4, s = +-1 per axis (+ on the element's high
// side).  Summed over the node's eight elements this is K u_affine + b exactly
// -- the interface forces of the piecewise-constant stress -- at about a
// quarter of a stencil pass's FP64 work and without the cancellation between
// K u_affine and b at the box faces.
static __device__ __forceinline__ void job_start_force(const JobDesc& J, int x, int y, int z, double (&g)[3]) {
  const GridDims& G = J.G;
  g[0] = g[1] = g[2] = 0.0;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int ox = a & 1, oy = (a >> 1) & 1, oz = (a >> 2) & 1;
    const int ex = wrapi(x - ox, G.nx), ey = wrapi(y - oy, G.ny), ez = wrapi(z - oz, G.nz);
    const int ph = J.pix[E3D_IDX((long long)ex + (long long)G.nx * ey + (long long)G.nx * G.ny * ez, G.ns)];
    const double* sg = J.sig + E3D_IDX(6LL * ph, 6LL * J.nphase_total);
    const double sx = ox ? 1.0 : -1.0, sy = oy ? 1.0 : -1.0, sz = oz ? 1.0 : -1.0;
    g[0] += sx * sg[0] + sy * sg[5] + sz * sg[3];
    g[1] += sx * sg[5] + sy * sg[1] + sz * sg[4];
    g[2] += sx * sg[3] + sy * sg[4] + sz * sg[2];
  }
  g[0] *= 0.25;
  g[1] *= 0.25;
  g[2] *= 0.25;
}

template <typename T>
__device__ ApplyArgs<T> job_apply_args(const JobDesc& J);

template <>
inline __device__ ApplyArgs<double> job_apply_args<double>(const JobDesc& J) {
  ApplyArgs<double> A{};
  A.g = J.G;
  A.pix = J.pix;
  A.cs = J.cs64;
  A.ncs = J.nphase_total;
  A.hx = J.hx;
  A.hy = J.hy;
  A.hd = J.hd;
  return A;
}

template <>
inline __device__ ApplyArgs<float> job_apply_args<float>(const JobDesc& J) {
  ApplyArgs<float> A{};
  A.g = J.G;
  A.pix = J.pix;
  A.cs = J.cs32;
  A.ncs = J.nphase_total;
  A.hx = reinterpret_cast<float*>(J.hx);
  A.hy = reinterpret_cast<float*>(J.hy);
  A.hd = reinterpret_cast<float*>(J.hd);
  return A;
}


// FP64 K u into g (in-tile part + halos), all parts, then a job barrier.  The
// apply arguments sit in shared memory (read there, not held in registers).
static __device__ __noinline__ void job_fp64_apply_tiles(const JobDesc& J, int part, ApplySmem<double>& sm) {
  __shared__ ApplyArgs<double> sA;
  if (threadIdx.x == 0) {
    ApplyArgs<double> A = job_apply_args<double>(J);
    A.x = J.u;
    A.y = J.g;
    sA = A;
  }
  __syncthreads();
  double dummy = 0.0;
  const long long nt = J.G.ntiles;
  const int np = J.nparts;
  for (long long t = part; t < nt; t += np) {
    apply_tile<double, false>(sA, t, sm, dummy);
    __syncthreads();
  }
}

static __device__ bool job_fp64_apply_u(const JobDesc& J, int part, ApplySmem<double>& sm, int* err,
                                 unsigned long long to) {
  job_fp64_apply_tiles(J, part, sm);
  return job_barrier(J.bar, J.nparts, err, to);
}

// After job_fp64_apply_u: g = Ku + b (+ halos), g32, z32 = Minv32 g32, partial z.g;
// optionally the energy terms.  Ends with a barrier.
static __device__ __noinline__ bool job_true_residual(const JobDesc& J, int part, bool energy, double* red, int* err,
                                  unsigned long long to) {
  const GridDims& G = J.G;
  const long long ns = G.ns;
  double zg = 0.0, eu = 0.0, gg = 0.0;
  for_part_nodes(J, part, [&](long long m, int, int, int, int tix, int tiy, int tiz, int lx, int ly, int lz) {
    double v[3] = {J.g[m], J.g[m + ns], J.g[m + 2 * ns]};
    halo_add_tile<double>(G, J.hx, J.hy, J.hd, tix, tiy, tiz, lx, ly, lz, v);
    float gv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long i = m + c * ns;
      const double bi = J.b[i];
      if (energy) eu += 0.5 * J.u[i] * v[c] + bi * J.u[i];
      const double gd = v[c] + bi;
      gg += gd * gd;
      J.g[i] = gd;
      gv[c] = (float)gd;
      J.g32[i] = gv[c];
    }
    float zv[3];
    precond3<float>(J.minv32, m, ns, gv, zv);
#pragma unroll
    for (int c = 0; c < 3; ++c) J.z32[m + c * ns] = zv[c];
    zg += (double)(zv[0] * gv[0] + zv[1] * gv[1] + zv[2] * gv[2]);
  });
  job_put(J, SL_ZG, part, zg, red);
  job_put(J, SL_U, part, eu, red);
  job_put(J, SL_GG, part, gg, red);
  return job_barrier(J.bar, J.nparts, err, to);
}

// The set-up's counterpart of job_true_residual: g already holds the whole
// start gradient K u + b (job_start_force), so g32, z32 and the partials of
// z.g, g.g and the energy terms u.(Ku)/2 + b.u = u.(g + b)/2 follow directly.
static __device__ __noinline__ bool job_start_residual(const JobDesc& J, int part, double* red, int* err,
                                                      unsigned long long to) {
  const long long ns = J.G.ns;
  double zg = 0.0, eu = 0.0, gg = 0.0;
  for_part_nodes(J, part, [&](long long m, int, int, int, int, int, int, int, int, int) {
    float gv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long i = m + c * ns;
      const double gd = J.g[i];
      eu += 0.5 * J.u[i] * (gd + J.b[i]);
      gg += gd * gd;
      gv[c] = (float)gd;
      J.g32[i] = gv[c];
    }
    float zv[3];
    precond3<float>(J.minv32, m, ns, gv, zv);
#pragma unroll
    for (int c = 0; c < 3; ++c) J.z32[m + c * ns] = zv[c];
    zg += (double)(zv[0] * gv[0] + zv[1] * gv[1] + zv[2] * gv[2]);
  });
  job_put(J, SL_ZG, part, zg, red);
  job_put(J, SL_U, part, eu, red);
  job_put(J, SL_GG, part, gg, red);
  return job_barrier(J.bar, J.nparts, err, to);
}

// One FP32 inner iteration's two sweeps, each kept out of line so that it gets
// its own register allocation rather than the engine kernel's.
// Fused direction update + stencil: returns this part's h.Ah.
#ifndef E3D_ENGINE_SWEEP_ATTR
#define E3D_ENGINE_SWEEP_ATTR __noinline__
#endif
#ifndef E3D_ENGINE_TAB_ASYNC
#define E3D_ENGINE_TAB_ASYNC 0  // stiffness rows staged one plane ahead (E3D_F32_TAB_ASYNC; slower there)
#endif
#ifndef E3D_ENGINE_POLD_SMEM
#define E3D_ENGINE_POLD_SMEM E3D_F32_POLD_SMEM  // lower node plane re-read from shared memory (1) or kept in registers (0)
#endif
#ifndef E3D_ENGINE_DEFER_U
#define E3D_ENGINE_DEFER_U 0  // du -= lam h of iteration k applied in phase A of k+1 (as E3D_F32_DEFER_U)
#endif
static __device__ E3D_ENGINE_SWEEP_ATTR double job_fp32_apply(const JobDesc& J, int part, float gamma, int reset, int cur,
                                                     float lam_prev, ApplySmem<float>& sm, float4* tab) {
  __shared__ ApplyArgs<float> sA;
  if (threadIdx.x == 0) {
    ApplyArgs<float> A = job_apply_args<float>(J);
    A.x = cur ? J.h1 : J.h0;
    A.hnew = cur ? J.h0 : J.h1;
    A.zv = J.z32;
    A.y = J.Ah;
    A.gamma = gamma;
    A.reset = reset;
    A.du = J.du;
    A.lam_prev = lam_prev;
    sA = A;
  }
  __syncthreads();
  double hAh = 0.0;
  const long long nt = J.G.ntiles;
  const int np = J.nparts;
  for (long long t = part; t < nt; t += np) {
    apply_tile<float, true, E3D_ENGINE_POLD_SMEM != 0, E3D_ENGINE_DEFER_U != 0, E3D_ENGINE_TAB_ASYNC != 0>(sA, t, sm,
                                                                                                         hAh, tab);
    __syncthreads();
  }
  return hAh;
}

// Phase-B planes in flight per thread through cp.async stages in the engine's
// dynamic shared memory (0: the one-node register form).
#ifndef E3D_ENGINE_PB_ASYNC
#define E3D_ENGINE_PB_ASYNC 2
#endif
constexpr int kEnginePbBytes =
    E3D_ENGINE_PB_ASYNC > 0 ? pb_async_bytes<float, (E3D_ENGINE_PB_ASYNC > 0 ? E3D_ENGINE_PB_ASYNC : 2), true>() : 0;
// the FP32 stencil's staged table rows share these bytes (the sweeps never overlap)
constexpr int kEngineDynSmem = (E3D_ENGINE_TAB_ASYNC && kTabAsyncBytes > kEnginePbBytes) ? kTabAsyncBytes : kEnginePbBytes;

// du -= lam h, g -= lam Ah, z = Minv g: returns this part's z.g.
static __device__ __noinline__ double job_fp32_update(const JobDesc& J, int part, float lam, int cur, float* stages) {
  if constexpr (E3D_ENGINE_PB_ASYNC > 0)
    return pcg_update_tiles_async<float, E3D_ENGINE_PB_ASYNC, E3D_ENGINE_DEFER_U == 0>(
        J.G, part, J.nparts, lam, cur ? J.h0 : J.h1, J.Ah, reinterpret_cast<const float*>(J.hx),
        reinterpret_cast<const float*>(J.hy), reinterpret_cast<const float*>(J.hd), J.minv32, J.du, J.g32, J.z32,
        stages);
  else
    return pcg_update_tiles<float, E3D_PB_UNROLL_F32, E3D_ENGINE_DEFER_U == 0>(J.G, part, J.nparts, lam,
                                                                                 cur ? J.h0 : J.h1, J.Ah,
                                   reinterpret_cast<const float*>(J.hx), reinterpret_cast<const float*>(J.hy),
                                   reinterpret_cast<const float*>(J.hd), J.minv32, J.du, J.g32, J.z32);
}

static __device__ void job_fold(const JobDesc& J, int part) {
  const long long ns = J.G.ns;
  for_part_nodes(J, part, [&](long long m, int, int, int, int, int, int, int, int, int) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long i = m + c * ns;
      J.u[i] += (double)J.du[i];
      J.du[i] = 0.0f;
    }
  });
}

// Residual drop after which the job engine replaces the FP32 recurrence's
// residual with an FP64 one (see the replacement step below).
#ifndef E3D_ENGINE_REFINE_DROP
#define E3D_ENGINE_REFINE_DROP 1e-3
#endif
constexpr double kRefineDrop = E3D_ENGINE_REFINE_DROP;

#ifndef E3D_ENGINE_BLOCKS_PER_SM
// Resident engine blocks per SM.  One block keeps the whole 255-register budget,
// so neither the FP32 nor the FP64 sweep spills: with the phase B in cp.async
// stages that beats two 128-register blocks (batch 8.35 vs 9.38 s).
#define E3D_ENGINE_BLOCKS_PER_SM 1
#endif
// The part's job descriptor and PCG scalars live in shared memory: thread 0
// writes them, every thread reads them after a barrier, so neither occupies
// registers during the sweeps.
static __global__ void __launch_bounds__(NT, E3D_ENGINE_BLOCKS_PER_SM) job_engine_kernel(EngineArgs E) {
  static_assert(sizeof(ApplySmem<float>) <= sizeof(ApplySmem<double>), "the FP32 tile shares the FP64 tile's memory");
  __shared__ __align__(16) unsigned char smraw[sizeof(ApplySmem<double>)];
  __shared__ double red[NT / 32];
  __shared__ int s_idx, s_part;
  __shared__ JobDesc sJ;
  __shared__ PcgState sS;
  extern __shared__ __align__(128) unsigned char e3d_engine_dyn[];
  float* pb_stages = reinterpret_cast<float*>(e3d_engine_dyn);  // kEngineDynSmem bytes
  ApplySmem<double>& sm64 = *reinterpret_cast<ApplySmem<double>*>(smraw);
  ApplySmem<float>& sm32 = *reinterpret_cast<ApplySmem<float>*>(smraw);
  const unsigned long long to = E.timeout_ns;
  const bool lead = threadIdx.x == 0;
  const JobDesc& J = sJ;
  PcgState& s = sS;
  for (;;) {
    __syncthreads();  // the previous part is done with sJ / sS
    if (lead) {
      const int idx = (int)atomicAdd(E.head, 1u);
      s_idx = idx;
      if (idx < E.nparts_total) {
        sJ = E.jobs[E3D_IDX(E.part_job[idx], E.njobs)];
        s_part = E.part_rank[idx];
      }
    }
    __syncthreads();
    if (s_idx >= E.nparts_total) break;
    const int part = s_part;
    const GridDims& G = J.G;
    const long long ns = G.ns;
    if (*(volatile int*)J.stage == JOB_DONE) continue;  // finished in an earlier launch (all parts agree)
    bool ok = true;
    // ---------------- set-up: b, C, affine u, energy, z, scalars
    if (*(volatile int*)J.stage == JOB_NEW) {
      double cpart = 0.0;
      const double exx = J.J.E[0][0], eyy = J.J.E[1][1], ezz = J.J.E[2][2];
      const double exy = J.J.E[0][1], exz = J.J.E[0][2], eyz = J.J.E[1][2];
      job_phase_stress(J, part);
      ok = job_barrier(J.bar, J.nparts, E.err, to);
      if (ok)
        for_part_nodes(J, part, [&](long long m, int x, int y, int z, int, int, int, int, int, int) {
          if (!(x == 0 || x == G.nx - 1 || y == 0 || y == G.ny - 1 || z == 0 || z == G.nz - 1))
            J.b[m] = J.b[m + ns] = J.b[m + 2 * ns] = 0.0;  // boundary nodes: below
          const double xd = x, yd = y, zd = z;
          J.u[m] = xd * exx + yd * exy + zd * exz;
          J.u[m + ns] = xd * exy + yd * eyy + zd * eyz;
          J.u[m + 2 * ns] = xd * exz + yd * eyz + zd * ezz;
          J.du[m] = J.du[m + ns] = J.du[m + 2 * ns] = 0.0f;
          double g0[3];
          job_start_force(J, x, y, z, g0);
          J.g[m] = g0[0];
          J.g[m + ns] = g0[1];
          J.g[m + 2 * ns] = g0[2];
        });
      // b at the boundary nodes and C over the boundary elements, both listed
      // compactly and shared by all threads of all parts
      const long long stride = (long long)J.nparts * NT, first = (long long)part * NT + threadIdx.x;
      const long long nbn = boundary_node_count(G);
      for (long long t = first; t < nbn; t += stride) {
        int x, y, z;
        boundary_node(G, t, x, y, z);
        double bb[3];
        job_b_node(J, x, y, z, bb);
        const long long m = E3D_IDX((long long)x + (long long)G.nx * y + (long long)G.nx * G.ny * z, ns);
        J.b[m] = bb[0];
        J.b[m + ns] = bb[1];
        J.b[m + 2 * ns] = bb[2];
      }
      const long long nbe = boundary_element_count(G);
      for (long long t = first; t < nbe; t += stride) {
        int i, j, k;
        boundary_element(G, t, i, j, k);
        cpart += job_c_elem(J, i, j, k);
      }
      job_put(J, SL_C, part, cpart, red);
      if (ok) ok = job_barrier(J.bar, J.nparts, E.err, to);
      if (ok) ok = job_start_residual(J, part, red, E.err, to);
      if (ok) {
        const double C = job_reduce(J, SL_C, red);
        const double U0 = C + job_reduce(J, SL_U, red);
        const double gg0 = job_reduce(J, SL_GG, red);
        const double gg = job_reduce(J, SL_ZG, red);
        if (lead) {
          s = PcgState{};
          s.gg = gg;
          s.gg0 = (J.criterion == 1) ? gg : gg0;
          s.rel_res_prev = sqrt(gg / s.gg0);
          s.rel_res = s.rel_res_prev;
          s.gamma = 0.0;
          s.tol = (double)J.tol;
          s.hAh = 0.0;
          s.gglast = gg;
          s.it = 0;
          s.status = PCG_RUNNING;
          s.reset = 1;
          s.resets = 0;
          s.cur = 0;
          s.max_iter = J.max_iter;
          s.divergence_reset = J.divergence_reset;
          s.refinements = 0;
          s.since_replace = 0;
          s.rel_at_replace = s.rel_res_prev;
          if (part == 0) {
            J.out->C = C;
            J.out->utot0 = U0;
            J.out->gg0 = gg0;
          }
        }
      }
    } else if (lead) {
      s = *J.st;  // resume
    }
    __syncthreads();
    // ---------------- FP32 inner iterations with FP64 residual replacement
    const int R = J.refine_every > 0 ? J.refine_every : 50;
    const int it_end = min(s.it + (J.it_round > 0 ? J.it_round : E.it_limit), s.max_iter);
    // E3D_ENGINE_DEFER_U: du -= lam_pending * h_pending is still owed; the next
    // phase A applies it, or flush_pending before du is read or the job yields
    float lam_pending = 0.f;
    const float* h_pending = nullptr;
    auto flush_pending = [&]() {
      if (E3D_ENGINE_DEFER_U && lam_pending != 0.f) flush_u_tiles<float>(G, part, J.nparts, lam_pending, h_pending, J.du);
      lam_pending = 0.f;
    };
    while (ok && s.status == PCG_RUNNING && s.it < it_end) {
      const int cur = s.cur;
      const double hAh_t = job_fp32_apply(J, part, (float)s.gamma, s.reset, cur, lam_pending, sm32,
                                          reinterpret_cast<float4*>(e3d_engine_dyn));
      lam_pending = 0.f;  // applied by this phase A
      job_put(J, SL_A, part, hAh_t, red);
      if (!(ok = job_barrier(J.bar, J.nparts, E.err, to))) break;
      const double hAh = job_reduce(J, SL_A, red);
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
      const float lam = (float)(s.gg / hAh);
      const double zg = job_fp32_update(J, part, lam, cur, pb_stages);
      if (E3D_ENGINE_DEFER_U) {
        lam_pending = lam;
        h_pending = cur ? J.h0 : J.h1;  // the h_new of this iteration's phase A
      }
      job_put(J, SL_B, part, zg, red);
      if (!(ok = job_barrier(J.bar, J.nparts, E.err, to))) break;
      const double gg_new = job_reduce(J, SL_B, red);
      if (lead) {
        const double gglast = s.gg;
        s.gg = gg_new;
        s.gglast = gglast;
        if (!isfinite(gg_new)) {
          s.status = PCG_BREAKDOWN;
        } else {
          const double rel = sqrt(gg_new / s.gg0);
          s.rel_res = rel;
          if (s.divergence_reset && rel > 10.0 * s.rel_res_prev && s.it > 1) {  // :1961-1981
            s.reset = 1;
            s.resets += 1;
          } else {
            s.gamma = gg_new / gglast;
            s.reset = 0;
          }
          s.rel_res_prev = rel;
          if (rel < s.tol) s.status = PCG_CONVERGED;
          s.since_replace += 1;
        }
      }
      __syncthreads();
      if (s.status == PCG_BREAKDOWN) break;
      // FP64 residual replacement when the FP32 loop meets the stop test, every R
      // iterations at most, and whenever the FP32 recurrence has driven its
      // residual kRefineDrop below the last FP64 one.  The drop rule is what keeps
      // a long period safe: with a replacement only every 200 iterations (about
      // four decades of residual under the true-residual stop), 147 of the 1536
      // batch solves stalled at the iteration cap; with the drop rule at 1e-3 all
      // converge in the same iterations as with one every 50, and the batch runs
      // at 64 instead of 50 solves/s (1e-2: 63; under the reference stop, which
      // ends within about two decades, 1e-3 adds no replacement and 1e-2 adds one)
      if (s.status == PCG_CONVERGED || s.since_replace >= R || s.rel_res < kRefineDrop * s.rel_at_replace) {
        // FP64 residual replacement: u += du, g = K u + b, restart the FP32 recurrence
        flush_pending();
        job_fold(J, part);
        if (!(ok = job_barrier(J.bar, J.nparts, E.err, to))) break;
        if (!(ok = job_fp64_apply_u(J, part, sm64, E.err, to))) break;
        // energy terms too: if this replacement ends the solve, the final
        // stage reuses them instead of another FP64 pass over the same u
        if (!(ok = job_true_residual(J, part, true, red, E.err, to))) break;
        const double ggt = job_reduce(J, SL_ZG, red);
        if (lead) {
          s.gg = ggt;
          s.refinements += 1;
          s.since_replace = 0;
          if (!isfinite(ggt)) {
            s.status = PCG_BREAKDOWN;
          } else {
            const double relt = sqrt(ggt / s.gg0);
            s.rel_res = relt;
            s.rel_res_prev = relt;
            s.rel_at_replace = relt;
            if (!s.reset) s.gamma = ggt / s.gglast;
            s.status = (relt < s.tol) ? PCG_CONVERGED : PCG_RUNNING;
            s.final_ready = s.status == PCG_CONVERGED;  // u, g and the energy slots are final
          }
        }
        __syncthreads();
      }
    }
    flush_pending();  // the part's own nodes, as phase A owns them: no barrier needed before the fold
    __syncthreads();
    if (lead) {
      if (!ok) s.status = PCG_TIMEOUT;
      if (ok && s.status == PCG_RUNNING && s.it >= s.max_iter) s.status = PCG_MAXITER;
    }
    __syncthreads();
    const bool finished = s.status != PCG_RUNNING;
    if (ok && !finished) {
      // out of iteration budget for this launch: persist and yield
      if (!(ok = job_barrier(J.bar, J.nparts, E.err, to)) && lead) s.status = PCG_TIMEOUT;
      if (part == 0 && lead) {
        *J.st = s;
        *J.stage = ok ? JOB_ITER : JOB_DONE;
        if (!ok) J.out->status = PCG_TIMEOUT;
      }
      continue;
    }
    // ---------------- final: u += du, FP64 energy, true residual, averaged stress
    // (the first three already done when the solve ended in a replacement)
    const bool fresh = s.status == PCG_CONVERGED && s.final_ready;
    if (ok && !fresh) {
      job_fold(J, part);
      ok = job_barrier(J.bar, J.nparts, E.err, to);
    }
    if (ok && !fresh) ok = job_fp64_apply_u(J, part, sm64, E.err, to);
    if (ok && !fresh) ok = job_true_residual(J, part, true, red, E.err, to);
    double sacc[12];
    for (int q = 0; q < 12; ++q) sacc[q] = 0.0;
    if (ok) {
      for_part_nodes(J, part, [&](long long m, int x, int y, int z, int, int, int, int, int, int) {
        double eps[6];
        voxel_strain(G, J.J, J.u, x, y, z, eps);
        const int ph = J.pix[m];
        for (int r = 0; r < 6; ++r) {
          double sv = 0.0;
          for (int c = 0; c < 6; ++c) sv += J.cmod[ph + (long long)J.nphase_total * (r + 6 * c)] * eps[c];
          sacc[r] += sv;
          sacc[6 + r] += eps[r];
        }
      });
      for (int q = 0; q < 12; ++q) job_put(J, SL_S + q, part, sacc[q], red);
      ok = job_barrier(J.bar, J.nparts, E.err, to);
    }
    if (ok) {
      const double C = J.out->C;
      const double U = C + job_reduce(J, SL_U, red);
      const double gg = job_reduce(J, SL_GG, red);
      double tot[12];
      for (int q = 0; q < 12; ++q) tot[q] = job_reduce(J, SL_S + q, red);
      if (part == 0 && lead) {
        J.out->utot = U;
        J.out->true_rel = sqrt(gg / J.out->gg0);
        for (int r = 0; r < 6; ++r) {
          J.out->strav[r] = tot[r] / (double)ns;
          J.out->epsav[r] = tot[6 + r] / (double)ns;
        }
      }
    } else if (lead) {
      s.status = PCG_TIMEOUT;
    }
    if (part == 0 && lead) {
      J.out->status = s.status;
      J.out->iterations = s.it;
      J.out->refinements = s.refinements;
      J.out->resets = s.resets;
      J.out->rel_res = s.rel_res;
      *J.st = s;
      *J.stage = JOB_DONE;
    }
  }
}

// Clears the job barriers (and, for a fresh solve, the stages) of n jobs.
static __global__ void reset_jobs_kernel(const JobDesc* __restrict__ jobs, int n, int reset_stage) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  jobs[j].bar->count = 0u;
  jobs[j].bar->gen = 0u;
  if (reset_stage) *jobs[j].stage = JOB_NEW;
}

// Phase tables for a batch: per phase its own material (per-RVE C11/C12/C44
// and orientation).  Same arithmetic as femat_phase_kernel.
struct PhaseMat {
  double c11, c12, c44;
  double r[3];
  int pore;  // 1: inclusion phase (K1, G1)
  double K1, G1;
};

static __global__ void batch_phase_kernel(const PhaseMat* __restrict__ mats, int nphase_total, double* __restrict__ cmod,
                                          double* __restrict__ cs, float* __restrict__ cs32, double* __restrict__ dk,
                                          double* __restrict__ dkd) {
  const int p = blockIdx.x;
  __shared__ double csh[kCsStride];
  __shared__ double col[24][24];
  if (threadIdx.x == 0) {
    const PhaseMat M = mats[p];
    double C6[6][6];
    if (M.pore) {
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
          const double ck = (i < 3 && j < 3) ? 1.0 : 0.0;
          double cmu = 0.0;
          if (i < 3 && j < 3) cmu = (i == j) ? 4.0 / 3.0 : -2.0 / 3.0;
          if (i >= 3 && i == j) cmu = 1.0;
          C6[i][j] = M.K1 * ck + M.G1 * cmu;
        }
    } else {
      bond_rotate(M.r, M.c11, M.c12, M.c44, C6);
    }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) cmod[p + (long long)nphase_total * (i + 6 * j)] = C6[i][j];
    modal_table(C6, csh);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kCsStride; i += blockDim.x) cs[(long long)p * kCsStride + i] = csh[i];
  for (int r = threadIdx.x; r < 6; r += blockDim.x)  // FP32: upper triangle of C/16
    for (int c = r; c < 6; ++c) cs32[(long long)p * kCs32Stride + sym6(r, c)] = (float)csh[6 * r + c];
  for (int i = 21 + threadIdx.x; i < kCs32Stride; i += blockDim.x) cs32[(long long)p * kCs32Stride + i] = 0.f;
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
  for (int e = threadIdx.x; e < 576; e += blockDim.x) {
    const int r = e / 24, c = e % 24;
    const double v = (r <= c) ? col[c][r] : col[r][c];
    dk[(long long)p * 576 + e] = v;
    const int ra = r / 3, i = r % 3, cb = c / 3, j = c % 3;
    if (ra == cb) dkd[(long long)p * 72 + ra * 9 + i * 3 + j] = v;
  }
}

}  // namespace e3d
