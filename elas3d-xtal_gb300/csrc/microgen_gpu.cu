// GPU back end of the synthetic-microstructure generator (include/e3d_micro.h).
//
// Grains: the host builds the plan (seeds, orientations, per-voxel-block
// candidate lists; microgen.cpp); one thread block per voxel block stages its
// candidates in shared memory and every thread finds the nearest seed of its
// voxels.  The distance arithmetic is written with explicitly rounded
// operations in the host's order (no contraction), and candidates are scanned
// in ascending grain id with a strict '<', so the phase ids are bitwise those
// of e3d_micro_grains.
//
// Pores: drawn on the host from the same random stream as the host loops
// (PoreStream) and painted by one thread block in order; after each pore the
// block counts the voxels it newly set (atomic exchange, so a voxel reached
// through two periodic images counts once) and stops at the pore that reaches
// the target fraction -- the host loop's stopping rule.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "e3d_micro.h"
#include "microgen_plan.h"
#include "e3d_trace.h"

void e3d_record_cuda_error(const char* what, cudaError_t e);

using namespace e3d_micro;

namespace {

constexpr int kCandCache = 512;  // candidates staged in shared memory per voxel block

struct GrainDev {
  int nx, ny, nz, ngrains, B, nb0, nb1;
  double L0, L1, L2;
  const int64_t* off;
  const uint8_t* brute;
  const int32_t* cg;
  const double* cx;
  const double* cy;
  const double* cz;
  const double* sx;
  const double* sy;
  const double* sz;
  const double* w;
};

__device__ __forceinline__ double wrap_rn(double d, double L) {
  if (d > 0.5 * L) d = __dsub_rn(d, L);
  if (d < -0.5 * L) d = __dadd_rn(d, L);
  return d;
}

// dx*dx + dy*dy + dz*dz - w, left to right, each operation rounded once.
__device__ __forceinline__ double pdist_rn(double dx, double dy, double dz, double w) {
  return __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), w);
}

__global__ void __launch_bounds__(256) grain_assign_kernel(GrainDev D, int32_t* __restrict__ pix, int* err) {
  __shared__ int32_t s_g[kCandCache];
  __shared__ double s_x[kCandCache], s_y[kCandCache], s_z[kCandCache], s_w[kCandCache];
  const long long blk = blockIdx.x;
  const int bi = (int)(blk % D.nb0), bj = (int)((blk / D.nb0) % D.nb1), bk = (int)(blk / ((long long)D.nb0 * D.nb1));
  const int i0 = bi * D.B, j0 = bj * D.B, k0 = bk * D.B;
  const int wi = min(D.nx, i0 + D.B) - i0, wj = min(D.ny, j0 + D.B) - j0, wk = min(D.nz, k0 + D.B) - k0;
  const long long c0 = D.off[blk], nc = D.off[blk + 1] - c0;
  const bool brute = D.brute[blk] != 0;
  const bool cached = !brute && nc <= kCandCache;
  if (cached) {
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
      const int g = D.cg[c0 + t];
      s_g[t] = g;
      s_x[t] = D.cx[c0 + t];
      s_y[t] = D.cy[c0 + t];
      s_z[t] = D.cz[c0 + t];
      s_w[t] = D.w[g];
    }
  }
  __syncthreads();
  const int vol = wi * wj * wk;
  for (int v = threadIdx.x; v < vol; v += blockDim.x) {
    const int i = i0 + v % wi, j = j0 + (v / wi) % wj, k = k0 + v / (wi * wj);
    const double px = i + 0.5, py = j + 0.5, pz = k + 0.5;
    double best = 1e300;
    int bg;
    if (brute) {
      bg = 0;
      for (int g = 0; g < D.ngrains; ++g) {
        const double d = pdist_rn(wrap_rn(__dsub_rn(D.sx[g], px), D.L0), wrap_rn(__dsub_rn(D.sy[g], py), D.L1),
                                  wrap_rn(__dsub_rn(D.sz[g], pz), D.L2), D.w[g]);
        if (d < best) {
          best = d;
          bg = g;
        }
      }
    } else if (cached) {
      bg = -1;
      for (int t = 0; t < nc; ++t) {
        const double d = pdist_rn(__dsub_rn(s_x[t], px), __dsub_rn(s_y[t], py), __dsub_rn(s_z[t], pz), s_w[t]);
        if (d < best) {
          best = d;
          bg = s_g[t];
        }
      }
    } else {
      bg = -1;
      for (long long t = c0; t < c0 + nc; ++t) {
        const int g = D.cg[t];
        const double d = pdist_rn(__dsub_rn(D.cx[t], px), __dsub_rn(D.cy[t], py), __dsub_rn(D.cz[t], pz), D.w[g]);
        if (d < best) {
          best = d;
          bg = g;
        }
      }
    }
    if (bg < 0) atomicExch(err, 1);
    pix[(long long)i + (long long)D.nx * ((long long)j + (long long)D.ny * k)] = bg + 1;
  }
}

__global__ void count_phase_kernel(long long ns, const int32_t* __restrict__ pix, int32_t phase,
                                   unsigned long long* count) {
  unsigned long long c = 0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < ns; m += (long long)gridDim.x * blockDim.x)
    c += pix[m] == phase;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

constexpr int kPaintThreads = 1024;

// Paints pores[0..n) in order; state[0] = count, state[1] = pores used,
// state[2] = 1 once the count reached the target.
__global__ void __launch_bounds__(kPaintThreads) pore_paint_kernel(const PoreShape* __restrict__ pores, int n, int nx,
                                                                   int ny, int nz, int32_t pore_phase, double target,
                                                                   int32_t* __restrict__ pix, long long* state) {
  __shared__ unsigned int s_add[kPaintThreads / 32];
  __shared__ int s_done;
  long long count = state[0];
  if (threadIdx.x == 0) s_done = 0;
  __syncthreads();
  int used = 0;
  for (int p = 0; p < n; ++p) {
    const PoreShape& P = pores[p];
    const int bx = P.i1 - P.i0 + 1, by = P.j1 - P.j0 + 1, bz = P.k1 - P.k0 + 1;
    const long long nbox = (long long)bx * by * bz;
    unsigned int added = 0;
    for (long long v = threadIdx.x; v < nbox; v += kPaintThreads) {
      const int i = P.i0 + (int)(v % bx), j = P.j0 + (int)((v / bx) % by), k = P.k0 + (int)(v / ((long long)bx * by));
      const double d0 = __dsub_rn(i + 0.5, P.c[0]), d1 = __dsub_rn(j + 0.5, P.c[1]), d2 = __dsub_rn(k + 0.5, P.c[2]);
      double q = 0.0;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const double t =
            __dadd_rn(__dadd_rn(__dmul_rn(P.A[r][0], d0), __dmul_rn(P.A[r][1], d1)), __dmul_rn(P.A[r][2], d2));
        q = __dadd_rn(q, __dmul_rn(t, t));
      }
      if (q > 1.0) continue;
      const int ii = ((i % nx) + nx) % nx, jj = ((j % ny) + ny) % ny, kk = ((k % nz) + nz) % nz;
      const int32_t old = atomicExch(pix + (long long)ii + (long long)nx * ((long long)jj + (long long)ny * kk),
                                     pore_phase);
      added += old != pore_phase;
    }
    for (int o = 16; o > 0; o >>= 1) added += __shfl_down_sync(0xffffffffu, added, o);
    if ((threadIdx.x & 31) == 0) s_add[threadIdx.x >> 5] = added;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long a = 0;
      for (int wv = 0; wv < kPaintThreads / 32; ++wv) a += s_add[wv];
      count += a;
      if (!((double)count < target)) s_done = 1;
    }
    __syncthreads();
    used = p + 1;
    if (s_done) break;
  }
  if (threadIdx.x == 0) {
    state[0] = count;
    state[1] += used;
    state[2] = s_done;
  }
}

#define MG_CUDA(call)                          \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) {                   \
      e3d_record_cuda_error(#call, e_);        \
      rc = -3;                                 \
      goto done;                               \
    }                                          \
  } while (0)

template <typename T>
cudaError_t to_device(T** d, const std::vector<T>& h) {
  *d = nullptr;
  if (h.empty()) return cudaMalloc(d, sizeof(T));
  cudaError_t e = cudaMalloc(d, sizeof(T) * h.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
}

int32_t add_pores_device(int kind, int32_t nx, int32_t ny, int32_t nz, double target_frac, double aspect,
                         double log_mu, double log_sigma, int32_t pore_phase, uint64_t seed, int32_t device,
                         int32_t* d_pix) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !d_pix || target_frac < 0.0 || target_frac >= 1.0 || aspect <= 0.0)
    return -1;
  const long long ns = (long long)nx * ny * nz;
  const double target = target_frac * (double)ns;
  constexpr int kChunk = 4096;
  int32_t rc = 0;
  unsigned long long* d_count = nullptr;
  long long* d_state = nullptr;
  PoreShape* d_pores = nullptr;
  long long state[3] = {0, 0, 0};
  unsigned long long count0 = 0;
  std::vector<PoreShape> chunk(kChunk);
  PoreStream S(kind, nx, ny, nz, aspect, log_mu, log_sigma, seed);
  MG_CUDA(cudaSetDevice(device));
  MG_CUDA(cudaMalloc(&d_count, sizeof(unsigned long long)));
  MG_CUDA(cudaMalloc(&d_state, sizeof state));
  MG_CUDA(cudaMalloc(&d_pores, sizeof(PoreShape) * kChunk));
  MG_CUDA(cudaMemset(d_count, 0, sizeof(unsigned long long)));
  count_phase_kernel<<<std::max<long long>(1, std::min<long long>(4096, (ns + 255) / 256)), 256>>>(ns, d_pix,
                                                                                                   pore_phase, d_count);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaMemcpy(&count0, d_count, sizeof count0, cudaMemcpyDeviceToHost));
  state[0] = (long long)count0;
  while ((double)state[0] < target) {
    if (state[1] > 100000000) {
      rc = -2;
      goto done;
    }
    for (int i = 0; i < kChunk; ++i) S.next(chunk[i]);
    MG_CUDA(cudaMemcpy(d_pores, chunk.data(), sizeof(PoreShape) * kChunk, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(d_state, state, sizeof state, cudaMemcpyHostToDevice));
    pore_paint_kernel<<<1, kPaintThreads>>>(d_pores, kChunk, nx, ny, nz, pore_phase, target, d_pix, d_state);
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaMemcpy(state, d_state, sizeof state, cudaMemcpyDeviceToHost));
    if (state[2]) break;
  }
  rc = (int32_t)state[1];
done:
  cudaFree(d_count);
  cudaFree(d_state);
  cudaFree(d_pores);
  return rc;
}

}  // namespace

extern "C" int32_t e3d_micro_grains_device(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                           double laguerre_sigma, uint64_t seed, int32_t device, int32_t* d_pix,
                                           double* rod) {
  E3D_TRACE("e3d_micro_grains_device");
  if (nx <= 0 || ny <= 0 || nz <= 0 || ngrains <= 0 || !d_pix || !rod) return -1;
  GrainPlan P;
  int32_t rc = grain_plan(nx, ny, nz, ngrains, laguerre_sigma, seed, rod, P);
  if (rc) return rc;
  GrainDev D{};
  int64_t* d_off = nullptr;
  uint8_t* d_brute = nullptr;
  int32_t* d_cg = nullptr;
  double *d_cx = nullptr, *d_cy = nullptr, *d_cz = nullptr, *d_sx = nullptr, *d_sy = nullptr, *d_sz = nullptr,
         *d_w = nullptr;
  int* d_err = nullptr;
  int herr = 0;
  const long long nblocks = (long long)P.nb[0] * P.nb[1] * P.nb[2];
  MG_CUDA(cudaSetDevice(device));
  MG_CUDA(to_device(&d_off, P.off));
  MG_CUDA(to_device(&d_brute, P.brute));
  MG_CUDA(to_device(&d_cg, P.cg));
  MG_CUDA(to_device(&d_cx, P.cx));
  MG_CUDA(to_device(&d_cy, P.cy));
  MG_CUDA(to_device(&d_cz, P.cz));
  MG_CUDA(to_device(&d_sx, P.sx));
  MG_CUDA(to_device(&d_sy, P.sy));
  MG_CUDA(to_device(&d_sz, P.sz));
  MG_CUDA(to_device(&d_w, P.w));
  MG_CUDA(cudaMalloc(&d_err, sizeof(int)));
  MG_CUDA(cudaMemset(d_err, 0, sizeof(int)));
  D.nx = nx;
  D.ny = ny;
  D.nz = nz;
  D.ngrains = ngrains;
  D.B = P.B;
  D.nb0 = P.nb[0];
  D.nb1 = P.nb[1];
  D.L0 = P.L[0];
  D.L1 = P.L[1];
  D.L2 = P.L[2];
  D.off = d_off;
  D.brute = d_brute;
  D.cg = d_cg;
  D.cx = d_cx;
  D.cy = d_cy;
  D.cz = d_cz;
  D.sx = d_sx;
  D.sy = d_sy;
  D.sz = d_sz;
  D.w = d_w;
  if (nblocks > 0x7fffffffLL) {
    rc = -1;
    goto done;
  }
  grain_assign_kernel<<<(unsigned)nblocks, 256>>>(D, d_pix, d_err);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  rc = herr ? -2 : 0;
done:
  cudaFree(d_off);
  cudaFree(d_brute);
  cudaFree(d_cg);
  cudaFree(d_cx);
  cudaFree(d_cy);
  cudaFree(d_cz);
  cudaFree(d_sx);
  cudaFree(d_sy);
  cudaFree(d_sz);
  cudaFree(d_w);
  cudaFree(d_err);
  return rc;
}

extern "C" int32_t e3d_micro_spherical_pores_device(int32_t nx, int32_t ny, int32_t nz, double target_frac,
                                                    double log_mu, double log_sigma, int32_t pore_phase,
                                                    uint64_t seed, int32_t device, int32_t* d_pix) {
  E3D_TRACE("e3d_micro_spherical_pores_device");
  return add_pores_device(0, nx, ny, nz, target_frac, 1.0, log_mu, log_sigma, pore_phase, seed, device, d_pix);
}

extern "C" int32_t e3d_micro_ellipsoidal_pores_device(int32_t nx, int32_t ny, int32_t nz, double target_frac,
                                                      double aspect, double log_mu, double log_sigma,
                                                      int32_t pore_phase, uint64_t seed, int32_t device,
                                                      int32_t* d_pix) {
  E3D_TRACE("e3d_micro_ellipsoidal_pores_device");
  return add_pores_device(1, nx, ny, nz, target_frac, aspect, log_mu, log_sigma, pore_phase, seed, device, d_pix);
}
