// e3d_apply_noalloc: the matrix-free K.x of e3d_apply_device, for callers that
// must not allocate device memory.
//
// Who needs it: a host framework that owns every device allocation and forbids
// library-side cudaMalloc (cudaMalloc also synchronises the device), or a
// serving loop that admits work under a fixed HBM budget and cannot let a call
// grow its footprint.  Such a caller passes its own device buffers for the
// inputs and the output; everything else this kernel needs -- the scaled
// stiffness table and the tile-edge force halos -- lives in one file-scope
// __device__ array of E3D_NOALLOC_SCRATCH_BYTES (16 MiB), which every GPU that
// loads this library holds until the process exits.
//
// Set-up: the first call on a device looks up the device address of that array
// (cudaGetSymbolAddress, with the device current) and caches it; make that first
// call before any stream capture.  Every call reuses the same array and finds
// the previous call's contents in it: the error flag is cleared on each call and
// the table and halos are fully rewritten before they are read.  Calls that
// overlap on the GPU (other streams, other host threads, same device) race on
// the array and must be serialised by the caller.  Each call reads the
// phase-check flag back into host memory and waits for its stream twice, so it
// returns only once y is complete.  x and y must not overlap.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "e3d_gpu.h"

// The kernel header defines non-template kernels; this translation unit takes
// its own copy of them inside a private namespace so the two objects link.
namespace e3d_noalloc_tu {
#include "e3d_kernels.cuh"
}  // namespace e3d_noalloc_tu

using namespace e3d_noalloc_tu::e3d;

// Record the text returned by e3d_last_cuda_error (defined in e3d_gpu.cu).
void e3d_record_cuda_error(const char* what, cudaError_t e);
void e3d_record_error_text(const char* text);

namespace {

constexpr long long kScratchDoubles = E3D_NOALLOC_SCRATCH_BYTES / 8;
constexpr long long kFlagDoubles = 32;  // first 256 bytes: error flag

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Stiffness tables for phases 1..nphase at rows 1..nphase (row 0 unused), so the
// 1-based phase ids of the caller index them directly.  Same arithmetic as
// femat_phase_kernel (modal_table).
__global__ void noalloc_table_kernel(const double* __restrict__ cmod, int nphase, double* __restrict__ table) {
  const int p = blockIdx.x;  // 0-based phase
  if (threadIdx.x != 0) return;
  double C6[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) C6[i][j] = cmod[p + (long long)nphase * (i + 6 * j)];
  modal_table(C6, table + (long long)(p + 1) * kCsStride);
}

__global__ void noalloc_check_pix_kernel(const int32_t* __restrict__ pix, long long ns, int nphase,
                                         int* __restrict__ flag) {
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < ns;
       m += (long long)gridDim.x * blockDim.x) {
    const int v = pix[m];
    if (v < 1 || v > nphase) atomicExch(flag, 1);
  }
}

__global__ void noalloc_finish_kernel(GridDims G, const double* __restrict__ hx, const double* __restrict__ hy,
                                      const double* __restrict__ hd, double* y) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= G.ns) return;
  const int x = (int)(m % G.nx);
  const int yy = (int)((m / G.nx) % G.ny);
  const int z = (int)(m / ((long long)G.nx * G.ny));
  double v[3] = {y[m], y[m + G.ns], y[m + 2 * G.ns]};
  halo_add<double>(G, hx, hy, hd, x, yy, z, v);
  y[m] = v[0];
  y[m + G.ns] = v[1];
  y[m + 2 * G.ns] = v[2];
}

int32_t fail(const char* what, cudaError_t e) {
  e3d_record_cuda_error(what, e);
  return E3D_ERR_CUDA;
}

// Same tiling as the handle path: z split into chunks so that a small grid
// still spreads over every SM; the halo size does not depend on the split.
GridDims noalloc_dims(int nx, int ny, int nz, int num_sms) {
  GridDims G{};
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.ns = (long long)nx * ny * nz;
  G.ntx = (int)(((long long)nx + TILE_X - 1) / TILE_X);
  G.nty = (int)(((long long)ny + TILE_Y - 1) / TILE_Y);
  const long long cols = (long long)G.ntx * G.nty;
  const long long want = (long long)(num_sms > 0 ? num_sms : 1) * 4;
  const int ntz = (int)(want > cols ? std::min<long long>(nz, (want + cols - 1) / cols) : 1);
  int tz = (int)(((long long)nz + ntz - 1) / ntz);
  if (tz < 16) tz = std::min(nz, 16);
  G.tz = tz;
  G.ntz = (int)(((long long)nz + tz - 1) / tz);
  G.ntiles = cols * G.ntz;
  return G;
}

// Doubles of scratch one call needs: flag, table rows 0..nphase, halos.
long long scratch_doubles(const GridDims& G, int nphase) {
  const long long halo = G.ntiles * G.tz;
  return kFlagDoubles + (long long)(nphase + 1) * kCsStride + 3 * halo * (TILE_X + TILE_Y + 1);
}

}  // namespace

extern "C" int32_t e3d_apply_noalloc(int32_t nx, int32_t ny, int32_t nz, int32_t nphase, const int32_t* d_pix,
                                     const double* d_cmod, const double* d_x, double* d_y, void* stream) {
  if (!d_pix || !d_cmod || !d_x || !d_y) {
    e3d_record_error_text("e3d_apply_noalloc: d_pix, d_cmod, d_x and d_y must not be NULL");
    return E3D_ERR_INPUT;
  }
  if (nx < 1 || ny < 1 || nz < 1 || nphase < 1) {
    e3d_record_error_text("e3d_apply_noalloc: nx, ny, nz and nphase must be at least 1");
    return E3D_ERR_INPUT;
  }
  // The halos alone take 3*(TILE_X+TILE_Y+1)/(TILE_X*TILE_Y) > 1/4 double per
  // node, so a grid above 4*kScratchDoubles nodes can never fit; refusing it
  // here keeps every size computed below within 64-bit range.
  const long long max_nodes = 4 * kScratchDoubles;
  if (nx > max_nodes || ny > max_nodes || nz > max_nodes || (long long)nx * ny > max_nodes ||
      (long long)nx * ny * nz > max_nodes) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "e3d_apply_noalloc: a %dx%dx%d grid cannot fit in E3D_NOALLOC_SCRATCH_BYTES = %lld "
                  "(at most %lld nodes)",
                  nx, ny, nz, (long long)E3D_NOALLOC_SCRATCH_BYTES, max_nodes);
    e3d_record_error_text(msg);
    return E3D_ERR_INPUT;
  }
  {
    // y = K x is formed in place of y while other blocks still read x
    const uintptr_t xb = reinterpret_cast<uintptr_t>(d_x), yb = reinterpret_cast<uintptr_t>(d_y);
    const uintptr_t bytes = (uintptr_t)(3LL * nx * ny * nz) * sizeof(double);
    if (xb < yb + bytes && yb < xb + bytes) {
      e3d_record_error_text("e3d_apply_noalloc: d_x and d_y overlap; y = K x needs separate buffers");
      return E3D_ERR_INPUT;
    }
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail("cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "e3d_apply_noalloc: device %d is beyond the %d devices this entry point serves",
                  dev, kMaxDevices);
    e3d_record_error_text(msg);
    return E3D_ERR_INPUT;
  }
  int num_sms = 0;
  if ((e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return fail("cudaDeviceGetAttribute", e);
  const GridDims G = noalloc_dims(nx, ny, nz, num_sms);
  const long long need = scratch_doubles(G, nphase);
  if (need > kScratchDoubles) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "e3d_apply_noalloc: a %dx%dx%d grid with %d phases needs %lld bytes of scratch, "
                  "more than E3D_NOALLOC_SCRATCH_BYTES = %lld",
                  nx, ny, nz, nphase, need * 8, (long long)E3D_NOALLOC_SCRATCH_BYTES);
    e3d_record_error_text(msg);
    return E3D_ERR_INPUT;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return fail("cudaGetSymbolAddress(g_noalloc_scratch)", e);
      g_scratch_addr[dev] = ptr;
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* scratch = static_cast<double*>(base);
  int* flag = reinterpret_cast<int*>(scratch);
  double* table = scratch + kFlagDoubles;
  double* hx = table + (long long)(nphase + 1) * kCsStride;
  const long long halo = G.ntiles * G.tz;
  double* hy = hx + 3 * halo * TILE_Y;
  double* hd = hy + 3 * halo * TILE_X;

  if ((e = cudaMemsetAsync(flag, 0, sizeof(int), s)) != cudaSuccess) return fail("cudaMemsetAsync(flag)", e);
  noalloc_check_pix_kernel<<<256, 256, 0, s>>>(d_pix, G.ns, nphase, flag);
  noalloc_table_kernel<<<nphase, 64, 0, s>>>(d_cmod, nphase, table);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("noalloc set-up kernels", e);
  int hflag = 0;
  if ((e = cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return fail("cudaMemcpyAsync(flag)", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail("cudaStreamSynchronize", e);
  if (hflag != 0) {  // a phase id outside [1, nphase]
    e3d_record_error_text("e3d_apply_noalloc: a phase id in d_pix is outside [1, nphase]");
    return E3D_ERR_INPUT;
  }

  ApplyArgs<double> A{};
  A.g = G;
  A.pix = d_pix;  // 1-based ids index the table (row 0 unused)
  A.cs = table;
  A.ncs = nphase + 1;
  A.x = d_x;
  A.y = d_y;
  A.hx = hx;
  A.hy = hy;
  A.hd = hd;
  apply_tiles_kernel<double><<<(unsigned)G.ntiles, NT, 0, s>>>(A, nullptr);
  noalloc_finish_kernel<<<(unsigned)((G.ns + 255) / 256), 256, 0, s>>>(G, hx, hy, hd, d_y);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("noalloc apply kernels", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail("cudaStreamSynchronize", e);
  return E3D_OK;
}

// Bounds-checked build: this translation unit's record (read by e3d_debug_bounds).
int e3d_bounds_take_noalloc(long long out[4]) { return e3d_noalloc_tu::e3d::bounds_take(out); }
