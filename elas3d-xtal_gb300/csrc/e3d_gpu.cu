// C ABI of the sm_103a voxel-FE solver (include/e3d_gpu.h).  Each entry point
// replaces one subroutine of src/elas3dxtal_pcg.f90; see the header for the
// mapping.  All device work runs on the handle's stream; calls return after it
// completes.
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "e3d_gpu.h"
#include "e3d_kernels.cuh"
#include "e3d_trace.h"

using namespace e3d;

namespace {

thread_local std::string g_last_cuda_error;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

// Error text for e3d_last_cuda_error, also used by the other translation units.
void e3d_record_error_text(const char* text) { g_last_cuda_error = text ? text : ""; }
void e3d_record_cuda_error(const char* what, cudaError_t e) {
  g_last_cuda_error = std::string(what) + ": " + cudaGetErrorString(e);
}

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, found through the runtime so the
// library does not link libcuda (it loads on hosts without a driver).
EncodeTiledFn encode_tiled_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

}  // namespace

// Tensor maps of the TMA-fed FP32 stencil for one grid: 4-D (x, y, z,
// component) maps of h0, h1 and z with the main / column / row / corner boxes,
// and a 3-D map of the phase ids.  Needs nx*4 to be a multiple of 16 bytes (the
// row stride of a tensor map) and 16-byte aligned bases.  Returns false when
// the grid or the driver does not allow it; the caller then keeps per-thread
// loads.
bool e3d_encode_plane_maps(PlaneMaps* out, const float* h0, const float* h1, const float* z, const int32_t* pix,
                           const GridDims& G) {
  EncodeTiledFn fn = encode_tiled_fn();
  if (!fn || G.nx % 4 != 0) return false;
  for (const void* b : {(const void*)h0, (const void*)h1, (const void*)z, (const void*)pix})
    if (reinterpret_cast<uintptr_t>(b) % 16 != 0) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)G.nx, (cuuint64_t)G.ny, (cuuint64_t)G.nz, 3};
  const cuuint64_t strides[3] = {(cuuint64_t)G.nx * 4, (cuuint64_t)G.nx * G.ny * 4, (cuuint64_t)G.ns * 4};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const float* bases[3] = {h0, h1, z};
  CUtensorMap* dst[3] = {out->h0, out->h1, out->z};
  for (int v = 0; v < 3; ++v)
    for (int k = 0; k < 4; ++k) {
      const cuuint32_t box[4] = {(cuuint32_t)kBoxX[k], (cuuint32_t)kBoxY[k], 1, 3};
      if (fn(&dst[v][k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(bases[v]), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    }
  const cuuint32_t pbox[3] = {32, 8, 1};
  if (fn(&out->pix, CU_TENSOR_MAP_DATA_TYPE_INT32, 3, const_cast<int32_t*>(pix), dims, strides, pbox, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  return true;
}

struct e3d_handle {
  e3d_problem_t prob{};
  GridDims G{};
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int64_t bytes = 0;
  int64_t launches = 0;
  std::vector<void*> allocs;

  // state (see e3d_kernels.cuh for the layout)
  int32_t* pix = nullptr;
  double* rod = nullptr;
  double* cmod = nullptr;
  double* cs = nullptr;
  float* cs32 = nullptr;
  double* dk = nullptr;
  double* dkd = nullptr;
  double* u = nullptr;
  double* g = nullptr;
  double* b = nullptr;
  double* z = nullptr;
  double* h0 = nullptr;
  double* h1 = nullptr;
  double* Ah = nullptr;
  double* minv = nullptr;
  // mixed precision (E3D_PREC_MIXED): FP32 inner-loop state
  float* du32 = nullptr;
  float* g32 = nullptr;
  float* z32 = nullptr;
  float* h32a = nullptr;
  float* h32b = nullptr;
  float* Ah32 = nullptr;
  float* minv32 = nullptr;
  int since_replace = 0;
  // TMA-fed FP32 stencil: tensor maps of h32a, h32b, z32, pix (null: per-thread loads)
  PlaneMaps* maps = nullptr;
  int pcg_grid32_tma = 0;
  double* hx = nullptr;
  double* hy = nullptr;
  double* hd = nullptr;
  double* partial = nullptr;  // reduction scratch
  int partial_n = 0;
  double* scalars = nullptr;  // small results
  double* history = nullptr;
  PcgState* st = nullptr;
  GridBarrier* bar = nullptr;
  int* err = nullptr;

  double C = 0.0;
  double gg0 = 0.0;
  bool uploaded = false, femat_done = false, energy_done = false, solve_ready = false, minv_ready = false;
  int pcg_grid = 0;
  int pcg_grid32 = 0;
  double ms_setup = 0.0, ms_iter = 0.0;
  JumpParams J{};
};

namespace {

int32_t cuda_fail(cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  g_last_cuda_error = buf;
  return E3D_ERR_CUDA;
}

#define E3D_CUDA(call)                                 \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

#define E3D_LAUNCHED(h)                                          \
  do {                                                           \
    (h)->launches++;                                             \
    cudaError_t e_ = cudaGetLastError();                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, "kernel launch"); \
  } while (0)

template <typename T>
int32_t dalloc(e3d_handle* h, T** p, size_t count) {
  const size_t bytes = count * sizeof(T) + 16;
  if (h->prob.hbm_budget > 0 && h->bytes + (int64_t)bytes > h->prob.hbm_budget) return E3D_ERR_OOM;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return E3D_ERR_OOM;
  }
  h->allocs.push_back(q);
  h->bytes += (int64_t)bytes;
  *p = static_cast<T*>(q);
  return E3D_OK;
}

int32_t sync(e3d_handle* h) {
  E3D_CUDA(cudaStreamSynchronize(h->stream));
  int derr = 0;
  E3D_CUDA(cudaMemcpy(&derr, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (derr == DEV_TIMEOUT) return E3D_ERR_TIMEOUT;
  if (derr != DEV_OK) return E3D_ERR_CUDA;
  return E3D_OK;
}

unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int reduction_grid(const e3d_handle* h) { return std::max(1, std::min(h->num_sms * 4, h->partial_n)); }

// Sum `nfields` interleaved fields of n partials into h->scalars[0..nfields).
int32_t reduce_to_host(e3d_handle* h, int n, int stride, int nfields, double* out) {
  reduce_partials_kernel<<<1, 256, 0, h->stream>>>(h->partial, n, stride, nfields, h->scalars);
  E3D_LAUNCHED(h);
  E3D_CUDA(cudaMemcpyAsync(out, h->scalars, sizeof(double) * nfields, cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

ApplyArgs<double> apply_args(e3d_handle* h, const double* x, double* y) {
  ApplyArgs<double> A{};
  A.g = h->G;
  A.pix = h->pix;
  A.cs = h->cs;
  A.ncs = h->prob.nphase;
  A.x = x;
  A.zv = nullptr;
  A.gamma = 0.0;
  A.reset = 0;
  A.hnew = nullptr;
  A.y = y;
  A.hx = h->hx;
  A.hy = h->hy;
  A.hd = h->hd;
  return A;
}

// y_partial = in-tile K x plus halos (not yet added).
int32_t launch_apply_tiles(e3d_handle* h, const double* x, double* y) {
  ApplyArgs<double> A = apply_args(h, x, y);
  apply_tiles_kernel<double><<<(unsigned)h->G.ntiles, NT, 0, h->stream>>>(A, nullptr);
  E3D_LAUNCHED(h);
  return E3D_OK;
}

int32_t apply_device(e3d_handle* h, const double* d_x, double* d_y) {
  int32_t rc = launch_apply_tiles(h, d_x, h->Ah);
  if (rc) return rc;
  apply_finish_kernel<double><<<blocks_for(h->G.ns, 256), 256, 0, h->stream>>>(h->G, h->Ah, h->hx, h->hy,
                                                                                 h->hd, d_y);
  E3D_LAUNCHED(h);
  return E3D_OK;
}

GridDims make_dims(int nx, int ny, int nz, int num_sms) {
  GridDims G{};
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.ns = (long long)nx * ny * nz;
  G.ntx = (nx + TILE_X - 1) / TILE_X;
  G.nty = (ny + TILE_Y - 1) / TILE_Y;
  // z chunk: keep >= ~16 tiles per SM in flight (load balance) but long
  // enough that the one redundant element plane per chunk stays small.
  const long long cols = (long long)G.ntx * G.nty;
  const long long want = std::max<long long>(1, (long long)num_sms * 16);
  int ntz = (int)std::max<long long>(1, std::min<long long>(nz, (want + cols - 1) / cols));
  int tz = (nz + ntz - 1) / ntz;
  if (tz < 16) tz = std::min(nz, 16);
  G.tz = tz;
  G.ntz = (nz + tz - 1) / tz;
  G.ntiles = cols * G.ntz;
  return G;
}

}  // namespace

extern "C" {

void e3d_problem_defaults(e3d_problem_t* p, int32_t nx, int32_t ny, int32_t nz, int32_t nphase) {
  std::memset(p, 0, sizeof *p);
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  p->nphase = nphase;
  p->flag_m = 1;
  p->criterion = E3D_CRIT_REF;
  p->precision = E3D_PREC_FP64;
  p->divergence_reset = 1;
  p->max_iter = 10000;
  p->device = 0;
  p->tol = 1.0e-8f;
  p->refine_every = 0;
  p->c11 = 206.0e9;
  p->c12 = 133.0e9;
  p->c44 = 119.0e9;
  p->e1 = 0.0;
  p->nu1 = 0.0;
  p->strain[2] = 1.0e-3;
  p->hbm_budget = 0;
}

const char* e3d_strerror(int32_t s) {
  switch (s) {
    case E3D_OK: return "ok";
    case E3D_ERR_INPUT: return "invalid input";
    case E3D_ERR_OOM: return "device memory exhausted or over the HBM budget";
    case E3D_ERR_BREAKDOWN: return "PCG breakdown (non-finite h.Ah or z.g)";
    case E3D_ERR_MAXITER: return "maximum iterations reached without convergence";
    case E3D_ERR_TIMEOUT: return "device-side wait exceeded its limit";
    case E3D_ERR_CUDA: return "CUDA runtime error";
    case E3D_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

const char* e3d_last_cuda_error(void) { return g_last_cuda_error.c_str(); }

int32_t e3d_create(e3d_handle_t** out, const e3d_problem_t* p) {
  if (!out || !p) return E3D_ERR_INPUT;
  *out = nullptr;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || p->nphase < 1 || p->max_iter < 0) return E3D_ERR_INPUT;
  if ((long long)p->nx * p->ny * p->nz > (1LL << 40)) return E3D_ERR_INPUT;
  if (p->precision != E3D_PREC_FP64 && p->precision != E3D_PREC_MIXED) return E3D_ERR_INPUT;
  if (p->criterion != E3D_CRIT_REF && p->criterion != E3D_CRIT_PRECOND_REL) return E3D_ERR_INPUT;
  if (p->preconditioner != E3D_PRECOND_BLOCK_JACOBI && p->preconditioner != E3D_PRECOND_NONE) return E3D_ERR_INPUT;
  if (p->refine_decades < 0 || p->refine_decades > 15) return E3D_ERR_INPUT;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  if (p->device < 0 || p->device >= ndev) return E3D_ERR_INPUT;
  e3d_handle* h = new e3d_handle();
  h->prob = *p;
  h->device = p->device;
  auto fail = [&](int32_t rc) {
    e3d_destroy(h);
    return rc;
  };
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "cudaSetDevice"));
  cudaDeviceProp prop{};
  if ((e = cudaGetDeviceProperties(&prop, h->device)) != cudaSuccess) return fail(cuda_fail(e, "props"));
  h->num_sms = prop.multiProcessorCount;
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(cuda_fail(e, "cudaStreamCreate"));
  h->G = make_dims(p->nx, p->ny, p->nz, h->num_sms);
  const long long ns = h->G.ns, n3 = 3 * ns;
  const int np = p->nphase;
  // PCG grid: as many co-resident tile blocks as the device holds.
  // (phase B of the per-thread-load kernels streams through dynamic shared memory)
  int per_sm = 0;
  if ((e = cudaFuncSetAttribute(pcg_persistent_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                pcg_dyn_smem_bytes<double>())) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_persistent_kernel<double>, NT,
                                                         pcg_dyn_smem_bytes<double>())) != cudaSuccess)
    return fail(cuda_fail(e, "occupancy"));
  if (per_sm < 1) return fail(E3D_ERR_CUDA);
  h->pcg_grid = per_sm * h->num_sms;
  int per_sm32 = 0;
  if ((e = cudaFuncSetAttribute(pcg_persistent_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                pcg_dyn_smem_bytes<float>())) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm32, pcg_persistent_kernel<float>, NT,
                                                         pcg_dyn_smem_bytes<float>())) != cudaSuccess)
    return fail(cuda_fail(e, "occupancy"));
  if (per_sm32 < 1) return fail(E3D_ERR_CUDA);
  h->pcg_grid32 = per_sm32 * h->num_sms;
  int per_sm_tma = 0;
  if (p->precision == E3D_PREC_MIXED) {
    if ((e = cudaFuncSetAttribute(pcg_persistent_kernel<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kRingSmemBytes)) != cudaSuccess ||
        (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_tma, pcg_persistent_kernel<float, true>, NT,
                                                           kRingSmemBytes)) != cudaSuccess)
      return fail(cuda_fail(e, "occupancy (TMA)"));
  }
  h->partial_n = std::max(std::max(h->pcg_grid, h->pcg_grid32), h->num_sms * 4) * 12;
  const long long halo = h->G.ntiles * h->G.tz;
  int32_t rc = E3D_OK;
  if ((rc = dalloc(h, &h->pix, ns)) || (rc = dalloc(h, &h->rod, 3 * (size_t)std::max(np - 1, 1))) ||
      (rc = dalloc(h, &h->cmod, 36 * (size_t)np)) || (rc = dalloc(h, &h->cs, kCsStride * (size_t)np)) ||
      (rc = dalloc(h, &h->cs32, kCs32Stride * (size_t)np)) || (rc = dalloc(h, &h->dk, 576 * (size_t)np)) ||
      (rc = dalloc(h, &h->dkd, 72 * (size_t)np)) || (rc = dalloc(h, &h->u, n3)) || (rc = dalloc(h, &h->g, n3)) ||
      (rc = dalloc(h, &h->b, n3)) || (rc = dalloc(h, &h->z, n3)) || (rc = dalloc(h, &h->h0, n3)) ||
      (rc = dalloc(h, &h->h1, n3)) || (rc = dalloc(h, &h->Ah, n3)) || (rc = dalloc(h, &h->minv, 6 * ns)) ||
      (rc = dalloc(h, &h->hx, 3 * halo * TILE_Y)) || (rc = dalloc(h, &h->hy, 3 * halo * TILE_X)) ||
      (rc = dalloc(h, &h->hd, 3 * halo)) || (rc = dalloc(h, &h->partial, (size_t)h->partial_n)) ||
      (rc = dalloc(h, &h->scalars, 64)) ||
      (rc = dalloc(h, &h->history, (size_t)std::max(p->max_iter, 1))) || (rc = dalloc(h, &h->st, 1)) ||
      (rc = dalloc(h, &h->bar, 1)) || (rc = dalloc(h, &h->err, 1)))
    return fail(rc);
  if (p->precision == E3D_PREC_MIXED) {
    if ((rc = dalloc(h, &h->du32, n3)) || (rc = dalloc(h, &h->g32, n3)) || (rc = dalloc(h, &h->z32, n3)) ||
        (rc = dalloc(h, &h->h32a, n3)) || (rc = dalloc(h, &h->h32b, n3)) || (rc = dalloc(h, &h->Ah32, n3)) ||
        (rc = dalloc(h, &h->minv32, 6 * ns)))
      return fail(rc);
    if ((e = cudaMemsetAsync(h->h32a, 0, sizeof(float) * n3, h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(h->h32b, 0, sizeof(float) * n3, h->stream)) != cudaSuccess)
      return fail(cuda_fail(e, "memset"));
    // Inner stencil: per-thread loads (500^3: 6.9 ms per inner iteration, the
    // TMA plane ring 8.0 ms); E3D_TMA=1 selects the ring where the grid allows it.
    const char* want_tma = std::getenv("E3D_TMA");
    PlaneMaps hm{};
    if (want_tma && want_tma[0] && want_tma[0] != '0' && per_sm_tma >= 1 &&
        e3d_encode_plane_maps(&hm, h->h32a, h->h32b, h->z32, h->pix, h->G)) {
      if ((rc = dalloc(h, &h->maps, 1))) return fail(rc);
      if ((e = cudaMemcpyAsync(h->maps, &hm, sizeof hm, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
        return fail(cuda_fail(e, "tensor maps"));
      h->pcg_grid32_tma = std::min(per_sm_tma * h->num_sms, h->pcg_grid32);
    }
  }
  if ((e = cudaMemsetAsync(h->err, 0, sizeof(int), h->stream)) != cudaSuccess) return fail(cuda_fail(e, "memset"));
  if ((e = cudaMemsetAsync(h->bar, 0, sizeof(GridBarrier), h->stream)) != cudaSuccess)
    return fail(cuda_fail(e, "memset"));
  if ((e = cudaMemsetAsync(h->h0, 0, sizeof(double) * n3, h->stream)) != cudaSuccess)
    return fail(cuda_fail(e, "memset"));
  if ((e = cudaMemsetAsync(h->h1, 0, sizeof(double) * n3, h->stream)) != cudaSuccess)
    return fail(cuda_fail(e, "memset"));
  if ((e = cudaMemsetAsync(h->u, 0, sizeof(double) * n3, h->stream)) != cudaSuccess)
    return fail(cuda_fail(e, "memset"));
  const double* s = p->strain;  // exx eyy ezz exz eyz exy
  const double E[3][3] = {{s[0], s[5], s[3]}, {s[5], s[1], s[4]}, {s[3], s[4], s[2]}};
  std::memcpy(h->J.E, E, sizeof E);
  if ((rc = sync(h))) return fail(rc);
  *out = h;
  return E3D_OK;
}

int32_t e3d_destroy(e3d_handle_t* h) {
  if (!h) return E3D_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* q : h->allocs) cudaFree(q);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return E3D_OK;
}

int64_t e3d_device_bytes(const e3d_handle_t* h) { return h ? h->bytes : 0; }
int64_t e3d_launch_count(const e3d_handle_t* h) { return h ? h->launches : 0; }
int32_t e3d_stencil_path(const e3d_handle_t* h) {
  if (!h || h->prob.precision != E3D_PREC_MIXED) return E3D_PATH_FP64;
  return h->maps ? E3D_PATH_F32_TMA : E3D_PATH_F32;
}

int32_t e3d_upload(e3d_handle_t* h, const int32_t* pix, const double* rod) {
  E3D_TRACE("e3d_upload");
  if (!h || !pix) return E3D_ERR_INPUT;
  const auto& p = h->prob;
  if (p.flag_m == 1 && p.nphase > 1 && !rod) return E3D_ERR_INPUT;
  const long long ns = h->G.ns;
  cudaSetDevice(h->device);
  // The ids go to the device as they are (one DMA from the caller's buffer,
  // at full speed when it is pinned); the phase range check (ppixel_hdf5,
  // src/elas3dxtal_pcg.f90:2986-2989) and the conversion to 0-based ids run
  // there, over the whole map in one pass.  A refused map leaves the handle
  // without an upload.
  h->uploaded = false;
  h->femat_done = h->energy_done = h->solve_ready = h->minv_ready = false;
  E3D_CUDA(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  E3D_CUDA(cudaMemcpyAsync(h->pix, pix, sizeof(int32_t) * ns, cudaMemcpyHostToDevice, h->stream));
  pix_to_zero_based_kernel<<<blocks_for(ns, 256), 256, 0, h->stream>>>(ns, p.nphase, h->pix, h->err);
  E3D_LAUNCHED(h);
  if (rod && p.nphase > 1)
    E3D_CUDA(cudaMemcpyAsync(h->rod, rod, sizeof(double) * 3 * (p.nphase - 1), cudaMemcpyHostToDevice, h->stream));
  else
    E3D_CUDA(cudaMemsetAsync(h->rod, 0, sizeof(double) * 3, h->stream));
  E3D_CUDA(cudaStreamSynchronize(h->stream));
  int derr = 0;
  E3D_CUDA(cudaMemcpy(&derr, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (derr != DEV_OK) {
    E3D_CUDA(cudaMemset(h->err, 0, sizeof(int)));
    e3d_record_error_text("e3d_upload: a phase id lies outside [1, nphase]");
    return E3D_ERR_INPUT;
  }
  h->uploaded = true;
  return E3D_OK;
}

int32_t e3d_upload_device(e3d_handle_t* h, const int32_t* d_pix, const double* rod) {
  E3D_TRACE("e3d_upload_device");
  if (!h || !d_pix) return E3D_ERR_INPUT;
  const auto& p = h->prob;
  if (p.flag_m == 1 && p.nphase > 1 && !rod) return E3D_ERR_INPUT;
  const long long ns = h->G.ns;
  cudaSetDevice(h->device);
  E3D_CUDA(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  pix_from_device_kernel<<<blocks_for(ns, 256), 256, 0, h->stream>>>(ns, d_pix, p.nphase, h->pix, h->err);
  E3D_LAUNCHED(h);
  if (rod && p.nphase > 1)
    E3D_CUDA(cudaMemcpyAsync(h->rod, rod, sizeof(double) * 3 * (p.nphase - 1), cudaMemcpyHostToDevice, h->stream));
  else
    E3D_CUDA(cudaMemsetAsync(h->rod, 0, sizeof(double) * 3, h->stream));
  E3D_CUDA(cudaStreamSynchronize(h->stream));
  int derr = 0;
  E3D_CUDA(cudaMemcpy(&derr, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (derr != DEV_OK) {
    E3D_CUDA(cudaMemset(h->err, 0, sizeof(int)));
    h->uploaded = false;
    return E3D_ERR_INPUT;
  }
  h->uploaded = true;
  h->femat_done = h->energy_done = h->solve_ready = h->minv_ready = false;
  return E3D_OK;
}

int32_t e3d_femat(e3d_handle_t* h) {
  E3D_TRACE("e3d_femat");
  if (!h) return E3D_ERR_INPUT;
  if (!h->uploaded) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const auto& p = h->prob;
  FematParams P{};
  P.nphase = p.nphase;
  P.flag_m = p.flag_m;
  P.c11 = p.c11;
  P.c12 = p.c12;
  P.c44 = p.c44;
  // inclusion K, G from E1, nu1 (src/elas3dxtal_pcg.f90:314-316)
  P.K1 = p.e1 / 3.0 / (1.0 - 2.0 * p.nu1);
  P.G1 = p.e1 / 2.0 / (1.0 + p.nu1);
  // isotropic matrix from C11/C12/C44 via E0, nu0 (:108-111, :305-312)
  {
    const double K0 = (p.c11 + 2.0 * p.c12) / 3.0;
    const double G0 = (p.c11 - p.c12 + 3.0 * p.c44) / 5.0;
    const double E0 = 9.0 * K0 * G0 / (3.0 * K0 + G0);
    const double nu0 = (3.0 * K0 - 2.0 * G0) / (2.0 * (3.0 * K0 + G0));
    P.Km = E0 / 3.0 / (1.0 - 2.0 * nu0);
    P.Gm = E0 / 2.0 / (1.0 + nu0);
  }
  femat_phase_kernel<<<p.nphase, 32, 0, h->stream>>>(P, h->rod, h->cmod, h->cs, h->cs32, h->dk, h->dkd);
  E3D_LAUNCHED(h);
  E3D_CUDA(cudaMemsetAsync(h->b, 0, sizeof(double) * 3 * h->G.ns, h->stream));  // interior nodes
  femat_b_kernel<<<blocks_for(boundary_node_count(h->G), 256), 256, 0, h->stream>>>(h->G, h->J, h->pix, h->dk,
                                                                                         h->b);
  E3D_LAUNCHED(h);
  const int grid = reduction_grid(h);
  femat_c_kernel<<<grid, 256, 0, h->stream>>>(h->G, h->J, h->pix, h->dk, h->partial);
  E3D_LAUNCHED(h);
  double C = 0.0;
  int32_t rc = reduce_to_host(h, grid, 1, 1, &C);
  if (rc) return rc;
  h->C = C;
  h->femat_done = true;
  h->energy_done = h->solve_ready = h->minv_ready = false;
  return E3D_OK;
}

int32_t e3d_init_affine(e3d_handle_t* h) {
  E3D_TRACE("e3d_init_affine");
  if (!h) return E3D_ERR_INPUT;
  cudaSetDevice(h->device);
  affine_kernel<<<blocks_for(h->G.ns, 256), 256, 0, h->stream>>>(h->G, h->J, h->u);
  E3D_LAUNCHED(h);
  h->energy_done = h->solve_ready = false;
  return sync(h);
}

int32_t e3d_energy(e3d_handle_t* h, double* utot, double* gg) {
  E3D_TRACE("e3d_energy");
  if (!h) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  int32_t rc = launch_apply_tiles(h, h->u, h->Ah);
  if (rc) return rc;
  const int grid = reduction_grid(h) / 2 > 0 ? std::min(reduction_grid(h), h->partial_n / 2) : 1;
  energy_finish_kernel<<<grid, 256, 0, h->stream>>>(h->G, h->Ah, h->hx, h->hy, h->hd, h->u, h->b, h->g,
                                                    h->partial);
  E3D_LAUNCHED(h);
  double out[2] = {0.0, 0.0};
  rc = reduce_to_host(h, grid, 2, 2, out);
  if (rc) return rc;
  if (utot) *utot = h->C + out[0];
  if (gg) *gg = out[1];
  h->gg0 = out[1];
  h->energy_done = true;
  h->solve_ready = false;
  return E3D_OK;
}

int32_t e3d_solve_begin(e3d_handle_t* h) {
  E3D_TRACE("e3d_solve_begin");
  if (!h) return E3D_ERR_INPUT;
  if (!h->energy_done) return E3D_ERR_STATE;
  const bool mixed = h->prob.precision == E3D_PREC_MIXED;
  cudaSetDevice(h->device);
  cudaEvent_t e0, e1;
  E3D_CUDA(cudaEventCreate(&e0));
  E3D_CUDA(cudaEventCreate(&e1));
  E3D_CUDA(cudaEventRecord(e0, h->stream));
  // block-Jacobi (kkk == 1, src/elas3dxtal_pcg.f90:1498-1520); the mixed form
  // keeps an FP32 copy of the FP64 inverse.
  bjacobi_kernel<<<blocks_for(h->G.ns, 256), 256, 0, h->stream>>>(
      h->G, h->pix, h->dkd, h->minv, mixed ? h->minv32 : nullptr, h->prob.preconditioner == E3D_PRECOND_NONE);
  E3D_LAUNCHED(h);
  const int grid = reduction_grid(h);
  if (mixed) {
    const long long n3 = 3 * h->G.ns;
    to_float_kernel<<<blocks_for(n3, 256), 256, 0, h->stream>>>(n3, h->g, h->g32);
    E3D_LAUNCHED(h);
    E3D_CUDA(cudaMemsetAsync(h->du32, 0, sizeof(float) * n3, h->stream));
    pcg_init_kernel<float><<<grid, 256, 0, h->stream>>>(h->G, h->minv32, h->g32, h->z32, h->partial);
  } else {
    pcg_init_kernel<double><<<grid, 256, 0, h->stream>>>(h->G, h->minv, h->g, h->z, h->partial);
  }
  E3D_LAUNCHED(h);
  const double drop = (h->prob.precision == E3D_PREC_MIXED && h->prob.refine_decades > 0)
                         ? std::pow(10.0, -(double)h->prob.refine_decades)
                         : 0.0;
  pcg_init_scalars_kernel<<<1, 256, 0, h->stream>>>(h->partial, grid, h->gg0, h->prob.criterion, h->prob.tol,
                                                    h->prob.max_iter, h->prob.divergence_reset, drop, h->st);
  E3D_LAUNCHED(h);
  E3D_CUDA(cudaEventRecord(e1, h->stream));
  int32_t rc = sync(h);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  h->ms_setup = ms;
  h->ms_iter = 0.0;
  h->since_replace = 0;
  h->minv_ready = true;
  h->solve_ready = true;
  return E3D_OK;
}

static int32_t fill_stats(e3d_handle* h, e3d_solve_stats_t* st, int32_t* exit_reason) {
  PcgState S{};
  E3D_CUDA(cudaMemcpy(&S, h->st, sizeof S, cudaMemcpyDeviceToHost));
  int32_t reason = E3D_EXIT_RUNNING;
  switch (S.status) {
    case PCG_CONVERGED: reason = E3D_EXIT_CONVERGED; break;
    case PCG_HAH: reason = E3D_EXIT_HAH_GUARD; break;
    case PCG_MAXITER: reason = E3D_EXIT_MAXITER; break;
    case PCG_BREAKDOWN: reason = E3D_EXIT_BREAKDOWN; break;
    case PCG_TIMEOUT: reason = E3D_EXIT_TIMEOUT; break;
    default: reason = E3D_EXIT_RUNNING;
  }
  *exit_reason = reason;
  if (st) {
    std::memset(st, 0, sizeof *st);
    st->iterations = S.it;
    st->exit_reason = reason;
    st->resets = S.resets;
    st->refinements = S.refinements;
    st->gg = S.gg;
    st->gg0 = S.gg0;
    st->rel_res = S.rel_res;
    st->true_rel = NAN;
    st->ms_setup = h->ms_setup;
    st->ms_iter = h->ms_iter;
  }
  return E3D_OK;
}

}  // extern "C"

namespace {

template <typename T>
PcgArgs<T> pcg_args(e3d_handle* h);

template <>
PcgArgs<double> pcg_args<double>(e3d_handle* h) {
  PcgArgs<double> P{};
  P.A = apply_args(h, nullptr, h->Ah);
  P.h0 = h->h0;
  P.h1 = h->h1;
  P.u = h->u;
  P.g = h->g;
  P.z = h->z;
  P.Ah = h->Ah;
  P.minv = h->minv;
  return P;
}

template <>
PcgArgs<float> pcg_args<float>(e3d_handle* h) {
  PcgArgs<float> P{};
  P.A.g = h->G;
  P.A.pix = h->pix;
  P.A.cs = h->cs32;
  P.A.ncs = h->prob.nphase;
  P.A.hx = reinterpret_cast<float*>(h->hx);  // the FP64 halo buffers, reused
  P.A.hy = reinterpret_cast<float*>(h->hy);
  P.A.hd = reinterpret_cast<float*>(h->hd);
  P.A.y = h->Ah32;
  P.h0 = h->h32a;
  P.h1 = h->h32b;
  P.u = h->du32;
  P.g = h->g32;
  P.z = h->z32;
  P.Ah = h->Ah32;
  P.minv = h->minv32;
  return P;
}

template <typename T>
int32_t launch_pcg(e3d_handle* h, int it_limit) {
  const bool tma = sizeof(T) == 4 && h->maps != nullptr;
  const int grid = sizeof(T) == 8 ? h->pcg_grid : (tma ? h->pcg_grid32_tma : h->pcg_grid32);
  PcgArgs<T> P = pcg_args<T>(h);
  P.maps = h->maps;
  P.partA = h->partial;
  P.partB = h->partial + grid;
  P.st = h->st;
  P.history = h->history;
  P.bar = h->bar;
  P.err = h->err;
  P.timeout_ns = 60ull * 1000000000ull;
  P.it_limit = it_limit;
  E3D_CUDA(cudaMemsetAsync(h->bar, 0, sizeof(GridBarrier), h->stream));
  void* args[] = {&P};
  const void* fn = tma ? (const void*)pcg_persistent_kernel<float, true> : (const void*)pcg_persistent_kernel<T>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(NT), args,
                                              tma ? kRingSmemBytes : pcg_dyn_smem_bytes<T>(), h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchCooperativeKernel(pcg)");
  return E3D_OK;
}

int32_t read_state(e3d_handle* h, PcgState* S) {
  E3D_CUDA(cudaMemcpyAsync(S, h->st, sizeof *S, cudaMemcpyDeviceToHost, h->stream));
  E3D_CUDA(cudaStreamSynchronize(h->stream));
  return E3D_OK;
}

// Mixed form: fold the FP32 correction into u (FP64).
int32_t fold_correction(e3d_handle* h) {
  const long long n3 = 3 * h->G.ns;
  fold_correction_kernel<<<blocks_for(n3, 256), 256, 0, h->stream>>>(n3, h->du32, h->u, h->du32);
  E3D_LAUNCHED(h);
  return E3D_OK;
}

// Mixed form: FP64 residual replacement -- fold du into u, recompute the true
// gradient g = K u + b with the FP64 stencil, and restart the FP32 recurrence
// from it (z = Minv32 g, gg = z.g accumulated in FP64).
int32_t residual_replacement(e3d_handle* h) {
  int32_t rc = fold_correction(h);
  if (rc) return rc;
  if ((rc = launch_apply_tiles(h, h->u, h->Ah))) return rc;
  const int grid = reduction_grid(h);
  true_residual_kernel<<<grid, 256, 0, h->stream>>>(h->G, h->Ah, h->hx, h->hy, h->hd, h->b, h->minv32, h->g,
                                                    h->g32, h->z32, h->partial);
  E3D_LAUNCHED(h);
  replace_scalars_kernel<<<1, 256, 0, h->stream>>>(h->partial, grid, h->st, h->history);
  E3D_LAUNCHED(h);
  h->since_replace = 0;
  return E3D_OK;
}

}  // namespace

extern "C" {

int32_t e3d_iterate(e3d_handle_t* h, int32_t n, e3d_solve_stats_t* st) {
  E3D_TRACE("e3d_iterate");
  if (!h || n < 0) return E3D_ERR_INPUT;
  if (!h->solve_ready) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const bool mixed = h->prob.precision == E3D_PREC_MIXED;
  const int R = h->prob.refine_every > 0 ? h->prob.refine_every : 50;
  cudaEvent_t e0, e1;
  E3D_CUDA(cudaEventCreate(&e0));
  E3D_CUDA(cudaEventCreate(&e1));
  E3D_CUDA(cudaEventRecord(e0, h->stream));
  // Chunks of iterations per cooperative launch keep single launches short;
  // the mixed form also ends a chunk at every residual replacement.
  int remaining = n;
  int32_t rc = E3D_OK;
  PcgState S{};
  if ((rc = read_state(h, &S))) remaining = 0;
  while (remaining > 0 && S.status == PCG_RUNNING) {
    int chunk = std::min(remaining, 256);
    if (mixed) chunk = std::min(chunk, R - h->since_replace);
    const int it0 = S.it;
    rc = mixed ? launch_pcg<float>(h, chunk) : launch_pcg<double>(h, chunk);
    if (rc) break;
    if ((rc = read_state(h, &S))) break;
    // a launch ends early when the solve stops or, in the mixed form with
    // refine_decades set, when the FP32 residual calls for a replacement
    const int done = S.it - it0;
    remaining -= done;
    if (mixed) {
      h->since_replace += done;
      if (S.status == PCG_CONVERGED || S.status == PCG_REPLACE ||
          (S.status == PCG_RUNNING && h->since_replace >= R)) {
        if ((rc = residual_replacement(h))) break;
        if ((rc = read_state(h, &S))) break;
      }
    }
    if (done == 0 && S.status == PCG_RUNNING) break;  // nothing advanced: do not spin
  }
  if (!rc && mixed) rc = fold_correction(h);  // u always holds the current iterate on return
  cudaEventRecord(e1, h->stream);
  int32_t rs = sync(h);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  h->ms_iter += ms;
  int32_t reason = 0;
  int32_t rf = fill_stats(h, st, &reason);
  if (rf) return rf;
  if (rs == E3D_ERR_TIMEOUT || reason == E3D_EXIT_TIMEOUT) return E3D_ERR_TIMEOUT;
  if (rs) return rs;
  if (reason == E3D_EXIT_BREAKDOWN) return E3D_ERR_BREAKDOWN;
  return E3D_OK;
}

int32_t e3d_solve(e3d_handle_t* h, e3d_solve_stats_t* st) {
  int32_t rc = e3d_solve_begin(h);
  if (rc) return rc;
  e3d_solve_stats_t local{};
  rc = e3d_iterate(h, h->prob.max_iter, &local);
  if (st) *st = local;
  if (rc) return rc;
  h->energy_done = false;  // g is now the recurrence residual; energy recomputes it
  if (local.exit_reason == E3D_EXIT_MAXITER) return E3D_ERR_MAXITER;
  return E3D_OK;
}

int32_t e3d_stress(e3d_handle_t* h, double strav[6], double epsav[6]) {
  E3D_TRACE("e3d_stress");
  if (!h) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const int grid = std::max(1, std::min(reduction_grid(h), h->partial_n / 12));
  stress_avg_kernel<<<grid, 256, 0, h->stream>>>(h->G, h->J, h->pix, h->cmod, h->prob.nphase, h->u, h->partial);
  E3D_LAUNCHED(h);
  double out[12];
  int32_t rc = reduce_to_host(h, grid, 12, 12, out);
  if (rc) return rc;
  const double ns = (double)h->G.ns;
  for (int r = 0; r < 6; ++r) {
    if (strav) strav[r] = out[r] / ns;
    if (epsav) epsav[r] = out[6 + r] / ns;
  }
  return E3D_OK;
}

int32_t e3d_stress_field(e3d_handle_t* h, double* sigma, double* vm) {
  E3D_TRACE("e3d_stress_field");
  if (!h) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const long long ns = h->G.ns;
  // sigma lands in z/h1 scratch (6*ns fits in z + half of h1? use Ah + z)
  double* dsig = nullptr;
  double* dvm = nullptr;
  int32_t rc = E3D_OK;
  if ((rc = dalloc(h, &dsig, 6 * (size_t)ns)) || (rc = dalloc(h, &dvm, (size_t)ns))) return rc;
  stress_field_kernel<<<blocks_for(ns, 256), 256, 0, h->stream>>>(h->G, h->J, h->pix, h->cmod, h->prob.nphase,
                                                                   h->u, dsig, dvm);
  E3D_LAUNCHED(h);
  if (sigma) E3D_CUDA(cudaMemcpyAsync(sigma, dsig, sizeof(double) * 6 * ns, cudaMemcpyDeviceToHost, h->stream));
  if (vm) E3D_CUDA(cudaMemcpyAsync(vm, dvm, sizeof(double) * ns, cudaMemcpyDeviceToHost, h->stream));
  rc = sync(h);
  // release the temporaries
  for (void* q : {(void*)dsig, (void*)dvm}) {
    for (size_t i = 0; i < h->allocs.size(); ++i)
      if (h->allocs[i] == q) {
        h->allocs.erase(h->allocs.begin() + (long)i);
        break;
      }
    cudaFree(q);
  }
  h->bytes -= (int64_t)(sizeof(double) * 7 * ns + 32);
  return rc;
}

int32_t e3d_run(e3d_handle_t* h, double utot[2], double out12[12], e3d_solve_stats_t* st) {
  E3D_TRACE("e3d_run");
  if (!h) return E3D_ERR_INPUT;
  int32_t rc;
  if ((rc = e3d_femat(h))) return rc;
  if ((rc = e3d_init_affine(h))) return rc;
  double u0 = 0.0, gg0 = 0.0;
  if ((rc = e3d_energy(h, &u0, &gg0))) return rc;
  e3d_solve_stats_t local{};
  int32_t rs = e3d_solve(h, &local);
  if (st) *st = local;
  if (rs != E3D_OK && rs != E3D_ERR_MAXITER) return rs;
  double u1 = 0.0, gg = 0.0;
  if ((rc = e3d_energy(h, &u1, &gg))) return rc;
  if (st) st->true_rel = std::sqrt(gg / gg0);
  if (utot) {
    utot[0] = u0;
    utot[1] = u1;
  }
  if ((rc = e3d_stress(h, out12 ? out12 : nullptr, out12 ? out12 + 6 : nullptr))) return rc;
  return rs;
}

int32_t e3d_apply(e3d_handle_t* h, const double* x, double* y) {
  if (!h || !x || !y) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const long long n3 = 3 * h->G.ns;
  // stage through z (input) and h1 (output); both are solver scratch
  E3D_CUDA(cudaMemcpyAsync(h->z, x, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  int32_t rc = apply_device(h, h->z, h->h1);
  if (rc) return rc;
  E3D_CUDA(cudaMemcpyAsync(y, h->h1, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->stream));
  h->solve_ready = false;
  return sync(h);
}

int32_t e3d_apply_device(e3d_handle_t* h, const double* d_x, double* d_y) {
  if (!h || !d_x || !d_y) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  int32_t rc = apply_device(h, d_x, d_y);
  if (rc) return rc;
  return sync(h);
}

int32_t e3d_set_u(e3d_handle_t* h, const double* u) {
  if (!h || !u) return E3D_ERR_INPUT;
  cudaSetDevice(h->device);
  E3D_CUDA(cudaMemcpyAsync(h->u, u, sizeof(double) * 3 * h->G.ns, cudaMemcpyHostToDevice, h->stream));
  h->energy_done = h->solve_ready = false;
  return sync(h);
}

static int32_t get_vec(e3d_handle_t* h, const double* d, double* out, size_t count) {
  if (!h || !out) return E3D_ERR_INPUT;
  cudaSetDevice(h->device);
  E3D_CUDA(cudaMemcpyAsync(out, d, sizeof(double) * count, cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int32_t e3d_get_u(e3d_handle_t* h, double* u) { return h ? get_vec(h, h->u, u, 3 * h->G.ns) : E3D_ERR_INPUT; }
int32_t e3d_get_g(e3d_handle_t* h, double* g) { return h ? get_vec(h, h->g, g, 3 * h->G.ns) : E3D_ERR_INPUT; }
int32_t e3d_get_b(e3d_handle_t* h, double* b) {
  if (!h) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  return get_vec(h, h->b, b, 3 * h->G.ns);
}

int32_t e3d_get_C(e3d_handle_t* h, double* C) {
  if (!h || !C) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  *C = h->C;
  return E3D_OK;
}

int32_t e3d_get_cmod(e3d_handle_t* h, double* cmod) {
  if (!h) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  return get_vec(h, h->cmod, cmod, 36 * (size_t)h->prob.nphase);
}

int32_t e3d_get_dk(e3d_handle_t* h, double* dk) {
  if (!h || !dk) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  const int np = h->prob.nphase;
  std::vector<double> t((size_t)576 * np);
  int32_t rc = get_vec(h, h->dk, t.data(), t.size());
  if (rc) return rc;
  // device [p][a][i][b][j] -> Fortran dk(nphase,8,3,8,3)
  for (int p = 0; p < np; ++p)
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i)
        for (int b = 0; b < 8; ++b)
          for (int j = 0; j < 3; ++j)
            dk[(size_t)p + (size_t)np * (a + 8 * (i + 3 * (b + 8 * j)))] =
                t[(size_t)p * 576 + (a * 3 + i) * 24 + b * 3 + j];
  return E3D_OK;
}

int32_t e3d_get_minv(e3d_handle_t* h, double* minv) {
  if (!h || !minv) return E3D_ERR_INPUT;
  if (!h->minv_ready) return E3D_ERR_STATE;
  const long long ns = h->G.ns;
  std::vector<double> t((size_t)6 * ns);
  int32_t rc = get_vec(h, h->minv, t.data(), t.size());
  if (rc) return rc;
  // 6 symmetric planes (00 11 22 01 02 12) -> M_block_inv(ns,3,3)
  const int map[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      std::memcpy(minv + (size_t)ns * (i + 3 * j), t.data() + (size_t)ns * map[i][j], sizeof(double) * ns);
  return E3D_OK;
}

int32_t e3d_get_history(e3d_handle_t* h, double* hist, int32_t n, int32_t* count) {
  if (!h || n < 0) return E3D_ERR_INPUT;
  PcgState S{};
  cudaSetDevice(h->device);
  E3D_CUDA(cudaMemcpy(&S, h->st, sizeof S, cudaMemcpyDeviceToHost));
  const int c = std::max(0, std::min(n, S.it));
  if (c > 0 && hist) E3D_CUDA(cudaMemcpy(hist, h->history, sizeof(double) * c, cudaMemcpyDeviceToHost));
  if (count) *count = c;
  return E3D_OK;
}

int32_t e3d_device_ptrs(e3d_handle_t* h, double** d_u, double** d_g, double** d_b) {
  if (!h) return E3D_ERR_INPUT;
  if (d_u) *d_u = h->u;
  if (d_g) *d_g = h->g;
  if (d_b) *d_b = h->b;
  return E3D_OK;
}

}  // extern "C"

namespace {

// Peak-rate probes: independent FMA chains (8 per thread) so the pipe, not
// latency, limits the rate.  The result is stored so nothing is elided.
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += v[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int32_t run_probe(int device, double* tflops) {
  cudaDeviceProp prop{};
  E3D_CUDA(cudaGetDeviceProperties(&prop, device));
  const int blocks = prop.multiProcessorCount * 8, threads = 256;
  T* out = nullptr;
  E3D_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = sizeof(T) == 8 ? 4096 : 65536;
  fma_probe_kernel<T><<<blocks, threads>>>(out, iters / 16, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  fma_probe_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "probe");
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return E3D_OK;
}

}  // namespace

extern "C" int32_t e3d_probe_peaks(int32_t device, double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return E3D_ERR_INPUT;
  E3D_CUDA(cudaSetDevice(device));
  int32_t rc = run_probe<double>(device, fp64_tflops);
  if (rc) return rc;
  return run_probe<float>(device, fp32_tflops);
}

// ---------------------------------------------------------------------------
// Failure-detection self-test: one kernel whose wait can never be satisfied --
// a two-block grid barrier that block 1 never reaches, or an mbarrier phase
// that expects 16 transaction bytes no copy will deliver -- and that must come
// back through the bounded wait with DEV_TIMEOUT, leaving the context usable.
namespace {

__global__ void selftest_timeout_kernel(int which, GridBarrier* bar, int* err, unsigned long long timeout_ns) {
  if (which == 0) {
    if (blockIdx.x == 1) return;  // the partner that never arrives
    (void)grid_barrier(bar, err, timeout_ns);
  } else {
    __shared__ uint64_t mb;
    if (threadIdx.x == 0) {
      mbar_init(&mb, 1);
      fence_mbar_init();
      mbar_arrive_expect_tx(&mb, 16);  // no copy will complete these bytes
    }
    __syncthreads();
    if (!mbar_wait(&mb, 0, timeout_ns, err) && threadIdx.x == 0) atomicExch(err, DEV_TIMEOUT);
  }
}

}  // namespace

extern "C" int32_t e3d_selftest_timeout(int32_t device, int32_t which, double timeout_s) {
  if ((which != 0 && which != 1) || !(timeout_s > 0.0) || timeout_s > 10.0) return E3D_ERR_INPUT;
  E3D_CUDA(cudaSetDevice(device));
  GridBarrier* bar = nullptr;
  int* err = nullptr;
  E3D_CUDA(cudaMalloc(&bar, sizeof(GridBarrier)));
  E3D_CUDA(cudaMalloc(&err, sizeof(int)));
  E3D_CUDA(cudaMemset(bar, 0, sizeof(GridBarrier)));
  E3D_CUDA(cudaMemset(err, 0, sizeof(int)));
  selftest_timeout_kernel<<<which == 0 ? 2 : 1, 32>>>(which, bar, err, (unsigned long long)(timeout_s * 1e9));
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int derr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&derr, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(bar);
  cudaFree(err);
  if (e != cudaSuccess) return cuda_fail(e, "selftest");
  return derr == DEV_TIMEOUT ? E3D_ERR_TIMEOUT : (derr == DEV_OK ? E3D_OK : E3D_ERR_CUDA);
}

// ---------------------------------------------------------------------------
// Bounds-checked debug build: each translation unit keeps its own record.
int e3d_bounds_take_batch(long long out[4]);    // e3d_batch.cu
int e3d_bounds_take_noalloc(long long out[4]);  // e3d_noalloc.cu

#ifdef E3D_BOUNDS
namespace {
// Thread 5 asks for element 37 of a 32-element buffer; the check sends it to 0.
__global__ void selftest_bounds_kernel(int* buf, int n) {
  const int i = (int)threadIdx.x + (threadIdx.x == 5 ? n : 0);
  buf[E3D_IDX(i, n)] = 1;
}
}  // namespace
#endif

extern "C" int32_t e3d_debug_bounds(int64_t report[5]) {
  if (!report) return E3D_ERR_INPUT;
  long long r[3][4];
  const int k[3] = {e3d::bounds_take(r[0]), e3d_bounds_take_batch(r[1]), e3d_bounds_take_noalloc(r[2])};
  for (int i = 0; i < 5; ++i) report[i] = 0;
  for (int u = 0; u < 3; ++u) {
    if (k[u] < 0) return cuda_fail(cudaGetLastError(), "e3d_debug_bounds");
    if (r[u][0] > 0 && report[0] == 0) {
      report[1] = u;
      report[2] = r[u][1];
      report[3] = r[u][2];
      report[4] = r[u][3];
    }
    report[0] += r[u][0];
  }
  return k[0] == 1 ? E3D_OK : E3D_ERR_STATE;
}

extern "C" int32_t e3d_selftest_bounds(int32_t device) {
#ifdef E3D_BOUNDS
  E3D_CUDA(cudaSetDevice(device));
  int64_t rep[5];
  int32_t rc = e3d_debug_bounds(rep);  // clear
  if (rc) return rc;
  int* buf = nullptr;
  E3D_CUDA(cudaMalloc(&buf, 32 * sizeof(int)));
  selftest_bounds_kernel<<<1, 32>>>(buf, 32);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(e, "selftest_bounds");
  if ((rc = e3d_debug_bounds(rep))) return rc;
  return (rep[0] == 1 && rep[1] == 0 && rep[3] == 37 && rep[4] == 32) ? E3D_OK : E3D_ERR_CUDA;
#else
  (void)device;
  return E3D_ERR_STATE;
#endif
}

// ---------------------------------------------------------------------------
// Checkpoint / resume.  File: 16-byte header "E3DCKPT1" + version, the problem
// dimensions and forms, gg0, the PcgState, then the state arrays and the
// rel_res history (host byte order).
namespace {

struct CkptHeader {
  char magic[8];
  int32_t version, nx, ny, nz, nphase, precision, criterion, preconditioner;
  double gg0;
  PcgState st;
};

template <typename T>
int32_t ckpt_write(FILE* f, const T* dev, size_t count, cudaStream_t s) {
  std::vector<T> buf(count);
  E3D_CUDA(cudaMemcpyAsync(buf.data(), dev, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
  E3D_CUDA(cudaStreamSynchronize(s));
  if (std::fwrite(buf.data(), sizeof(T), count, f) != count) return E3D_ERR_INPUT;
  return E3D_OK;
}

template <typename T>
int32_t ckpt_read(FILE* f, T* dev, size_t count, cudaStream_t s) {
  std::vector<T> buf(count);
  if (std::fread(buf.data(), sizeof(T), count, f) != count) return E3D_ERR_INPUT;
  E3D_CUDA(cudaMemcpyAsync(dev, buf.data(), sizeof(T) * count, cudaMemcpyHostToDevice, s));
  E3D_CUDA(cudaStreamSynchronize(s));
  return E3D_OK;
}

}  // namespace

extern "C" int32_t e3d_checkpoint_save(e3d_handle_t* h, const char* path) {
  E3D_TRACE("e3d_checkpoint_save");
  if (!h || !path) return E3D_ERR_INPUT;
  if (!h->solve_ready) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  const bool mixed = h->prob.precision == E3D_PREC_MIXED;
  if (mixed) {  // u holds the current iterate, du is zero
    int32_t rc = fold_correction(h);
    if (rc) return rc;
  }
  CkptHeader H{};
  std::memcpy(H.magic, "E3DCKPT1", 8);
  H.version = 1;
  H.nx = h->prob.nx;
  H.ny = h->prob.ny;
  H.nz = h->prob.nz;
  H.nphase = h->prob.nphase;
  H.precision = h->prob.precision;
  H.criterion = h->prob.criterion;
  H.preconditioner = h->prob.preconditioner;
  H.gg0 = h->gg0;
  E3D_CUDA(cudaMemcpyAsync(&H.st, h->st, sizeof(PcgState), cudaMemcpyDeviceToHost, h->stream));
  E3D_CUDA(cudaStreamSynchronize(h->stream));
  H.st.since_replace = h->since_replace;
  FILE* f = std::fopen(path, "wb");
  if (!f) return E3D_ERR_INPUT;
  const size_t n3 = 3 * (size_t)h->G.ns;
  int32_t rc = std::fwrite(&H, sizeof H, 1, f) == 1 ? E3D_OK : E3D_ERR_INPUT;
  if (!rc) rc = ckpt_write(f, h->u, n3, h->stream);
  if (!rc) rc = ckpt_write(f, h->g, n3, h->stream);
  if (!mixed) {
    if (!rc) rc = ckpt_write(f, h->z, n3, h->stream);
    if (!rc) rc = ckpt_write(f, H.st.cur ? h->h1 : h->h0, n3, h->stream);
  } else {
    if (!rc) rc = ckpt_write(f, h->g32, n3, h->stream);
    if (!rc) rc = ckpt_write(f, h->z32, n3, h->stream);
    if (!rc) rc = ckpt_write(f, H.st.cur ? h->h32b : h->h32a, n3, h->stream);
  }
  if (!rc && H.st.it > 0) rc = ckpt_write(f, h->history, (size_t)H.st.it, h->stream);
  if (std::fclose(f) != 0 && !rc) rc = E3D_ERR_INPUT;
  return rc;
}

extern "C" int32_t e3d_checkpoint_load(e3d_handle_t* h, const char* path) {
  E3D_TRACE("e3d_checkpoint_load");
  if (!h || !path) return E3D_ERR_INPUT;
  if (!h->femat_done) return E3D_ERR_STATE;
  cudaSetDevice(h->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return E3D_ERR_INPUT;
  CkptHeader H{};
  if (std::fread(&H, sizeof H, 1, f) != 1 || std::memcmp(H.magic, "E3DCKPT1", 8) != 0 || H.version != 1 ||
      H.nx != h->prob.nx || H.ny != h->prob.ny || H.nz != h->prob.nz || H.nphase != h->prob.nphase ||
      H.precision != h->prob.precision || H.criterion != h->prob.criterion ||
      H.preconditioner != h->prob.preconditioner || H.st.it > h->prob.max_iter) {
    std::fclose(f);
    return E3D_ERR_INPUT;
  }
  const bool mixed = h->prob.precision == E3D_PREC_MIXED;
  // preconditioner of this problem (deterministic, so it is rebuilt, not stored)
  bjacobi_kernel<<<blocks_for(h->G.ns, 256), 256, 0, h->stream>>>(
      h->G, h->pix, h->dkd, h->minv, mixed ? h->minv32 : nullptr, h->prob.preconditioner == E3D_PRECOND_NONE);
  E3D_LAUNCHED(h);
  const size_t n3 = 3 * (size_t)h->G.ns;
  PcgState S = H.st;
  int32_t rc = ckpt_read(f, h->u, n3, h->stream);
  if (!rc) rc = ckpt_read(f, h->g, n3, h->stream);
  if (!mixed) {
    if (!rc) rc = ckpt_read(f, h->z, n3, h->stream);
    if (!rc) rc = ckpt_read(f, S.cur ? h->h1 : h->h0, n3, h->stream);
  } else {
    if (!rc) rc = ckpt_read(f, h->g32, n3, h->stream);
    if (!rc) rc = ckpt_read(f, h->z32, n3, h->stream);
    if (!rc) rc = ckpt_read(f, S.cur ? h->h32b : h->h32a, n3, h->stream);
    if (!rc) {
      E3D_CUDA(cudaMemsetAsync(h->du32, 0, sizeof(float) * n3, h->stream));
    }
  }
  if (!rc && S.it > 0) rc = ckpt_read(f, h->history, (size_t)S.it, h->stream);
  std::fclose(f);
  if (rc) return rc;
  E3D_CUDA(cudaMemcpyAsync(h->st, &S, sizeof S, cudaMemcpyHostToDevice, h->stream));
  rc = sync(h);
  if (rc) return rc;
  h->gg0 = H.gg0;
  h->since_replace = S.since_replace;
  h->energy_done = true;
  h->minv_ready = true;
  h->solve_ready = true;
  h->ms_setup = 0.0;
  h->ms_iter = 0.0;
  return E3D_OK;
}
