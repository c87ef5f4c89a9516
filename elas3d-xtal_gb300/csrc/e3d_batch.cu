// Batched ensembles and the continuous-batching server (include/e3d_batch.h),
// both driving the job engine of e3d_jobs.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "e3d_batch.h"
#include "e3d_gpu.h"
#include "e3d_jobs.cuh"
#include "e3d_trace.h"

using namespace e3d;

void e3d_record_error_text(const char* text);
void e3d_record_cuda_error(const char* what, cudaError_t e);

namespace {

#define BCUDA(call)                                  \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) {                         \
      e3d_record_cuda_error(#call, e_);              \
      return E3D_ERR_CUDA;                           \
    }                                                \
  } while (0)

constexpr int kPartChoices[] = {1, 2, 4, 8, 16, 32, 64};
constexpr int kMaxParts = 64;
// Tile depths along z the autotuner tries (0: the rule of job_dims).  Each
// candidate costs two timed launches per size class and k.
constexpr int kTzChoices[] = {0, 32};
constexpr unsigned long long kTimeoutNs = 120ull * 1000000000ull;

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Tiles of one solve run by k parts.  tz_req > 0: z chunks of that many planes
// (the tile shape the autotuner picked); otherwise split z so that there are at
// least ~4 tiles per part, keeping chunks of >= 16 planes (one redundant
// element plane each).
GridDims job_dims(int nx, int ny, int nz, int k, int tz_req = 0) {
  GridDims G{};
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.ns = (long long)nx * ny * nz;
  G.ntx = (nx + TILE_X - 1) / TILE_X;
  G.nty = (ny + TILE_Y - 1) / TILE_Y;
  const long long cols = (long long)G.ntx * G.nty;
  const long long want = 4LL * k;
  int ntz = (int)std::max<long long>(1, std::min<long long>(nz, (want + cols - 1) / cols));
  int tz = (nz + ntz - 1) / ntz;
  if (tz < 16) tz = std::min(nz, 16);
  if (tz_req > 0) tz = std::min(nz, tz_req);
  G.tz = tz;
  G.ntz = (nz + tz - 1) / tz;
  G.ntiles = cols * G.ntz;
  return G;
}

long long halo_doubles(const GridDims& G) { return 3LL * G.ntiles * G.tz * (TILE_X + TILE_Y + 1); }

long long max_halo_doubles(int nx, int ny, int nz) {
  long long m = 0;
  for (int k = 1; k <= kMaxParts; ++k)
    for (int tz : kTzChoices) m = std::max(m, halo_doubles(job_dims(nx, ny, nz, k, tz)));
  return m;
}

JumpParams strain_params(const double s[6]) {  // exx eyy ezz exz eyz exy
  JumpParams J{};
  const double E[3][3] = {{s[0], s[5], s[3]}, {s[5], s[1], s[4]}, {s[3], s[4], s[2]}};
  std::memcpy(J.E, E, sizeof E);
  return J;
}

// Unit load case l in Voigt slot l (xx yy zz xz yz xy) with engineering
// magnitude `mag`: tensor strain components.
void unit_load(int l, double mag, double s[6]) {
  for (int i = 0; i < 6; ++i) s[i] = 0.0;
  s[l] = (l < 3) ? mag : 0.5 * mag;
}

int exit_reason(int status) {
  switch (status) {
    case PCG_CONVERGED: return E3D_EXIT_CONVERGED;
    case PCG_HAH: return E3D_EXIT_HAH_GUARD;
    case PCG_MAXITER: return E3D_EXIT_MAXITER;
    case PCG_BREAKDOWN: return E3D_EXIT_BREAKDOWN;
    case PCG_TIMEOUT: return E3D_EXIT_TIMEOUT;
    default: return E3D_EXIT_RUNNING;
  }
}

// Device memory of one RVE (phase tables, phase map, preconditioner) and of its
// solves, carved from one allocation.
struct RveDev {
  int nx = 0, ny = 0, nz = 0, nphase = 0;
  long long ns = 0;
  int32_t* pix = nullptr;  // 0-based into this RVE's own tables
  double* cmod = nullptr;
  double* cs64 = nullptr;
  float* cs32 = nullptr;
  double* dk = nullptr;
  double* dkd = nullptr;
  float* minv32 = nullptr;
  PhaseMat* mats = nullptr;
};

struct JobDev {
  JobDesc d{};
  long long halo_cap = 0;
  int rve = 0, load_case = -1;
};

size_t rve_bytes(long long ns, int nphase) {
  return align256(4 * ns) + align256(8 * 36 * (size_t)nphase) + align256(8 * kCsStride * (size_t)nphase) +
         align256(4 * kCs32Stride * (size_t)nphase) + align256(8 * 576 * (size_t)nphase) +
         align256(8 * 72 * (size_t)nphase) + align256(4 * 6 * ns) + align256(sizeof(PhaseMat) * (size_t)nphase);
}

size_t job_bytes(int nx, int ny, int nz, int nphase) {
  const long long ns = (long long)nx * ny * nz, n3 = 3 * ns;
  return 3 * align256(8 * n3) + 6 * align256(4 * n3) + align256(8 * max_halo_doubles(nx, ny, nz)) +
         align256(8 * 6 * (size_t)nphase) +
         align256(8 * kJobSlots * kMaxParts) + align256(sizeof(GridBarrier)) + align256(sizeof(PcgState)) + align256(4) +
         align256(sizeof(JobResult));
}

template <typename T>
T* carve(char*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  p += align256(sizeof(T) * count);
  return r;
}

// Fills the RVE's device tables: upload pix (to 0-based), phase materials,
// phase kernel, block-Jacobi.  `base` must hold rve_bytes().  checked: the phase
// ids were range-checked already (at submission), so the map is copied as it is
// and made 0-based on the device.
int32_t setup_rve(RveDev& R, char* base, const e3d_rve_t& in, double e1, double nu1, cudaStream_t s,
                  std::vector<int32_t>& scratch, bool checked = false) {
  R.nx = in.nx;
  R.ny = in.ny;
  R.nz = in.nz;
  R.nphase = in.ngrains + 1;
  R.ns = (long long)in.nx * in.ny * in.nz;
  char* p = base;
  R.pix = carve<int32_t>(p, R.ns);
  R.cmod = carve<double>(p, 36 * (size_t)R.nphase);
  R.cs64 = carve<double>(p, kCsStride * (size_t)R.nphase);
  R.cs32 = carve<float>(p, kCs32Stride * (size_t)R.nphase);
  R.dk = carve<double>(p, 576 * (size_t)R.nphase);
  R.dkd = carve<double>(p, 72 * (size_t)R.nphase);
  R.minv32 = carve<float>(p, 6 * R.ns);
  R.mats = carve<PhaseMat>(p, R.nphase);
  if (!checked) {
    scratch.resize((size_t)R.ns);
    for (long long m = 0; m < R.ns; ++m) {
      const int v = in.pix[m];
      if (v < 1 || v > R.nphase) return E3D_ERR_INPUT;
      scratch[(size_t)m] = v - 1;
    }
  }
  std::vector<PhaseMat> mats((size_t)R.nphase);
  for (int g = 0; g < R.nphase; ++g) {
    PhaseMat& M = mats[(size_t)g];
    M.c11 = in.c11;
    M.c12 = in.c12;
    M.c44 = in.c44;
    M.pore = (g == R.nphase - 1);
    M.K1 = e1 / 3.0 / (1.0 - 2.0 * nu1);
    M.G1 = e1 / 2.0 / (1.0 + nu1);
    for (int d = 0; d < 3; ++d) M.r[d] = M.pore ? 0.0 : in.rodrigues[3 * g + d];
  }
  if (checked) {
    BCUDA(cudaMemcpyAsync(R.pix, in.pix, 4 * R.ns, cudaMemcpyHostToDevice, s));
    pix_to_zero_based_kernel<<<(unsigned)((R.ns + 255) / 256), 256, 0, s>>>(R.ns, R.nphase, R.pix, nullptr);
  } else {
    BCUDA(cudaMemcpyAsync(R.pix, scratch.data(), 4 * R.ns, cudaMemcpyHostToDevice, s));
  }
  BCUDA(cudaMemcpyAsync(R.mats, mats.data(), sizeof(PhaseMat) * mats.size(), cudaMemcpyHostToDevice, s));
  batch_phase_kernel<<<R.nphase, 32, 0, s>>>(R.mats, R.nphase, R.cmod, R.cs64, R.cs32, R.dk, R.dkd);
  GridDims G = job_dims(R.nx, R.ny, R.nz, 1);
  bjacobi_kernel<<<(unsigned)((R.ns + 255) / 256), 256, 0, s>>>(G, R.pix, R.dkd, nullptr, R.minv32);
  BCUDA(cudaGetLastError());
  // the host copies above read `scratch`/`mats`: finish before they go away
  BCUDA(cudaStreamSynchronize(s));
  return E3D_OK;
}

void fill_job(JobDev& J, const RveDev& R, char*& p, const double strain[6], int max_iter, int refine, int crit,
              int divreset, float tol) {
  const long long ns = R.ns, n3 = 3 * ns;
  JobDesc& d = J.d;
  d = JobDesc{};
  d.J = strain_params(strain);
  d.pix = R.pix;
  d.cs32 = R.cs32;
  d.cs64 = R.cs64;
  d.dk = R.dk;
  d.cmod = R.cmod;
  d.nphase_total = R.nphase;
  d.minv32 = R.minv32;
  d.u = carve<double>(p, n3);
  d.g = carve<double>(p, n3);
  d.b = carve<double>(p, n3);
  d.du = carve<float>(p, n3);
  d.g32 = carve<float>(p, n3);
  d.z32 = carve<float>(p, n3);
  d.h0 = carve<float>(p, n3);
  d.h1 = carve<float>(p, n3);
  d.Ah = carve<float>(p, n3);
  d.sig = carve<double>(p, 6 * (size_t)R.nphase);
  J.halo_cap = max_halo_doubles(R.nx, R.ny, R.nz);
  double* halo = carve<double>(p, (size_t)J.halo_cap);
  d.hx = halo;  // split per k in set_parts
  d.partial = carve<double>(p, (size_t)kJobSlots * kMaxParts);
  d.bar = carve<GridBarrier>(p, 1);
  d.st = carve<PcgState>(p, 1);
  d.stage = carve<int>(p, 1);
  d.out = carve<JobResult>(p, 1);
  d.max_iter = max_iter;
  d.refine_every = refine;
  d.criterion = crit;
  d.divergence_reset = divreset;
  d.tol = tol;
}

void set_parts(JobDev& J, const RveDev& R, int k, int tz_req = 0) {
  JobDesc& d = J.d;
  d.G = job_dims(R.nx, R.ny, R.nz, k, tz_req);
  d.nparts = k;
  const long long h = (long long)d.G.ntiles * d.G.tz;
  double* base = d.hx;
  d.hy = base + 3 * h * TILE_Y;
  d.hd = d.hy + 3 * h * TILE_X;
}

int default_parts(long long ns) {
  // about 128K nodes per block, at most kMaxParts blocks per solve
  int k = 1;
  while (k < kMaxParts && ns > (long long)k * 131072) k *= 2;
  return k;
}

struct Engine {
  int grid = 0;
  JobDesc* d_jobs = nullptr;
  int* d_part_job = nullptr;
  int* d_part_rank = nullptr;
  unsigned int* d_head = nullptr;
  int* d_err = nullptr;
  int cap_jobs = 0, cap_parts = 0;

  int32_t init(int device) {
    int per_sm = 0, sms = 0;
    BCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    BCUDA(cudaFuncSetAttribute(job_engine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kEngineDynSmem));
    BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, job_engine_kernel, NT, kEngineDynSmem));
    if (per_sm < 1) return E3D_ERR_CUDA;
    grid = per_sm * sms;
    BCUDA(cudaMalloc(&d_head, 256));
    BCUDA(cudaMalloc(&d_err, 256));
    return E3D_OK;
  }
  int32_t reserve(int njobs, int nparts) {
    if (njobs > cap_jobs) {
      if (d_jobs) cudaFree(d_jobs);
      cap_jobs = std::max(njobs, 2 * cap_jobs);
      BCUDA(cudaMalloc(&d_jobs, sizeof(JobDesc) * cap_jobs));
    }
    if (nparts > cap_parts) {
      if (d_part_job) cudaFree(d_part_job);
      if (d_part_rank) cudaFree(d_part_rank);
      cap_parts = std::max(nparts, 2 * cap_parts);
      BCUDA(cudaMalloc(&d_part_job, sizeof(int) * cap_parts));
      BCUDA(cudaMalloc(&d_part_rank, sizeof(int) * cap_parts));
    }
    return E3D_OK;
  }
  void release() {
    for (void* q : {(void*)d_jobs, (void*)d_part_job, (void*)d_part_rank, (void*)d_head, (void*)d_err})
      if (q) cudaFree(q);
    d_jobs = nullptr;
    d_part_job = d_part_rank = nullptr;
    d_head = nullptr;
    d_err = nullptr;
  }
  // Uploads jobs (in the given order) and the part list; stages are left as they are.
  int32_t upload(const std::vector<JobDesc>& jobs, cudaStream_t s, int* nparts_total) {
    std::vector<int> pj, pr;
    for (size_t j = 0; j < jobs.size(); ++j)
      for (int p = 0; p < jobs[j].nparts; ++p) {
        pj.push_back((int)j);
        pr.push_back(p);
      }
    int32_t rc = reserve((int)jobs.size(), (int)pj.size());
    if (rc) return rc;
    BCUDA(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(JobDesc) * jobs.size(), cudaMemcpyHostToDevice, s));
    BCUDA(cudaMemcpyAsync(d_part_job, pj.data(), sizeof(int) * pj.size(), cudaMemcpyHostToDevice, s));
    BCUDA(cudaMemcpyAsync(d_part_rank, pr.data(), sizeof(int) * pr.size(), cudaMemcpyHostToDevice, s));
    BCUDA(cudaStreamSynchronize(s));
    *nparts_total = (int)pj.size();
    return E3D_OK;
  }
  // Resets dispenser, error flag and the jobs' barriers (and stages when
  // reset_stage), then launches the persistent engine.
  int32_t launch(int njobs, int nparts_total, int it_limit, int reset_stage, cudaStream_t s) {
    BCUDA(cudaMemsetAsync(d_head, 0, 4, s));
    BCUDA(cudaMemsetAsync(d_err, 0, 4, s));
    reset_jobs_kernel<<<(njobs + 127) / 128, 128, 0, s>>>(d_jobs, njobs, reset_stage);
    EngineArgs E{};
    E.jobs = d_jobs;
    E.part_job = d_part_job;
    E.part_rank = d_part_rank;
    E.nparts_total = nparts_total;
    E.njobs = njobs;
    E.head = d_head;
    E.err = d_err;
    E.it_limit = it_limit;
    E.timeout_ns = kTimeoutNs;
    job_engine_kernel<<<grid, NT, kEngineDynSmem, s>>>(E);
    BCUDA(cudaGetLastError());
    return E3D_OK;
  }
};

}  // namespace

// ============================================================== batch
struct e3d_batch {
  e3d_batch_opts_t opts{};
  int device = 0;
  cudaStream_t stream = nullptr;
  void* pool = nullptr;
  size_t pool_bytes = 0;
  std::vector<RveDev> rves;
  std::vector<JobDev> jobs;   // solve order (largest first)
  std::vector<int> order;     // result slot for each solve in `jobs`
  std::vector<JobDesc> descs;
  Engine eng;
  int nparts_total = 0;
  int it_all = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<JobResult> results;
};

namespace {

int32_t batch_time_job(e3d_batch* b, size_t j, int k, int tz_req, int iters, float* ms) {
  JobDev J = b->jobs[j];
  set_parts(J, b->rves[(size_t)J.rve], k, tz_req);
  std::vector<JobDesc> one{J.d};
  int np = 0;
  int32_t rc = b->eng.upload(one, b->stream, &np);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  BCUDA(cudaEventCreate(&e0));
  BCUDA(cudaEventCreate(&e1));
  BCUDA(cudaEventRecord(e0, b->stream));
  rc = b->eng.launch(1, np, iters, 1, b->stream);
  BCUDA(cudaEventRecord(e1, b->stream));
  BCUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  return rc;
}

// Autotuner: per size class (node count within a factor of two), time the
// engine on one representative solve for each candidate schedule -- blocks per
// solve k and tile shape (element planes per tile, kTzChoices) -- as set-up + 10
// iterations minus set-up + 2; keep the fastest tile shape per k, then choose k
// per class to minimise the estimated makespan max(total block-time / resident
// blocks, longest solve).
int32_t batch_autotune(e3d_batch* b, std::vector<int>& kjob, std::vector<int>& tzjob) {
  std::map<int, std::vector<size_t>> cls;  // log2(ns) -> solves
  for (size_t j = 0; j < b->jobs.size(); ++j) {
    const long long ns = b->rves[(size_t)b->jobs[j].rve].ns;
    cls[(int)std::floor(std::log2((double)ns))].push_back(j);
  }
  struct C {
    std::vector<int> ks, tzs;  // per k: the fastest tile depth
    std::vector<double> t;     // ms per iteration per solve
    int pick = 0;
    size_t n = 0;
  };
  std::map<int, C> cc;
  for (auto& kv : cls) {
    C c;
    c.n = kv.second.size();
    const size_t rep = kv.second.front();
    const RveDev& R = b->rves[(size_t)b->jobs[rep].rve];
    for (int k : kPartChoices) {
      const GridDims G = job_dims(R.nx, R.ny, R.nz, k);
      if (k > 1 && G.ntiles < 2LL * k) break;  // too few tiles to share
      double best_t = 1e300;
      int best_tz = 0;
      for (int tz : kTzChoices) {
        const GridDims Gt = job_dims(R.nx, R.ny, R.nz, k, tz);
        if (tz > 0 && (Gt.tz == G.tz || Gt.ntiles < (long long)k)) continue;  // same shape, or too few tiles
        float t2 = 0.f, t10 = 0.f;
        int32_t rc = batch_time_job(b, rep, k, tz, 2, &t2);
        if (!rc) rc = batch_time_job(b, rep, k, tz, 10, &t10);
        if (rc) return rc;
        const double t = std::max(1e-6, (double)(t10 - t2) / 8.0);
        if (t < best_t) {
          best_t = t;
          best_tz = tz;
        }
      }
      c.ks.push_back(k);
      c.tzs.push_back(best_tz);
      c.t.push_back(best_t);
    }
    // start from the most block-efficient choice
    size_t best = 0;
    for (size_t i = 1; i < c.ks.size(); ++i)
      if (c.ks[i] * c.t[i] < c.ks[best] * c.t[best]) best = i;
    c.pick = (int)best;
    cc[kv.first] = c;
  }
  const double B = b->eng.grid;
  for (int guard = 0; guard < 64; ++guard) {
    double total = 0.0, longest = 0.0;
    int arg = -1;
    for (auto& kv : cc) {
      const C& c = kv.second;
      total += c.n * c.ks[(size_t)c.pick] * c.t[(size_t)c.pick];
      if (c.t[(size_t)c.pick] > longest) {
        longest = c.t[(size_t)c.pick];
        arg = kv.first;
      }
    }
    C& c = cc[arg];
    if (longest <= total / B || (size_t)c.pick + 1 >= c.ks.size()) break;
    c.pick += 1;  // split the longest solves over more blocks
  }
  kjob.assign(b->jobs.size(), 1);
  tzjob.assign(b->jobs.size(), 0);
  for (auto& kv : cls)
    for (size_t j : kv.second) {
      const C& c = cc[kv.first];
      kjob[j] = c.ks[(size_t)c.pick];
      tzjob[j] = c.tzs[(size_t)c.pick];
    }
  return E3D_OK;
}

}  // namespace

extern "C" {

void e3d_batch_opts_defaults(e3d_batch_opts_t* o) {
  std::memset(o, 0, sizeof *o);
  o->device = 0;
  o->max_iter = 10000;
  o->refine_every = 50;
  o->criterion = E3D_CRIT_REF;
  o->divergence_reset = 1;
  o->tol = 1.0e-8f;
  o->load_cases = 0;
  o->parts = 0;
  o->strain = 1.0e-3;
  o->e1 = 0.0;
  o->nu1 = 0.0;
  o->hbm_budget = 0;
}

int32_t e3d_batch_destroy(e3d_batch_t* b) {
  if (!b) return E3D_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->eng.release();
  if (b->pool) cudaFree(b->pool);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return E3D_OK;
}

int32_t e3d_batch_create(e3d_batch_t** out, const e3d_rve_t* rves, int32_t n, const e3d_batch_opts_t* o) {
  E3D_TRACE("e3d_batch_create");
  if (!out || !rves || n < 1 || !o) return E3D_ERR_INPUT;
  *out = nullptr;
  const int mask = o->load_cases ? o->load_cases : 0x3f;
  if (mask & ~0x3f) return E3D_ERR_INPUT;
  for (int r = 0; r < n; ++r) {
    const e3d_rve_t& R = rves[r];
    if (R.nx < 1 || R.ny < 1 || R.nz < 1 || R.ngrains < 1 || !R.pix || !R.rodrigues) return E3D_ERR_INPUT;
  }
  e3d_batch* b = new e3d_batch();
  b->opts = *o;
  b->device = o->device;
  auto fail = [&](int32_t rc) {
    e3d_batch_destroy(b);
    return rc;
  };
  if (cudaSetDevice(b->device) != cudaSuccess) return fail(E3D_ERR_INPUT);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(E3D_ERR_CUDA);
  int32_t rc = b->eng.init(b->device);
  if (rc) return fail(rc);
  // memory plan
  size_t total = 0;
  std::vector<int> cases;
  for (int l = 0; l < 6; ++l)
    if (mask & (1 << l)) cases.push_back(l);
  for (int r = 0; r < n; ++r) {
    const e3d_rve_t& R = rves[r];
    total += rve_bytes((long long)R.nx * R.ny * R.nz, R.ngrains + 1);
    total += cases.size() * job_bytes(R.nx, R.ny, R.nz, R.ngrains + 1);
  }
  if (o->hbm_budget > 0 && (int64_t)total > o->hbm_budget) return fail(E3D_ERR_OOM);
  if (cudaMalloc(&b->pool, total) != cudaSuccess) {
    cudaGetLastError();
    return fail(E3D_ERR_OOM);
  }
  b->pool_bytes = total;
  char* p = static_cast<char*>(b->pool);
  std::vector<int32_t> scratch;
  b->rves.resize((size_t)n);
  for (int r = 0; r < n; ++r) {
    RveDev& R = b->rves[(size_t)r];
    char* base = p;
    p += rve_bytes((long long)rves[r].nx * rves[r].ny * rves[r].nz, rves[r].ngrains + 1);
    if ((rc = setup_rve(R, base, rves[r], o->e1, o->nu1, b->stream, scratch))) return fail(rc);
  }
  // solves, largest first (in-order dispensing then fills the tail with small ones)
  std::vector<std::pair<long long, std::pair<int, int>>> list;
  for (int r = 0; r < n; ++r)
    for (int l : cases) list.push_back({b->rves[(size_t)r].ns, {r, l}});
  std::stable_sort(list.begin(), list.end(), [](auto& a, auto& c) { return a.first > c.first; });
  std::vector<int> slot_of;  // result slot = r * ncases + case index
  for (auto& it : list) {
    JobDev J;
    J.rve = it.second.first;
    J.load_case = it.second.second;
    double s[6];
    unit_load(J.load_case, o->strain, s);
    fill_job(J, b->rves[(size_t)J.rve], p, s, o->max_iter, o->refine_every, o->criterion, o->divergence_reset,
             o->tol);
    set_parts(J, b->rves[(size_t)J.rve], 1);
    b->jobs.push_back(J);
    const int ci = (int)(std::find(cases.begin(), cases.end(), J.load_case) - cases.begin());
    b->order.push_back(J.rve * (int)cases.size() + ci);
  }
  // blocks per solve
  std::vector<int> kjob(b->jobs.size(), 1), tzjob(b->jobs.size(), 0);
  if (o->parts > 0) {
    for (size_t j = 0; j < b->jobs.size(); ++j) kjob[j] = std::min(o->parts, kMaxParts);
  } else if ((rc = batch_autotune(b, kjob, tzjob))) {
    return fail(rc);
  }
  for (size_t j = 0; j < b->jobs.size(); ++j) {
    set_parts(b->jobs[j], b->rves[(size_t)b->jobs[j].rve], std::min(kjob[j], b->eng.grid), tzjob[j]);
    b->descs.push_back(b->jobs[j].d);
  }
  if ((rc = b->eng.upload(b->descs, b->stream, &b->nparts_total))) return fail(rc);
  // capture the solve: reset stages, then one persistent launch
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail(E3D_ERR_CUDA);
  rc = b->eng.launch((int)b->descs.size(), b->nparts_total, o->max_iter, 1, b->stream);
  cudaError_t ce = cudaStreamEndCapture(b->stream, &b->graph);
  if (rc) return fail(rc);
  if (ce != cudaSuccess) {
    e3d_record_cuda_error("cudaStreamEndCapture", ce);
    return fail(E3D_ERR_CUDA);
  }
  if ((ce = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) {
    e3d_record_cuda_error("cudaGraphInstantiate", ce);
    return fail(E3D_ERR_CUDA);
  }
  b->results.resize(b->jobs.size());
  *out = b;
  return E3D_OK;
}

int32_t e3d_batch_solve(e3d_batch_t* b, double* ceff, double* seconds) {
  E3D_TRACE("e3d_batch_solve");
  if (!b) return E3D_ERR_INPUT;
  cudaSetDevice(b->device);
  cudaEvent_t e0, e1;
  BCUDA(cudaEventCreate(&e0));
  BCUDA(cudaEventCreate(&e1));
  BCUDA(cudaEventRecord(e0, b->stream));
  BCUDA(cudaGraphLaunch(b->exec, b->stream));
  BCUDA(cudaEventRecord(e1, b->stream));
  BCUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (seconds) *seconds = ms * 1e-3;
  for (size_t j = 0; j < b->jobs.size(); ++j)
    BCUDA(cudaMemcpyAsync(&b->results[j], b->jobs[j].d.out, sizeof(JobResult), cudaMemcpyDeviceToHost, b->stream));
  int err = 0;
  BCUDA(cudaMemcpyAsync(&err, b->eng.d_err, 4, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaStreamSynchronize(b->stream));
  if (ceff) {
    const int n = (int)b->rves.size();
    std::fill(ceff, ceff + 36 * (size_t)n, NAN);
    for (size_t j = 0; j < b->jobs.size(); ++j) {
      const JobDev& J = b->jobs[j];
      for (int i = 0; i < 6; ++i) ceff[36 * (size_t)J.rve + 6 * i + J.load_case] = b->results[j].strav[i] / b->opts.strain;
    }
  }
  if (err == DEV_TIMEOUT) return E3D_ERR_TIMEOUT;
  for (const JobResult& r : b->results) {
    if (r.status == PCG_BREAKDOWN) return E3D_ERR_BREAKDOWN;
    if (r.status == PCG_TIMEOUT) return E3D_ERR_TIMEOUT;
  }
  for (const JobResult& r : b->results)
    if (r.status == PCG_MAXITER) return E3D_ERR_MAXITER;
  return E3D_OK;
}

int32_t e3d_batch_results(e3d_batch_t* b, e3d_job_result_t* out, int32_t capacity, int32_t* count) {
  if (!b) return E3D_ERR_INPUT;
  const int nj = (int)b->jobs.size();
  if (count) *count = nj;
  if (!out) return E3D_OK;
  if (capacity < nj) return E3D_ERR_INPUT;
  for (int j = 0; j < nj; ++j) {
    const JobResult& r = b->results[(size_t)j];
    e3d_job_result_t& o = out[b->order[(size_t)j]];
    std::memset(&o, 0, sizeof o);
    o.rve = b->jobs[(size_t)j].rve;
    o.load_case = b->jobs[(size_t)j].load_case;
    o.status = exit_reason(r.status);
    o.iterations = r.iterations;
    o.refinements = r.refinements;
    o.resets = r.resets;
    o.parts = b->jobs[(size_t)j].d.nparts;
    o.tile_z = b->jobs[(size_t)j].d.G.tz;
    o.utot0 = r.utot0;
    o.utot = r.utot;
    o.rel_res = r.rel_res;
    o.true_rel = r.true_rel;
    for (int i = 0; i < 6; ++i) {
      o.strav[i] = r.strav[i];
      o.epsav[i] = r.epsav[i];
    }
  }
  return E3D_OK;
}

int32_t e3d_batch_parts(e3d_batch_t* b, int32_t* parts, int32_t capacity) {
  if (!b || !parts || capacity < (int)b->jobs.size()) return E3D_ERR_INPUT;
  for (size_t j = 0; j < b->jobs.size(); ++j) parts[b->order[j]] = b->jobs[j].d.nparts;
  return E3D_OK;
}

}  // extern "C"

// ============================================================== server
struct ServeJob {
  int64_t id = 0;
  int parts = 1;  // blocks per solve, fixed at admission
  e3d_rve_t rve{};
  std::vector<int32_t> pix;
  std::vector<double> rod;
  double strain[6] = {0};
  size_t bytes = 0;
  void* mem = nullptr;
  RveDev R;
  JobDev J;
  std::chrono::steady_clock::time_point t_submit;
  bool done = false;
  e3d_job_result_t result{};
};

struct e3d_server {
  e3d_serve_opts_t opts{};
  int device = 0;
  cudaStream_t stream = nullptr;
  Engine eng;
  int64_t next_id = 1;
  std::deque<ServeJob*> queue;
  std::vector<ServeJob*> active;
  std::map<int64_t, ServeJob*> finished;
  int64_t bytes_now = 0, bytes_peak = 0;
  std::vector<int32_t> scratch;
};

// Nodes per block the serving loop aims at when it splits a solve into parts.
#ifndef E3D_SERVE_BLOCK_NODES
#define E3D_SERVE_BLOCK_NODES 131072
#endif

// Iterations per round of one solve: round_iters, or with round balancing
// round_iters x (target nodes per block / this solve's nodes per block), within
// [1, 8] x round_iters, so that a small solve's block is not left idle while
// the large solves' blocks finish the round.  A function of the solve alone:
// its results do not depend on what else is on the device.
int serve_round_iters(const e3d_serve_opts_t& o, long long ns, int k) {
  if (!o.round_balance) return o.round_iters;
  const double per_block = (double)ns / k;
  const double f = std::min(8.0, std::max(1.0, (double)E3D_SERVE_BLOCK_NODES / per_block));
  return (int)std::min<double>(2.0e9, std::floor(o.round_iters * f));
}

extern "C" {

void e3d_serve_opts_defaults(e3d_serve_opts_t* o) {
  std::memset(o, 0, sizeof *o);
  o->device = 0;
  o->max_iter = 10000;
  o->refine_every = 50;
  o->criterion = E3D_CRIT_REF;
  o->divergence_reset = 1;
  o->tol = 1.0e-8f;
  o->max_active = 64;
  o->round_iters = 50;
  o->parts = 0;
  o->round_balance = 0;
  o->hbm_budget = 0;
}

int32_t e3d_serve_create(e3d_server_t** out, const e3d_serve_opts_t* o) {
  if (!out || !o || o->max_active < 1 || o->round_iters < 1) return E3D_ERR_INPUT;
  *out = nullptr;
  e3d_server* s = new e3d_server();
  s->opts = *o;
  s->device = o->device;
  if (cudaSetDevice(s->device) != cudaSuccess || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return E3D_ERR_CUDA;
  }
  int32_t rc = s->eng.init(s->device);
  if (rc) {
    e3d_serve_destroy(s);
    return rc;
  }
  *out = s;
  return E3D_OK;
}

int32_t e3d_serve_destroy(e3d_server_t* s) {
  if (!s) return E3D_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  auto drop = [&](ServeJob* j) {
    if (j->mem) cudaFreeAsync(j->mem, s->stream);
    delete j;
  };
  for (ServeJob* j : s->queue) drop(j);
  for (ServeJob* j : s->active) drop(j);
  for (auto& kv : s->finished) drop(kv.second);
  if (s->stream) cudaStreamSynchronize(s->stream);
  s->eng.release();
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return E3D_OK;
}

int32_t e3d_serve_submit(e3d_server_t* s, const e3d_rve_t* rve, const double strain[6], int64_t* id) {
  if (!s || !rve || !strain || !rve->pix || !rve->rodrigues || rve->nx < 1 || rve->ny < 1 || rve->nz < 1 ||
      rve->ngrains < 1)
    return E3D_ERR_INPUT;
  const long long ns = (long long)rve->nx * rve->ny * rve->nz;
  // the phase-id range check of ppixel_hdf5 (src/elas3dxtal_pcg.f90:2986-2989),
  // at submission so that a bad request is refused before it takes a slot; the
  // server keeps its own copy of the map, checked as it is copied
  ServeJob* j = new ServeJob();
  j->pix.assign(rve->pix, rve->pix + ns);
  const int32_t hi = rve->ngrains + 1;
  for (const int32_t v : j->pix)
    if (v < 1 || v > hi) {
      delete j;
      return E3D_ERR_INPUT;
    }
  j->id = s->next_id++;
  j->rve = *rve;
  j->rod.assign(rve->rodrigues, rve->rodrigues + 3 * (size_t)rve->ngrains);
  j->rve.pix = j->pix.data();
  j->rve.rodrigues = j->rod.data();
  std::memcpy(j->strain, strain, sizeof j->strain);
  j->bytes = rve_bytes(ns, rve->ngrains + 1) + job_bytes(rve->nx, rve->ny, rve->nz, rve->ngrains + 1);
  if (s->opts.hbm_budget > 0 && (int64_t)j->bytes > s->opts.hbm_budget) {
    delete j;
    return E3D_ERR_OOM;  // could never be admitted
  }
  j->t_submit = std::chrono::steady_clock::now();
  s->queue.push_back(j);
  if (id) *id = j->id;
  return E3D_OK;
}

int32_t e3d_serve_step(e3d_server_t* s, int32_t* pending) {
  E3D_TRACE("e3d_serve_step");
  if (!s) return E3D_ERR_INPUT;
  cudaSetDevice(s->device);
  // admit in arrival order while slots and budget allow
  while (!s->queue.empty() && (int)s->active.size() < s->opts.max_active) {
    ServeJob* j = s->queue.front();
    if (s->opts.hbm_budget > 0 && s->bytes_now + (int64_t)j->bytes > s->opts.hbm_budget) break;
    {
      const long long ns_j = (long long)j->rve.nx * j->rve.ny * j->rve.nz;
      const int kk = s->opts.parts > 0 ? std::min(s->opts.parts, kMaxParts) : default_parts(ns_j);
      j->parts = std::min(kk, s->eng.grid);
    }
    cudaError_t e = cudaMallocAsync(&j->mem, j->bytes, s->stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      break;  // the device is full: wait for retirements
    }
    s->queue.pop_front();
    s->bytes_now += (int64_t)j->bytes;
    s->bytes_peak = std::max(s->bytes_peak, s->bytes_now);
    char* p = static_cast<char*>(j->mem);
    const long long ns = (long long)j->rve.nx * j->rve.ny * j->rve.nz;
    char* base = p;
    p += rve_bytes(ns, j->rve.ngrains + 1);
    int32_t rc = setup_rve(j->R, base, j->rve, s->opts.e1, s->opts.nu1, s->stream, s->scratch, true);
    if (rc) {
      j->done = true;
      j->result.status = E3D_EXIT_BREAKDOWN;
      cudaFreeAsync(j->mem, s->stream);
      j->mem = nullptr;
      s->bytes_now -= (int64_t)j->bytes;
      s->finished[j->id] = j;
      continue;
    }
    fill_job(j->J, j->R, p, j->strain, s->opts.max_iter, s->opts.refine_every, s->opts.criterion,
             s->opts.divergence_reset, s->opts.tol);
    set_parts(j->J, j->R, j->parts);
    j->J.d.it_round = serve_round_iters(s->opts, ns, j->parts);
    BCUDA(cudaMemsetAsync(j->J.d.stage, 0, 4, s->stream));
    s->active.push_back(j);
  }
  if (!s->active.empty()) {
    // largest solves first: their parts start early and the round's tail is
    // filled with small ones
    std::stable_sort(s->active.begin(), s->active.end(),
                     [](const ServeJob* a, const ServeJob* c) { return a->R.ns > c->R.ns; });
    std::vector<JobDesc> descs;
    for (ServeJob* j : s->active) descs.push_back(j->J.d);
    int np = 0;
    int32_t rc = s->eng.upload(descs, s->stream, &np);
    if (rc) return rc;
    if ((rc = s->eng.launch((int)descs.size(), np, s->opts.round_iters, 0, s->stream))) return rc;
    BCUDA(cudaStreamSynchronize(s->stream));
    const auto now = std::chrono::steady_clock::now();
    std::vector<ServeJob*> still;
    for (ServeJob* j : s->active) {
      int stage = 0;
      BCUDA(cudaMemcpy(&stage, j->J.d.stage, 4, cudaMemcpyDeviceToHost));
      if (stage != JOB_DONE) {
        still.push_back(j);
        continue;
      }
      JobResult r{};
      BCUDA(cudaMemcpy(&r, j->J.d.out, sizeof r, cudaMemcpyDeviceToHost));
      e3d_job_result_t& o = j->result;
      std::memset(&o, 0, sizeof o);
      o.rve = -1;
      o.load_case = -1;
      o.status = exit_reason(r.status);
      o.iterations = r.iterations;
      o.refinements = r.refinements;
      o.resets = r.resets;
      o.parts = j->J.d.nparts;
      o.tile_z = j->J.d.G.tz;
      o.utot0 = r.utot0;
      o.utot = r.utot;
      o.rel_res = r.rel_res;
      o.true_rel = r.true_rel;
      for (int i = 0; i < 6; ++i) {
        o.strav[i] = r.strav[i];
        o.epsav[i] = r.epsav[i];
      }
      o.seconds = std::chrono::duration<double>(now - j->t_submit).count();
      j->done = true;
      cudaFreeAsync(j->mem, s->stream);
      j->mem = nullptr;
      s->bytes_now -= (int64_t)j->bytes;
      j->pix.clear();
      j->pix.shrink_to_fit();
      s->finished[j->id] = j;
    }
    s->active.swap(still);
  }
  if (pending) *pending = (int32_t)(s->queue.size() + s->active.size());
  return E3D_OK;
}

int32_t e3d_serve_result(e3d_server_t* s, int64_t id, e3d_job_result_t* out) {
  if (!s || !out) return E3D_ERR_INPUT;
  auto it = s->finished.find(id);
  if (it == s->finished.end()) return E3D_ERR_STATE;
  *out = it->second->result;
  return E3D_OK;
}

int32_t e3d_serve_cancel(e3d_server_t* s, int64_t id) {
  E3D_TRACE("e3d_serve_cancel");
  if (!s) return E3D_ERR_INPUT;
  if (s->finished.count(id)) return E3D_ERR_STATE;
  cudaSetDevice(s->device);
  auto finish = [&](ServeJob* j, int iterations) {
    e3d_job_result_t& o = j->result;
    std::memset(&o, 0, sizeof o);
    o.rve = -1;
    o.load_case = -1;
    o.status = E3D_EXIT_CANCELLED;
    o.iterations = iterations;
    o.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - j->t_submit).count();
    j->done = true;
    j->pix.clear();
    j->pix.shrink_to_fit();
    s->finished[j->id] = j;
  };
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
    if ((*it)->id == id) {
      ServeJob* j = *it;
      s->queue.erase(it);
      finish(j, 0);
      return E3D_OK;
    }
  for (auto it = s->active.begin(); it != s->active.end(); ++it)
    if ((*it)->id == id) {
      ServeJob* j = *it;
      PcgState st{};
      BCUDA(cudaMemcpyAsync(&st, j->J.d.st, sizeof st, cudaMemcpyDeviceToHost, s->stream));
      BCUDA(cudaStreamSynchronize(s->stream));
      int stage = 0;
      BCUDA(cudaMemcpy(&stage, j->J.d.stage, 4, cudaMemcpyDeviceToHost));
      BCUDA(cudaFreeAsync(j->mem, s->stream));
      j->mem = nullptr;
      s->bytes_now -= (int64_t)j->bytes;
      s->active.erase(it);
      finish(j, stage == JOB_NEW ? 0 : st.it);
      return E3D_OK;
    }
  return E3D_ERR_INPUT;
}

int32_t e3d_serve_memory(e3d_server_t* s, int64_t* now, int64_t* peak) {
  if (!s) return E3D_ERR_INPUT;
  if (now) *now = s->bytes_now;
  if (peak) *peak = s->bytes_peak;
  return E3D_OK;
}

}  // extern "C"

// Bounds-checked build: this translation unit's record (read by e3d_debug_bounds).
int e3d_bounds_take_batch(long long out[4]) { return e3d::bounds_take(out); }
