// Seeded synthetic microstructures (host code).  Writes the reference's input
// arrays: pix (int32, 1-based phase per voxel) and one Rodrigues vector per
// grain (src/microstructure_gen.m:774-800, 866-892).  Deterministic for a
// given seed; the grain/orientation stream uses only IEEE +,-,*,/ and sqrt and
// the file is compiled without floating-point contraction, so it is
// bit-identical on x86-64 and AArch64 and to the GPU back end
// (microgen_gpu.cu), which shares the plan built here.
#include "e3d_micro.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "microgen_plan.h"

namespace e3d_micro {

inline double wrap_delta(double d, double L) {
  if (d > 0.5 * L) d -= L;
  if (d < -0.5 * L) d += L;
  return d;
}

int32_t grain_plan(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains, double laguerre_sigma, uint64_t seed,
                   double* rod, GrainPlan& P) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || ngrains <= 0 || !rod) return -1;
  Rng rng(seed);
  P.nx = nx;
  P.ny = ny;
  P.nz = nz;
  P.ngrains = ngrains;
  P.L[0] = nx;
  P.L[1] = ny;
  P.L[2] = nz;
  const double* L = P.L;
  P.sx.assign(ngrains, 0.0);
  P.sy.assign(ngrains, 0.0);
  P.sz.assign(ngrains, 0.0);
  P.w.assign(ngrains, 0.0);
  for (int g = 0; g < ngrains; ++g) {
    P.sx[g] = rng.uniform() * L[0];
    P.sy[g] = rng.uniform() * L[1];
    P.sz[g] = rng.uniform() * L[2];
  }
  for (int g = 0; g < ngrains; ++g) {
    double q[4];
    rng.quaternion(q);
    rod[3 * g + 0] = q[1] / q[0];
    rod[3 * g + 1] = q[2] / q[0];
    rod[3 * g + 2] = q[3] / q[0];
  }
  const double vol = L[0] * L[1] * L[2];
  const double spacing = std::cbrt(vol / ngrains);
  double wmax = 0.0;
  if (laguerre_sigma > 0.0) {
    // Power-diagram weights w = r^2 with r ~ V^(1/3), V ~ lognormal(0, sigma),
    // scaled so the mean radius is a third of the seed spacing.
    std::vector<double> r(ngrains);
    double mean = 0.0;
    for (int g = 0; g < ngrains; ++g) {
      r[g] = std::cbrt(std::exp(laguerre_sigma * rng.normal()));
      mean += r[g];
    }
    mean /= ngrains;
    for (int g = 0; g < ngrains; ++g) {
      const double rr = r[g] / mean * spacing / 3.0;
      P.w[g] = rr * rr;
      wmax = std::max(wmax, P.w[g]);
    }
  }
  const double* sx = P.sx.data();
  const double* sy = P.sy.data();
  const double* sz = P.sz.data();
  const double* w = P.w.data();
  // Seed cell grid for the candidate search.
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = std::max(1, (int)std::floor(L[d] / spacing));
  const double cs[3] = {L[0] / nc[0], L[1] / nc[1], L[2] / nc[2]};
  std::vector<std::vector<int>> cell((size_t)nc[0] * nc[1] * nc[2]);
  for (int g = 0; g < ngrains; ++g) {
    int ci = std::min(nc[0] - 1, (int)(sx[g] / cs[0]));
    int cj = std::min(nc[1] - 1, (int)(sy[g] / cs[1]));
    int ck = std::min(nc[2] - 1, (int)(sz[g] / cs[2]));
    cell[(size_t)ci + (size_t)nc[0] * ((size_t)cj + (size_t)nc[1] * ck)].push_back(g);
  }
  const int B = std::max(2, (int)(spacing / 2.0));  // voxel block edge
  P.B = B;
  P.nb[0] = (nx + B - 1) / B;
  P.nb[1] = (ny + B - 1) / B;
  P.nb[2] = (nz + B - 1) / B;
  const int* nb = P.nb;
  const long nblocks = (long)nb[0] * nb[1] * nb[2];
  std::vector<std::vector<int32_t>> bg_ids(nblocks);
  std::vector<std::vector<double>> bx(nblocks), by(nblocks), bz(nblocks);
  P.brute.assign(nblocks, 0);
#pragma omp parallel for schedule(dynamic, 16)
  for (long blk = 0; blk < nblocks; ++blk) {
    const int bi = (int)(blk % nb[0]), bj = (int)((blk / nb[0]) % nb[1]), bk = (int)(blk / ((long)nb[0] * nb[1]));
    const int i0 = bi * B, j0 = bj * B, k0 = bk * B;
    const int i1 = std::min(nx, i0 + B), j1 = std::min(ny, j0 + B), k1 = std::min(nz, k0 + B);
    const double c[3] = {0.5 * (i0 + i1), 0.5 * (j0 + j1), 0.5 * (k0 + k1)};
    const double rb = 0.5 * std::sqrt((double)(i1 - i0) * (i1 - i0) + (double)(j1 - j0) * (j1 - j0) +
                                      (double)(k1 - k0) * (k1 - k0));
    // Upper bound on the best power distance from any voxel of the block:
    // take the best seed for the centre over an expanding shell of cells.
    double best_c = 1e300;
    bool brute = false;
    for (int ring = 1;; ++ring) {
      if (2 * ring + 1 > nc[0] || 2 * ring + 1 > nc[1] || 2 * ring + 1 > nc[2]) {
        brute = true;
        break;
      }
      const int ci = (int)(c[0] / cs[0]), cj = (int)(c[1] / cs[1]), ck = (int)(c[2] / cs[2]);
      for (int dk = -ring; dk <= ring; ++dk)
        for (int dj = -ring; dj <= ring; ++dj)
          for (int di = -ring; di <= ring; ++di) {
            const int a = ((ci + di) % nc[0] + nc[0]) % nc[0];
            const int bb = ((cj + dj) % nc[1] + nc[1]) % nc[1];
            const int cc = ((ck + dk) % nc[2] + nc[2]) % nc[2];
            for (int g : cell[(size_t)a + (size_t)nc[0] * ((size_t)bb + (size_t)nc[1] * cc)]) {
              const double dx = wrap_delta(sx[g] - c[0], L[0]);
              const double dy = wrap_delta(sy[g] - c[1], L[1]);
              const double dz = wrap_delta(sz[g] - c[2], L[2]);
              const double dd = std::sqrt(dx * dx + dy * dy + dz * dz);
              best_c = std::min(best_c, (dd + rb) * (dd + rb) - w[g]);
            }
          }
      // Every seed outside this shell is at least ring*min(cs) - cs away.
      const double reach = (ring - 1) * std::min(cs[0], std::min(cs[1], cs[2]));
      if (best_c < 1e299) {
        const double need = rb + std::sqrt(std::max(0.0, best_c + wmax));
        if (reach >= need) break;
      }
    }
    const double R = brute ? 1e300 : rb + std::sqrt(std::max(0.0, best_c + wmax));
    if (!brute && (R + rb >= 0.5 * L[0] || R + rb >= 0.5 * L[1] || R + rb >= 0.5 * L[2])) brute = true;
    if (brute) {
      P.brute[blk] = 1;
      continue;
    }
    // Candidate list: seeds that can be the (power-)nearest of some voxel here,
    // at their periodic image nearest the block centre.
    std::vector<int> cgv;
    std::vector<double> cxv, cyv, czv;
    const int ci0 = (int)std::floor((c[0] - R) / cs[0]), ci1 = (int)std::floor((c[0] + R) / cs[0]);
    const int cj0 = (int)std::floor((c[1] - R) / cs[1]), cj1 = (int)std::floor((c[1] + R) / cs[1]);
    const int ck0 = (int)std::floor((c[2] - R) / cs[2]), ck1 = (int)std::floor((c[2] + R) / cs[2]);
    for (int dk = ck0; dk <= ck1; ++dk)
      for (int dj = cj0; dj <= cj1; ++dj)
        for (int di = ci0; di <= ci1; ++di) {
          const int a = (di % nc[0] + nc[0]) % nc[0];
          const int bb = (dj % nc[1] + nc[1]) % nc[1];
          const int cc = (dk % nc[2] + nc[2]) % nc[2];
          for (int g : cell[(size_t)a + (size_t)nc[0] * ((size_t)bb + (size_t)nc[1] * cc)]) {
            const double dx = wrap_delta(sx[g] - c[0], L[0]);
            const double dy = wrap_delta(sy[g] - c[1], L[1]);
            const double dz = wrap_delta(sz[g] - c[2], L[2]);
            if (std::sqrt(dx * dx + dy * dy + dz * dz) <= R + 1e-9 &&
                std::find(cgv.begin(), cgv.end(), g) == cgv.end()) {
              cgv.push_back(g);
              cxv.push_back(c[0] + dx);
              cyv.push_back(c[1] + dy);
              czv.push_back(c[2] + dz);
            }
          }
        }
    // ascending grain id, so that ties resolve to the lower id
    std::vector<int> order(cgv.size());
    for (size_t t = 0; t < order.size(); ++t) order[t] = (int)t;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return cgv[x] < cgv[y]; });
    for (int t : order) {
      bg_ids[blk].push_back(cgv[t]);
      bx[blk].push_back(cxv[t]);
      by[blk].push_back(cyv[t]);
      bz[blk].push_back(czv[t]);
    }
  }
  P.off.assign(nblocks + 1, 0);
  for (long b = 0; b < nblocks; ++b) P.off[b + 1] = P.off[b] + (int64_t)bg_ids[b].size();
  const size_t nc_tot = (size_t)P.off[nblocks];
  P.cg.resize(nc_tot);
  P.cx.resize(nc_tot);
  P.cy.resize(nc_tot);
  P.cz.resize(nc_tot);
  for (long b = 0; b < nblocks; ++b) {
    const size_t o = (size_t)P.off[b];
    std::copy(bg_ids[b].begin(), bg_ids[b].end(), P.cg.begin() + o);
    std::copy(bx[b].begin(), bx[b].end(), P.cx.begin() + o);
    std::copy(by[b].begin(), by[b].end(), P.cy.begin() + o);
    std::copy(bz[b].begin(), bz[b].end(), P.cz.begin() + o);
  }
  return 0;
}

PoreStream::PoreStream(int kind, int nx, int ny, int nz, double aspect, double log_mu, double log_sigma,
                       uint64_t seed)
    : kind_(kind),
      nx_(nx),
      ny_(ny),
      nz_(nz),
      aspect_(aspect),
      log_mu_(log_mu),
      log_sigma_(log_sigma),
      maxr_(0.25 * std::min(nx, std::min(ny, nz))),
      rng_(seed ^ (kind == 0 ? 0x51ed27a1b3c4d5e6ULL : 0x2b7e151628aed2a6ULL)) {}

void PoreStream::next(PoreShape& p) {
  p.c[0] = rng_.uniform() * nx_;
  p.c[1] = rng_.uniform() * ny_;
  p.c[2] = rng_.uniform() * nz_;
  double rmax;
  if (kind_ == 0) {
    double r = std::exp(log_mu_ + log_sigma_ * rng_.normal());
    r = std::min(std::max(r, 0.5), maxr_);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) p.A[i][j] = i == j ? 1.0 / r : 0.0;
    rmax = r;
  } else {
    double a = std::exp(log_mu_ + log_sigma_ * rng_.normal());
    a = std::max(a, 0.5);
    if (aspect_ * a > maxr_) a = maxr_ / aspect_;
    double q[4];
    rng_.quaternion(q);
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                            {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                            {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    const double semi[3] = {aspect_ * a, a, a};
    // A = diag(1/semi) R^T maps lab offsets into the unit sphere.
    for (int r = 0; r < 3; ++r)
      for (int s = 0; s < 3; ++s) p.A[r][s] = R[s][r] / semi[r];
    rmax = aspect_ * a;
  }
  p.i0 = (int)std::floor(p.c[0] - rmax - 1);
  p.i1 = (int)std::ceil(p.c[0] + rmax + 1);
  p.j0 = (int)std::floor(p.c[1] - rmax - 1);
  p.j1 = (int)std::ceil(p.c[1] + rmax + 1);
  p.k0 = (int)std::floor(p.c[2] - rmax - 1);
  p.k1 = (int)std::ceil(p.c[2] + rmax + 1);
}

}  // namespace e3d_micro

using namespace e3d_micro;

namespace {

inline size_t lin(int i, int j, int k, int nx, int ny) {
  return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k);
}

// Marks every voxel whose centre lies inside the (periodic) pore; returns the
// number of voxels newly set to pore_phase.
long paint_pore(int nx, int ny, int nz, const PoreShape& p, int32_t pore_phase, int32_t* pix) {
  long added = 0;
  for (int k = p.k0; k <= p.k1; ++k)
    for (int j = p.j0; j <= p.j1; ++j)
      for (int i = p.i0; i <= p.i1; ++i) {
        const double d[3] = {i + 0.5 - p.c[0], j + 0.5 - p.c[1], k + 0.5 - p.c[2]};
        double q = 0.0;
        for (int r = 0; r < 3; ++r) {
          const double t = p.A[r][0] * d[0] + p.A[r][1] * d[1] + p.A[r][2] * d[2];
          q += t * t;
        }
        if (q > 1.0) continue;
        const int ii = ((i % nx) + nx) % nx, jj = ((j % ny) + ny) % ny, kk = ((k % nz) + nz) % nz;
        int32_t& v = pix[lin(ii, jj, kk, nx, ny)];
        if (v != pore_phase) {
          v = pore_phase;
          ++added;
        }
      }
  return added;
}

int32_t add_pores(int kind, int32_t nx, int32_t ny, int32_t nz, double target_frac, double aspect, double log_mu,
                  double log_sigma, int32_t pore_phase, uint64_t seed, int32_t* pix) {
  const long ns = (long)nx * ny * nz;
  long count = 0;
  for (long m = 0; m < ns; ++m) count += (pix[m] == pore_phase);
  PoreStream S(kind, nx, ny, nz, aspect, log_mu, log_sigma, seed);
  int32_t placed = 0;
  while ((double)count < target_frac * (double)ns) {
    PoreShape p;
    S.next(p);
    count += paint_pore(nx, ny, nz, p, pore_phase, pix);
    ++placed;
    if (placed > 100000000) return -2;
  }
  return placed;
}

}  // namespace

extern "C" int32_t e3d_micro_grains(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                    double laguerre_sigma, uint64_t seed, int32_t* pix,
                                    double* rod) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || ngrains <= 0 || !pix || !rod) return -1;
  GrainPlan P;
  int32_t status = grain_plan(nx, ny, nz, ngrains, laguerre_sigma, seed, rod, P);
  if (status) return status;
  const int B = P.B;
  const long nblocks = (long)P.nb[0] * P.nb[1] * P.nb[2];
#pragma omp parallel for schedule(dynamic, 4)
  for (long blk = 0; blk < nblocks; ++blk) {
    const int bi = (int)(blk % P.nb[0]), bj = (int)((blk / P.nb[0]) % P.nb[1]);
    const int bk = (int)(blk / ((long)P.nb[0] * P.nb[1]));
    const int i0 = bi * B, j0 = bj * B, k0 = bk * B;
    const int i1 = std::min(nx, i0 + B), j1 = std::min(ny, j0 + B), k1 = std::min(nz, k0 + B);
    const size_t c0 = (size_t)P.off[blk], c1 = (size_t)P.off[blk + 1];
    for (int k = k0; k < k1; ++k)
      for (int j = j0; j < j1; ++j)
        for (int i = i0; i < i1; ++i) {
          const double px = i + 0.5, py = j + 0.5, pz = k + 0.5;
          double best = 1e300;
          int bg;
          if (P.brute[blk]) {
            bg = 0;
            for (int g = 0; g < ngrains; ++g) {
              const double dx = wrap_delta(P.sx[g] - px, P.L[0]);
              const double dy = wrap_delta(P.sy[g] - py, P.L[1]);
              const double dz = wrap_delta(P.sz[g] - pz, P.L[2]);
              const double d = dx * dx + dy * dy + dz * dz - P.w[g];
              if (d < best) {
                best = d;
                bg = g;
              }
            }
          } else {
            bg = -1;
            for (size_t t = c0; t < c1; ++t) {
              const double dx = P.cx[t] - px, dy = P.cy[t] - py, dz = P.cz[t] - pz;
              const double d = dx * dx + dy * dy + dz * dz - P.w[P.cg[t]];
              if (d < best) {
                best = d;
                bg = P.cg[t];
              }
            }
            if (bg < 0) {
#pragma omp atomic write
              status = -2;
            }
          }
          pix[lin(i, j, k, nx, ny)] = bg + 1;
        }
  }
  return status;
}

extern "C" int32_t e3d_micro_spherical_pores(int32_t nx, int32_t ny, int32_t nz,
                                             double target_frac, double log_mu,
                                             double log_sigma, int32_t pore_phase,
                                             uint64_t seed, int32_t* pix) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !pix || target_frac < 0.0 || target_frac >= 1.0) return -1;
  return add_pores(0, nx, ny, nz, target_frac, 1.0, log_mu, log_sigma, pore_phase, seed, pix);
}

extern "C" int32_t e3d_micro_ellipsoidal_pores(int32_t nx, int32_t ny, int32_t nz,
                                               double target_frac, double aspect,
                                               double log_mu, double log_sigma,
                                               int32_t pore_phase, uint64_t seed,
                                               int32_t* pix) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !pix || target_frac < 0.0 || target_frac >= 1.0 || aspect <= 0.0)
    return -1;
  return add_pores(1, nx, ny, nz, target_frac, aspect, log_mu, log_sigma, pore_phase, seed, pix);
}

extern "C" void e3d_euler_to_rodrigues(int32_t n, const double* euler, double* rod) {
  for (int i = 0; i < n; ++i) {
    const double p1 = euler[3 * i], P = euler[3 * i + 1], p2 = euler[3 * i + 2];
    // Bunge ZXZ: quaternion of R = Rz(phi1) Rx(Phi) Rz(phi2)
    const double cP = std::cos(0.5 * P), sP = std::sin(0.5 * P);
    double q0 = cP * std::cos(0.5 * (p1 + p2));
    double q1 = sP * std::cos(0.5 * (p1 - p2));
    double q2 = sP * std::sin(0.5 * (p1 - p2));
    double q3 = cP * std::sin(0.5 * (p1 + p2));
    if (q0 < 0) {
      q0 = -q0, q1 = -q1, q2 = -q2, q3 = -q3;
    }
    const double d = q0 > 1e-9 ? q0 : 1e-9;
    rod[3 * i + 0] = q1 / d;
    rod[3 * i + 1] = q2 / d;
    rod[3 * i + 2] = q3 / d;
  }
}

// ---------------------------------------------------------------------------
// .e3d container (see include/e3d_micro.h).
namespace {
struct MicroHeader {
  char magic[8];
  int32_t version, nx, ny, nz, ngrains, reserved;
};
}  // namespace

extern "C" int32_t e3d_micro_write(const char* path, int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                   const int32_t* pix, const double* rod) {
  if (!path || !pix || !rod || nx < 1 || ny < 1 || nz < 1 || ngrains < 1) return -2;
  FILE* f = std::fopen(path, "wb");
  if (!f) return -1;
  MicroHeader H{};
  std::memcpy(H.magic, "E3DMICRO", 8);
  H.version = 1;
  H.nx = nx;
  H.ny = ny;
  H.nz = nz;
  H.ngrains = ngrains;
  const size_t ns = (size_t)nx * ny * nz;
  bool ok = std::fwrite(&H, sizeof H, 1, f) == 1 && std::fwrite(pix, sizeof(int32_t), ns, f) == ns &&
            std::fwrite(rod, sizeof(double), 3 * (size_t)ngrains, f) == 3 * (size_t)ngrains;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : -1;
}

extern "C" int32_t e3d_micro_read_header(const char* path, int32_t* nx, int32_t* ny, int32_t* nz,
                                         int32_t* ngrains) {
  if (!path) return -2;
  FILE* f = std::fopen(path, "rb");
  if (!f) return -1;
  MicroHeader H{};
  const bool ok = std::fread(&H, sizeof H, 1, f) == 1;
  std::fclose(f);
  if (!ok || std::memcmp(H.magic, "E3DMICRO", 8) != 0 || H.version != 1 || H.nx < 1 || H.ny < 1 || H.nz < 1 ||
      H.ngrains < 1)
    return -2;
  if (nx) *nx = H.nx;
  if (ny) *ny = H.ny;
  if (nz) *nz = H.nz;
  if (ngrains) *ngrains = H.ngrains;
  return 0;
}

extern "C" int32_t e3d_micro_read(const char* path, int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                  int32_t* pix, double* rod) {
  int32_t hx, hy, hz, hg;
  int32_t rc = e3d_micro_read_header(path, &hx, &hy, &hz, &hg);
  if (rc) return rc;
  // size checks as ppixel_hdf5 (src/elas3dxtal_pcg.f90:2939-2942, 2966-2969)
  if (hx != nx || hy != ny || hz != nz || hg != ngrains || !pix || !rod) return -2;
  FILE* f = std::fopen(path, "rb");
  if (!f) return -1;
  std::fseek(f, (long)sizeof(MicroHeader), SEEK_SET);
  const size_t ns = (size_t)nx * ny * nz;
  const bool ok = std::fread(pix, sizeof(int32_t), ns, f) == ns &&
                  std::fread(rod, sizeof(double), 3 * (size_t)ngrains, f) == 3 * (size_t)ngrains;
  std::fclose(f);
  if (!ok) return -2;
  // phase range (src/elas3dxtal_pcg.f90:2986-2989)
  for (size_t m = 0; m < ns; ++m)
    if (pix[m] < 1 || pix[m] > ngrains + 1) return -2;
  return 0;
}
