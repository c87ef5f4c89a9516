// Internal interface of the synthetic-microstructure generator, shared by the
// host implementation (microgen.cpp) and its GPU back end (microgen_gpu.cu).
//
// Grains: the host draws seeds, orientations and power weights, bins the seeds
// into cells and, for every voxel block, lists the seeds that can be nearest to
// one of its voxels (ascending grain id, each at its periodic image nearest the
// block centre).  The per-voxel search over those candidates -- the O(voxels x
// candidates) part -- then runs on either side with the same arithmetic, so
// both give the same phase ids.
//
// Pores: PoreStream replays the random draws of the pore loops in order; the
// painter (host loop or GPU block) applies them one at a time until the target
// fraction is reached.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace e3d_micro {

struct Rng {  // xoshiro256** seeded through splitmix64
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) {
      x += 0x9e3779b97f4a7c15ULL;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      s[i] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double normal() {  // Box-Muller (libm; used only for pore sizes and Laguerre weights)
    double u1 = uniform();
    while (u1 <= 0.0) u1 = uniform();
    const double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  // Uniform unit quaternion: rejection from the unit 4-ball, then normalise.
  // Same distribution on S^3 as a normalised 4-Gaussian, using only sqrt.
  void quaternion(double q[4]) {
    for (;;) {
      double v[4], n2 = 0.0;
      for (int i = 0; i < 4; ++i) {
        v[i] = 2.0 * uniform() - 1.0;
        n2 += v[i] * v[i];
      }
      if (n2 > 1.0 || n2 < 1e-6) continue;
      const double inv = 1.0 / std::sqrt(n2);
      for (int i = 0; i < 4; ++i) q[i] = v[i] * inv;
      if (q[0] < 0.0)
        for (int i = 0; i < 4; ++i) q[i] = -q[i];
      if (q[0] < 1e-9) continue;  // Rodrigues vector would be unbounded
      return;
    }
  }
};

struct GrainPlan {
  int nx = 0, ny = 0, nz = 0, ngrains = 0;
  double L[3] = {0, 0, 0};
  int B = 0;                           // voxel block edge
  int nb[3] = {0, 0, 0};               // voxel blocks per direction
  std::vector<double> sx, sy, sz, w;   // seeds and power weights (0 for Voronoi)
  std::vector<int64_t> off;            // per block: candidates [off[b], off[b+1])
  std::vector<uint8_t> brute;          // per block: 1 = search every seed (tiny boxes)
  std::vector<int32_t> cg;             // candidate grain ids, ascending within a block
  std::vector<double> cx, cy, cz;      // candidate seed image nearest the block centre
};

// Seeds, orientations (rod: 3*ngrains Rodrigues vectors) and candidate lists.
int32_t grain_plan(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains, double laguerre_sigma, uint64_t seed,
                   double* rod, GrainPlan& P);

// One pore: voxel centres x with |A (x - c)|^2 <= 1 (periodic), searched over
// the integer box [i0, i1] x [j0, j1] x [k0, k1] (unwrapped indices).
struct PoreShape {
  double c[3];
  double A[3][3];
  int i0, i1, j0, j1, k0, k1;
};

class PoreStream {
 public:
  // kind 0: spheres, radius ~ lognormal(log_mu, log_sigma) voxels;
  // kind 1: ellipsoids with semi-axes (aspect a, a, a), random orientation.
  PoreStream(int kind, int nx, int ny, int nz, double aspect, double log_mu, double log_sigma, uint64_t seed);
  void next(PoreShape& p);

 private:
  int kind_, nx_, ny_, nz_;
  double aspect_, log_mu_, log_sigma_, maxr_;
  Rng rng_;
};

}  // namespace e3d_micro
