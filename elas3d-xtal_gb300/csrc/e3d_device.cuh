// Device-side building blocks of the sm_103a voxel-FE solver.
//
// Element arithmetic.  The reference integrates the 24x24 element matrix
// dk = sum_q w_q B_q^T C B_q over 3x3x3 Simpson points
// (src/elas3dxtal_pcg.f90:713-805) and applies it node by node with 576
// multiply-adds (:1176-1321).  The integrand is at most quadratic in each
// coordinate, so that rule is exact, and so is the 2x2x2 Gauss rule.  Under the
// Gauss rule the strain field of a trilinear element splits into 7 mutually
// orthogonal modes (constant, x, y, z, xy, xz, yz), so
//     K_e u = H^T [ sum_k W_k M_k^T C M_k ] H u,
// with H the 8-point Walsh-Hadamard transform of the nodal values, M_k a
// sparse selector and W = 1/16, 1/48, 1/144.  That is the same matrix to
// rounding (checked against the Simpson dk to 4e-16) at ~276 FP64 operations
// per element instead of 576.  GB300 runs FP64 at 1/64 of its FP32 rate, so
// the stencil is FP64-issue-bound and this count, not HBM bytes, sets its time.
//
// Corner index inside an element: a = ox + 2*oy + 4*oz.  Hadamard index
// b = bx + 2*by + 4*bz (bit set = difference along that axis).
#pragma once
#include <cstdint>

namespace e3d {

enum : int { HX_ = 1, HY_ = 2, HXY = 3, HZ_ = 4, HXZ = 5, HYZ = 6, HXYZ = 7 };

// FP64 stiffness table per phase (kCsStride doubles):
//   [0, 36)    C/16, row-major 6x6: the constant mode, which takes the nine
//              first-order Hadamard components (u, v, w at HX_, HY_, HZ_);
//   [36, 117)  M2, row-major 9x9: the nine second-order components (u, v, w at
//              HXY, HXZ, HYZ, in that order) -> the forces there, i.e. the x, y
//              and z modes (weight 1/48) summed into one matrix;
//   [117, 126) M3, row-major 3x3: the three third-order components (u, v, w at
//              HXYZ) -> the forces there, the xy, xz and yz modes (1/144) summed.
// Summing the modes of one Hadamard order into one matrix ahead of time turns
// 3 x 25 + 12 and 3 x 9 + 6 operations into 81 and 9 multiply-adds per
// element: 30 fewer FP64 instructions on the stencil's critical pipe.
constexpr int kCsStride = 126;
constexpr int kM2 = 36, kM3 = 117;

template <typename T>
__host__ __device__ __forceinline__ T fma_(T a, T b, T c) {
  return fma(a, b, c);
}

// s[r] = sum_c C[r][c] e[c] for r, c in the index set IDX (N entries).
template <typename T, int N>
__host__ __device__ __forceinline__ void matvec_sub(const T* __restrict__ Cm, const int (&idx)[N],
                                                    const T (&e)[N], T (&s)[N]) {
#pragma unroll
  for (int r = 0; r < N; ++r) {
    T acc = Cm[6 * idx[r] + idx[0]] * e[0];
#pragma unroll
    for (int c = 1; c < N; ++c) acc = fma_(Cm[6 * idx[r] + idx[c]], e[c], acc);
    s[r] = acc;
  }
}

// The second-order modes one by one (C1 = C/48): in / out are the nine
// components u, v, w at HXY, HXZ, HYZ.
__host__ __device__ inline void second_order_modes(const double* C1, const double (&in)[9], double (&out)[9]) {
  const double uxy = in[0], vxy = in[1], wxy = in[2], uxz = in[3], vxz = in[4], wxz = in[5];
  const double uyz = in[6], vyz = in[7], wyz = in[8];
  double sx[5], sy[5], sz[5];
  {  // x mode: yy, zz, xz, yz, xy
    const int idx[5] = {1, 2, 3, 4, 5};
    const double e[5] = {vxy, wxz, uxz, vxz + wxy, uxy};
    matvec_sub<double, 5>(C1, idx, e, sx);
  }
  {  // y mode: xx, zz, xz, yz, xy
    const int idx[5] = {0, 2, 3, 4, 5};
    const double e[5] = {uxy, wyz, uyz + wxy, vyz, vxy};
    matvec_sub<double, 5>(C1, idx, e, sy);
  }
  {  // z mode: xx, yy, xz, yz, xy
    const int idx[5] = {0, 1, 3, 4, 5};
    const double e[5] = {uxz, vyz, wxz, wyz, uyz + vxz};
    matvec_sub<double, 5>(C1, idx, e, sz);
  }
  out[0] = sx[4] + sy[0];  // u at HXY
  out[1] = sx[0] + sy[4];  // v at HXY
  out[2] = sx[3] + sy[2];  // w at HXY
  out[3] = sx[2] + sz[0];  // u at HXZ
  out[4] = sx[3] + sz[4];
  out[5] = sx[1] + sz[2];
  out[6] = sy[2] + sz[4];  // u at HYZ
  out[7] = sy[3] + sz[1];
  out[8] = sy[1] + sz[3];
}

// The third-order modes (C2 = C/144): u, v, w at HXYZ in and out.
__host__ __device__ inline void third_order_modes(const double* C2, const double (&in)[3], double (&out)[3]) {
  const double u = in[0], v = in[1], w = in[2];
  double sxy[3], sxz[3], syz[3];
  {  // xy mode: zz, xz, yz
    const int idx[3] = {2, 3, 4};
    const double e[3] = {w, u, v};
    matvec_sub<double, 3>(C2, idx, e, sxy);
  }
  {  // xz mode: yy, yz, xy
    const int idx[3] = {1, 4, 5};
    const double e[3] = {v, w, u};
    matvec_sub<double, 3>(C2, idx, e, sxz);
  }
  {  // yz mode: xx, xz, xy
    const int idx[3] = {0, 3, 5};
    const double e[3] = {u, w, v};
    matvec_sub<double, 3>(C2, idx, e, syz);
  }
  out[0] = sxy[1] + sxz[2] + syz[0];
  out[1] = sxy[2] + sxz[0] + syz[2];
  out[2] = sxy[0] + sxz[1] + syz[1];
}

// Builds a phase's FP64 table from its 6x6 stiffness (Voigt xx, yy, zz, xz, yz, xy).
__host__ __device__ inline void modal_table(const double (&C6)[6][6], double* tab) {
  double C1[36], C2[36];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      tab[6 * i + j] = C6[i][j] / 16.0;
      C1[6 * i + j] = C6[i][j] / 48.0;
      C2[6 * i + j] = C6[i][j] / 144.0;
    }
  for (int c = 0; c < 9; ++c) {  // column c of M2: the response to unit component c
    double in[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, out[9];
    in[c] = 1.0;
    second_order_modes(C1, in, out);
    for (int r = 0; r < 9; ++r) tab[kM2 + 9 * r + c] = out[r];
  }
  for (int c = 0; c < 3; ++c) {
    double in[3] = {0, 0, 0}, out[3];
    in[c] = 1.0;
    third_order_modes(C2, in, out);
    for (int r = 0; r < 3; ++r) tab[kM3 + 3 * r + c] = out[r];
  }
}

// Element forces in the Hadamard domain: (hu, hv, hw) -> (fu, fv, fw).
// cs points at the phase's kCsStride-entry table.
template <typename T>
__device__ __forceinline__ void element_modal(const T* __restrict__ cs, const T (&hu)[8],
                                              const T (&hv)[8], const T (&hw)[8], T (&fu)[8],
                                              T (&fv)[8], T (&fw)[8]) {
  // constant mode, all six Voigt components (xx, yy, zz, xz, yz, xy)
  {
    const int idx[6] = {0, 1, 2, 3, 4, 5};
    const T e[6] = {hu[HX_], hv[HY_], hw[HZ_], hu[HZ_] + hw[HX_], hv[HZ_] + hw[HY_], hu[HY_] + hv[HX_]};
    T s[6];
    matvec_sub<T, 6>(cs, idx, e, s);
    fu[HX_] = s[0];
    fv[HY_] = s[1];
    fw[HZ_] = s[2];
    fu[HZ_] = s[3];
    fw[HX_] = s[3];
    fv[HZ_] = s[4];
    fw[HY_] = s[4];
    fu[HY_] = s[5];
    fv[HX_] = s[5];
  }
  {  // second order: one 9x9 matrix
    const T in[9] = {hu[HXY], hv[HXY], hw[HXY], hu[HXZ], hv[HXZ], hw[HXZ], hu[HYZ], hv[HYZ], hw[HYZ]};
    T out[9];
    const T* M = cs + kM2;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      T acc = M[9 * r] * in[0];
#pragma unroll
      for (int c = 1; c < 9; ++c) acc = fma_(M[9 * r + c], in[c], acc);
      out[r] = acc;
    }
    fu[HXY] = out[0];
    fv[HXY] = out[1];
    fw[HXY] = out[2];
    fu[HXZ] = out[3];
    fv[HXZ] = out[4];
    fw[HXZ] = out[5];
    fu[HYZ] = out[6];
    fv[HYZ] = out[7];
    fw[HYZ] = out[8];
  }
  {  // third order: one 3x3 matrix
    const T* M = cs + kM3;
    const T u = hu[HXYZ], v = hv[HXYZ], w = hw[HXYZ];
    fu[HXYZ] = fma_(M[2], w, fma_(M[1], v, M[0] * u));
    fv[HXYZ] = fma_(M[5], w, fma_(M[4], v, M[3] * u));
    fw[HXYZ] = fma_(M[8], w, fma_(M[7], v, M[6] * u));
  }
  fu[0] = T(0);
  fv[0] = T(0);
  fw[0] = T(0);
}

// FP32 table: the upper triangle of C/16 (row-major, 21 entries, 3 pad), read
// with six 16-byte loads.  Every Hadamard component belongs to one mode class --
// first order (HX_, HY_, HZ_) to the constant mode (weight 1/16), second order
// (HXY, HXZ, HYZ) to the x/y/z modes (1/48 = 1/16 * 1/3), third order (HXYZ) to
// the xy/xz/yz modes (1/144 = 1/16 * 1/9) -- so scaling the 9 second-order
// inputs by 1/3 and the 3 third-order inputs by 1/9 lets all seven modes share
// C/16: 12 multiplies instead of 87 table loads per element.
constexpr int kCs32Stride = 24;

__host__ __device__ constexpr int sym6(int r, int c) {
  return r <= c ? r * 6 - r * (r - 1) / 2 + (c - r) : c * 6 - c * (c - 1) / 2 + (r - c);
}

template <int N>
__device__ __forceinline__ void matvec_sym(const float (&t)[kCs32Stride], const int (&idx)[N], const float (&e)[N],
                                           float (&s)[N]) {
#pragma unroll
  for (int r = 0; r < N; ++r) {
    float acc = t[sym6(idx[r], idx[0])] * e[0];
#pragma unroll
    for (int c = 1; c < N; ++c) acc = fmaf(t[sym6(idx[r], idx[c])], e[c], acc);
    s[r] = acc;
  }
}

// The table row comes from global memory (tstride == 0: six consecutive float4,
// read through the read-only path) or from a shared-memory slot whose six
// float4 lie tstride float4 apart (staged there ahead of use).
template <int TSTRIDE = 0>
__device__ __forceinline__ void element_modal_f32(const float* __restrict__ cs, const float (&hu)[8],
                                                  const float (&hv)[8], const float (&hw)[8], float (&fu)[8],
                                                  float (&fv)[8], float (&fw)[8]) {
  float t[kCs32Stride];
  const float4* t4 = reinterpret_cast<const float4*>(cs);
#pragma unroll
  for (int i = 0; i < kCs32Stride / 4; ++i) {
    const float4 q = TSTRIDE == 0 ? __ldg(t4 + i) : t4[i * TSTRIDE];
    t[4 * i] = q.x;
    t[4 * i + 1] = q.y;
    t[4 * i + 2] = q.z;
    t[4 * i + 3] = q.w;
  }
  const float k3 = 1.0f / 3.0f, k9 = 1.0f / 9.0f;
  const float uxy = hu[HXY] * k3, vxy = hv[HXY] * k3, wxy = hw[HXY] * k3;
  const float uxz = hu[HXZ] * k3, vxz = hv[HXZ] * k3, wxz = hw[HXZ] * k3;
  const float uyz = hu[HYZ] * k3, vyz = hv[HYZ] * k3, wyz = hw[HYZ] * k3;
  const float uxyz = hu[HXYZ] * k9, vxyz = hv[HXYZ] * k9, wxyz = hw[HXYZ] * k9;
  {
    const int idx[6] = {0, 1, 2, 3, 4, 5};
    const float e[6] = {hu[HX_], hv[HY_], hw[HZ_], hu[HZ_] + hw[HX_], hv[HZ_] + hw[HY_], hu[HY_] + hv[HX_]};
    float s[6];
    matvec_sym<6>(t, idx, e, s);
    fu[HX_] = s[0];
    fv[HY_] = s[1];
    fw[HZ_] = s[2];
    fu[HZ_] = s[3];
    fw[HX_] = s[3];
    fv[HZ_] = s[4];
    fw[HY_] = s[4];
    fu[HY_] = s[5];
    fv[HX_] = s[5];
  }
  float sx[5], sy[5], sz[5];
  {
    const int idx[5] = {1, 2, 3, 4, 5};
    const float e[5] = {vxy, wxz, uxz, vxz + wxy, uxy};
    matvec_sym<5>(t, idx, e, sx);
  }
  {
    const int idx[5] = {0, 2, 3, 4, 5};
    const float e[5] = {uxy, wyz, uyz + wxy, vyz, vxy};
    matvec_sym<5>(t, idx, e, sy);
  }
  {
    const int idx[5] = {0, 1, 3, 4, 5};
    const float e[5] = {uxz, vyz, wxz, wyz, uyz + vxz};
    matvec_sym<5>(t, idx, e, sz);
  }
  fu[HXY] = sx[4] + sy[0];
  fv[HXY] = sx[0] + sy[4];
  fw[HXY] = sx[3] + sy[2];
  fu[HXZ] = sx[2] + sz[0];
  fv[HXZ] = sx[3] + sz[4];
  fw[HXZ] = sx[1] + sz[2];
  fu[HYZ] = sy[2] + sz[4];
  fv[HYZ] = sy[3] + sz[1];
  fw[HYZ] = sy[1] + sz[3];
  float sxy[3], sxz[3], syz[3];
  {
    const int idx[3] = {2, 3, 4};
    const float e[3] = {wxyz, uxyz, vxyz};
    matvec_sym<3>(t, idx, e, sxy);
  }
  {
    const int idx[3] = {1, 4, 5};
    const float e[3] = {vxyz, wxyz, uxyz};
    matvec_sym<3>(t, idx, e, sxz);
  }
  {
    const int idx[3] = {0, 3, 5};
    const float e[3] = {uxyz, wxyz, vxyz};
    matvec_sym<3>(t, idx, e, syz);
  }
  fu[HXYZ] = sxy[1] + sxz[2] + syz[0];
  fv[HXYZ] = sxy[2] + sxz[0] + syz[2];
  fw[HXYZ] = sxy[0] + sxz[1] + syz[1];
  fu[0] = 0.f;
  fv[0] = 0.f;
  fw[0] = 0.f;
}

// Forward Hadamard of one plane of 4 corner values v[oy*2+ox] -> P[by*2+bx].
template <typename T>
__device__ __forceinline__ void had_xy(const T (&v)[4], T (&P)[4]) {
  const T s0 = v[1] + v[0], d0 = v[1] - v[0];
  const T s1 = v[3] + v[2], d1 = v[3] - v[2];
  P[0] = s1 + s0;
  P[2] = s1 - s0;
  P[1] = d1 + d0;
  P[3] = d1 - d0;
}

// Adjoint of had_xy: T[by*2+bx] -> corner forces r[oy*2+ox].
template <typename T>
__device__ __forceinline__ void had_xy_adj(const T (&Tm)[4], T (&r)[4]) {
  const T e0 = Tm[0] - Tm[2], e1 = Tm[0] + Tm[2];
  const T g0 = Tm[1] - Tm[3], g1 = Tm[1] + Tm[3];
  r[0] = e0 - g0;
  r[1] = e0 + g0;
  r[2] = e1 - g1;
  r[3] = e1 + g1;
}

// Full element: 8 corner values per component (a = ox + 2oy + 4oz) -> forces.
// Used by the one-off kernels (dk build, boundary terms, tests of the tile path).
template <typename T>
__device__ __forceinline__ void element_apply(const T* __restrict__ cs, const T (&u)[3][8],
                                              T (&r)[3][8]) {
  T h[3][8];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const T lo[4] = {u[c][0], u[c][1], u[c][2], u[c][3]};
    const T hi[4] = {u[c][4], u[c][5], u[c][6], u[c][7]};
    T Plo[4], Phi[4];
    had_xy(lo, Plo);
    had_xy(hi, Phi);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      h[c][b] = Phi[b] + Plo[b];
      h[c][b + 4] = Phi[b] - Plo[b];
    }
  }
  T f[3][8];
  element_modal<T>(cs, h[0], h[1], h[2], f[0], f[1], f[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    T tlo[4], thi[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      tlo[b] = f[c][b] - f[c][b + 4];
      thi[b] = f[c][b] + f[c][b + 4];
    }
    T rlo[4], rhi[4];
    had_xy_adj(tlo, rlo);
    had_xy_adj(thi, rhi);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      r[c][a] = rlo[a];
      r[c][a + 4] = rhi[a];
    }
  }
}

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Block-wide sum of one value per thread (fixed shuffle + shared-memory tree,
// so the result does not depend on scheduling).  Result valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) s += scratch[i];
  }
  return s;
}

}  // namespace e3d
