/*
 * e3d_oracle.c -- CPU oracle (plain C + OpenMP) restating the ELAS3D-Xtal
 * voxel-FE PCG solve of src/elas3dxtal_pcg.f90.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, by the smoke check and by the CPU
 * baseline leg of bench.py.  The product library never links or calls it.
 *
 * Parity status: UNPINNED by reference outputs (the reference ships no tests
 * or golden vectors and cannot be compiled here: Fortran + HDF5).  Pinned by
 * analytical known-answer tests and an independent scipy restatement instead.
 *
 * The loop structure is kept "faithful" to the reference so that the CPU
 * timing is representative: the ib(ns,27) neighbour table, the pix
 * indirection into dk(nphase,8,3,8,3), guided OpenMP scheduling and the
 * 8192-node apply chunks.  Reductions are deterministic (fixed chunk partials
 * summed in order) so results do not depend on the thread count.
 */
#include "e3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Deterministic reductions: fixed-size chunk partials summed in order.  The
 * chunk length only changes the rounding of the sums; tests set another one
 * to see how far two equally valid FP64 summation orders drift apart along a
 * solve. */
static size_t RCHUNK = 4096;
void orc_set_reduction_chunk(int64_t n) { RCHUNK = n > 0 ? (size_t)n : 4096; }

static double wtime(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

int32_t orc_num_threads(void) {
#ifdef _OPENMP
  return (int32_t)omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Neighbour numbering (src/elas3dxtal_pcg.f90:326-341).  Column n (0-based)
 * of ib holds the node at offset (IM[n], JM[n], KM[n]).
 * ------------------------------------------------------------------------- */
static const int IM[27] = {0, 1, 1, 1, 0, -1, -1, -1, 0, 1, 1, 1, 0, -1, -1, -1,
                           0, 1, 1, 1, 0, -1, -1, -1, 0, 0, 0};
static const int JM[27] = {1, 1, 0, -1, -1, -1, 0, 1, 1, 1, 0, -1, -1, -1, 0, 1,
                           1, 1, 0, -1, -1, -1, 0, 1, 0, 0, 0};
static const int KM[27] = {0, 0, 0, 0, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1,
                           1, 1, 1, 1, 1, 1, 1, 1, -1, 1, 0};

/* Local hexahedron node offsets, reference numbering 1..8
 * (is = 27,3,2,1,26,19,18,17 at src/elas3dxtal_pcg.f90:639). */
static const int LOX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int LOY[8] = {0, 0, 1, 1, 0, 0, 1, 1};
static const int LOZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};

/* The 8 elements that contain node m: lower corners at neighbours
 * 27,7,6,5,25,15,14,13 where m is local node 1..8 (src/elas3dxtal_pcg.f90:1508-1511). */
static const int ELEM_NBR[8] = {26, 6, 5, 4, 24, 14, 13, 12};

static int offset_to_nbr(int di, int dj, int dk) {
  for (int n = 0; n < 27; ++n)
    if (IM[n] == di && JM[n] == dj && KM[n] == dk) return n;
  return -1;
}

/* For each neighbour q, the (element e, local node b) pairs whose node sits at
 * q, in element order.  Mirrors the grouping of the unrolled stencil
 * (src/elas3dxtal_pcg.f90:1194-1226). */
typedef struct {
  int count;
  int e[8];
  int b[8];
} nbr_terms;

static void build_terms(nbr_terms* t) {
  for (int q = 0; q < 27; ++q) t[q].count = 0;
  for (int e = 0; e < 8; ++e) {
    const int ln = ELEM_NBR[e];
    for (int b = 0; b < 8; ++b) {
      const int q = offset_to_nbr(IM[ln] + LOX[b], JM[ln] + LOY[b], KM[ln] + LOZ[b]);
      nbr_terms* tt = &t[q];
      tt->e[tt->count] = e;
      tt->b[tt->count] = b;
      tt->count++;
    }
  }
}

static inline size_t DK(int np, int p, int a, int i, int b, int j) {
  return (size_t)p + (size_t)np * (size_t)(a + 8 * (i + 3 * (b + 8 * j)));
}

/* ---------------------------------------------------------------------------
 * rotatestiffnessby (src/elas3dxtal_pcg.f90:2470-2637).  Rodrigues vector ->
 * Q, Bond matrix newr, rotated = newr^T C newr, row-major storage.
 * ------------------------------------------------------------------------- */
void orc_rotate_stiffness(int32_t ngrains, const double* rod, double c11,
                          double c12, double c44, double* rotated) {
  double Cc[6][6];
  memset(Cc, 0, sizeof Cc);
  Cc[0][0] = Cc[1][1] = Cc[2][2] = c11;
  Cc[0][1] = Cc[0][2] = Cc[1][2] = Cc[1][0] = Cc[2][0] = Cc[2][1] = c12;
  Cc[3][3] = Cc[4][4] = Cc[5][5] = c44;

  for (int g = 0; g < ngrains; ++g) {
    const double r[3] = {rod[3 * g + 0], rod[3 * g + 1], rod[3 * g + 2]};
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
    /* Bond matrix, rows as at src/elas3dxtal_pcg.f90:2578-2621 (0-based here). */
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
    /* rotated = matmul(matmul(transpose(newr), Cc), newr) (:2627) */
    double T[6][6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double s = 0.0;
        for (int k = 0; k < 6; ++k) s += N[k][i] * Cc[k][j];
        T[i][j] = s;
      }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double s = 0.0;
        for (int k = 0; k < 6; ++k) s += T[i][k] * N[k][j];
        rotated[36 * (size_t)g + 6 * i + j] = s;
      }
  }
}

/* Isotropic projection ck, cmu (src/elas3dxtal_pcg.f90:655-664). */
static void iso_proj(double ck[6][6], double cmu[6][6]) {
  memset(ck, 0, sizeof(double) * 36);
  memset(cmu, 0, sizeof(double) * 36);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      ck[i][j] = 1.0;
      cmu[i][j] = (i == j) ? 4.0 / 3.0 : -2.0 / 3.0;
    }
  cmu[3][3] = cmu[4][4] = cmu[5][5] = 1.0;
}

/* E, nu -> K, G as done in the driver (src/elas3dxtal_pcg.f90:305-317). */
static void e_nu_to_kg(double E, double nu, double* K, double* G) {
  const double youngs = E;
  *K = E / 3.0 / (1.0 - 2.0 * nu);
  *G = youngs / 2.0 / (1.0 + nu);
}

void orc_cmod(const orc_problem* p, const double* rod, double* cmod) {
  const int np = p->nphase;
  double ck[6][6], cmu[6][6];
  iso_proj(ck, cmu);
  memset(cmod, 0, sizeof(double) * 36 * (size_t)np);
  double K1, G1;
  e_nu_to_kg(p->e1, p->nu1, &K1, &G1);
  if (p->flag_m == 0) {
    /* Voigt-Reuss-Hill style isotropic matrix (src/elas3dxtal_pcg.f90:108-111, 295-312)
     * for phases 1..nphase-1; the inclusion phase nphase takes (E1, nu1) as in
     * applications/sec3_1/pcg/n_100x100x100/elas3dxtal_pcg.f90:191-206. */
    const double K0 = (p->c11 + 2.0 * p->c12) / 3.0;
    const double G0 = (p->c11 - p->c12 + 3.0 * p->c44) / 5.0;
    const double E0 = 9.0 * K0 * G0 / (3.0 * K0 + G0);
    const double nu0 = (3.0 * K0 - 2.0 * G0) / (2.0 * (3.0 * K0 + G0));
    double Km, Gm;
    e_nu_to_kg(E0, nu0, &Km, &Gm);
    for (int k = 0; k < np - 1; ++k)
      for (int j = 0; j < 6; ++j)
        for (int i = 0; i < 6; ++i) cmod[k + np * (i + 6 * j)] = Km * ck[i][j] + Gm * cmu[i][j];
  } else {
    double* rot = (double*)malloc(sizeof(double) * 36 * (size_t)(np - 1 > 0 ? np - 1 : 1));
    orc_rotate_stiffness(np - 1, rod, p->c11, p->c12, p->c44, rot);
    for (int k = 0; k < np - 1; ++k)
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) cmod[k + np * (i + 6 * j)] = rot[36 * (size_t)k + 6 * i + j];
    free(rot);
  }
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i)
      cmod[(np - 1) + np * (i + 6 * j)] = K1 * ck[i][j] + G1 * cmu[i][j];
}

/* Element stiffness by 3x3x3 Simpson integration (src/elas3dxtal_pcg.f90:713-805). */
void orc_dk(const orc_problem* p, const double* cmod, double* dk) {
  const int np = p->nphase;
  memset(dk, 0, sizeof(double) * 576 * (size_t)np);
  double g[3][3][3];
  for (int k3 = 0; k3 < 3; ++k3)
    for (int j3 = 0; j3 < 3; ++j3)
      for (int i3 = 0; i3 < 3; ++i3) {
        int n = (i3 == 1) + (j3 == 1) + (k3 == 1);
        g[i3][j3][k3] = pow(4.0, n);
      }
#pragma omp parallel for schedule(guided)
  for (int ph = 0; ph < np; ++ph) {
    double C6[6][6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) C6[i][j] = cmod[ph + np * (i + 6 * j)];
    for (int k3 = 0; k3 < 3; ++k3)
      for (int j3 = 0; j3 < 3; ++j3)
        for (int i3 = 0; i3 < 3; ++i3) {
          const double x = i3 / 2.0, y = j3 / 2.0, z = k3 / 2.0;
          double dndx[8], dndy[8], dndz[8];
          dndx[0] = -(1.0 - y) * (1.0 - z);
          dndx[1] = (1.0 - y) * (1.0 - z);
          dndx[2] = y * (1.0 - z);
          dndx[3] = -y * (1.0 - z);
          dndx[4] = -(1.0 - y) * z;
          dndx[5] = (1.0 - y) * z;
          dndx[6] = y * z;
          dndx[7] = -y * z;
          dndy[0] = -(1.0 - x) * (1.0 - z);
          dndy[1] = -x * (1.0 - z);
          dndy[2] = x * (1.0 - z);
          dndy[3] = (1.0 - x) * (1.0 - z);
          dndy[4] = -(1.0 - x) * z;
          dndy[5] = -x * z;
          dndy[6] = x * z;
          dndy[7] = (1.0 - x) * z;
          dndz[0] = -(1.0 - x) * (1.0 - y);
          dndz[1] = -x * (1.0 - y);
          dndz[2] = -x * y;
          dndz[3] = -(1.0 - x) * y;
          dndz[4] = (1.0 - x) * (1.0 - y);
          dndz[5] = x * (1.0 - y);
          dndz[6] = x * y;
          dndz[7] = (1.0 - x) * y;
          double es[6][8][3];
          memset(es, 0, sizeof es);
          for (int n8 = 0; n8 < 8; ++n8) {
            es[0][n8][0] = dndx[n8];
            es[1][n8][1] = dndy[n8];
            es[2][n8][2] = dndz[n8];
            es[3][n8][0] = dndz[n8];
            es[3][n8][2] = dndx[n8];
            es[4][n8][1] = dndz[n8];
            es[4][n8][2] = dndy[n8];
            es[5][n8][0] = dndy[n8];
            es[5][n8][1] = dndx[n8];
          }
          const double w = g[i3][j3][k3];
          for (int mm = 0; mm < 3; ++mm)
            for (int nn = 0; nn < 3; ++nn)
              for (int ii = 0; ii < 8; ++ii)
                for (int jj = 0; jj < 8; ++jj) {
                  /* sumval = left . (cmod * right) */
                  double cr[6];
                  for (int r = 0; r < 6; ++r) {
                    double s = 0.0;
                    for (int c = 0; c < 6; ++c) s += C6[r][c] * es[c][jj][nn];
                    cr[r] = s;
                  }
                  double sumval = 0.0;
                  for (int r = 0; r < 6; ++r) sumval += es[r][ii][mm] * cr[r];
                  dk[DK(np, ph, ii, mm, jj, nn)] += w * sumval / 216.0;
                }
        }
  }
}

void orc_build_ib(int32_t nx, int32_t ny, int32_t nz, int32_t* ib) {
  const size_t ns = (size_t)nx * ny * nz;
#pragma omp parallel for collapse(2) schedule(guided)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t m = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
        for (int n = 0; n < 27; ++n) {
          int i1 = i + IM[n], j1 = j + JM[n], k1 = k + KM[n];
          if (i1 < 0) i1 += nx;
          if (i1 >= nx) i1 -= nx;
          if (j1 < 0) j1 += ny;
          if (j1 >= ny) j1 -= ny;
          if (k1 < 0) k1 += nz;
          if (k1 >= nz) k1 -= nz;
          ib[m + ns * n] = (int32_t)((size_t)i1 + (size_t)nx * ((size_t)j1 + (size_t)ny * k1));
        }
      }
}

/* One boundary element: b(ib(m,is(mm)),nn) += sum delta.dk ; C += 0.5 delta.dk.delta
 * (src/elas3dxtal_pcg.f90:837-850).  delta is [8][3] (reference local order). */
static const int IS_NBR[8] = {26, 2, 1, 0, 25, 18, 17, 16}; /* is = 27,3,2,1,26,19,18,17 */

static void bc_element(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                       const double* dk, size_t m, double delta[8][3], double* b,
                       double* C) {
  const int np = p->nphase;
  const size_t ns = (size_t)p->nx * p->ny * p->nz;
  const int ph = pix[m] - 1;
  for (int nn = 0; nn < 3; ++nn)
    for (int mm = 0; mm < 8; ++mm) {
      double sumval = 0.0;
      for (int m3 = 0; m3 < 3; ++m3)
        for (int m8 = 0; m8 < 8; ++m8) {
          const double d = dk[DK(np, ph, m8, m3, mm, nn)];
          sumval += delta[m8][m3] * d;
          *C += 0.5 * delta[m8][m3] * d * delta[mm][nn];
        }
      const size_t ind = (size_t)ib[m + ns * IS_NBR[mm]];
      b[ind + ns * nn] += sumval;
    }
}

void orc_femat_bc(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                  const double* dk, double* b, double* C) {
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  const size_t nxy = (size_t)nx * ny, ns = nxy * nz;
  const double exx = p->exx, eyy = p->eyy, ezz = p->ezz;
  const double exz = p->exz, eyz = p->eyz, exy = p->exy;
  memset(b, 0, sizeof(double) * 3 * ns);
  double Cacc = 0.0;
  double delta[8][3];
#define SETD(n, a, bb, c) \
  do {                    \
    delta[n][0] = (a);    \
    delta[n][1] = (bb);   \
    delta[n][2] = (c);    \
  } while (0)

  /* Face x = nx (src/elas3dxtal_pcg.f90:821-854) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8)
    if (i8 == 1 || i8 == 2 || i8 == 5 || i8 == 6) SETD(i8, exx * nx, exy * nx, exz * nx);
  for (int j = 1; j <= ny - 1; ++j)
    for (int k = 1; k <= nz - 1; ++k) {
      const size_t m = nxy * (k - 1) + (size_t)j * nx - 1;
      bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
    }
  /* Face y = ny (:856-886) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8)
    if (i8 == 2 || i8 == 3 || i8 == 6 || i8 == 7) SETD(i8, exy * ny, eyy * ny, eyz * ny);
  for (int i = 1; i <= nx - 1; ++i)
    for (int k = 1; k <= nz - 1; ++k) {
      const size_t m = nxy * (k - 1) + (size_t)nx * (ny - 1) + i - 1;
      bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
    }
  /* Face z = nz (:888-918) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8)
    if (i8 >= 4) SETD(i8, exz * nz, eyz * nz, ezz * nz);
  for (int i = 1; i <= nx - 1; ++i)
    for (int j = 1; j <= ny - 1; ++j) {
      const size_t m = nxy * (nz - 1) + (size_t)nx * (j - 1) + i - 1;
      bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
    }
  /* Edge x = nx, y = ny (:920-959) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8) {
    if (i8 == 1 || i8 == 5) SETD(i8, exx * nx, exy * nx, exz * nx);
    if (i8 == 3 || i8 == 7) SETD(i8, exy * ny, eyy * ny, eyz * ny);
    if (i8 == 2 || i8 == 6) SETD(i8, exy * ny + exx * nx, eyy * ny + exy * nx, eyz * ny + exz * nx);
  }
  for (int k = 1; k <= nz - 1; ++k) {
    const size_t m = nxy * k - 1;
    bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
  }
  /* Edge x = nx, z = nz (:961-999) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8) {
    if (i8 == 1 || i8 == 2) SETD(i8, exx * nx, exy * nx, exz * nx);
    if (i8 == 4 || i8 == 7) SETD(i8, exz * nz, eyz * nz, ezz * nz);
    if (i8 == 5 || i8 == 6) SETD(i8, exz * nz + exx * nx, eyz * nz + exy * nx, ezz * nz + exz * nx);
  }
  for (int j = 1; j <= ny - 1; ++j) {
    const size_t m = nxy * (nz - 1) + (size_t)nx * (j - 1) + nx - 1;
    bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
  }
  /* Edge y = ny, z = nz (:1001-1039) */
  memset(delta, 0, sizeof delta);
  for (int i8 = 0; i8 < 8; ++i8) {
    if (i8 == 4 || i8 == 5) SETD(i8, exz * nz, eyz * nz, ezz * nz);
    if (i8 == 2 || i8 == 3) SETD(i8, exy * ny, eyy * ny, eyz * ny);
    if (i8 == 6 || i8 == 7) SETD(i8, exy * ny + exz * nz, eyy * ny + eyz * nz, eyz * ny + ezz * nz);
  }
  for (int i = 1; i <= nx - 1; ++i) {
    const size_t m = nxy * (nz - 1) + (size_t)nx * (ny - 1) + i - 1;
    bc_element(p, pix, ib, dk, m, delta, b, &Cacc);
  }
  /* Corner x = nx, y = ny, z = nz (:1041-1094) */
  memset(delta, 0, sizeof delta);
  SETD(1, exx * nx, exy * nx, exz * nx);
  SETD(3, exy * ny, eyy * ny, eyz * ny);
  SETD(4, exz * nz, eyz * nz, ezz * nz);
  SETD(7, exy * ny + exz * nz, eyy * ny + eyz * nz, eyz * ny + ezz * nz);
  SETD(5, exx * nx + exz * nz, exy * nx + eyz * nz, exz * nx + ezz * nz);
  SETD(2, exx * nx + exy * ny, exy * nx + eyy * ny, exz * nx + eyz * ny);
  SETD(6, exx * nx + exy * ny + exz * nz, exy * nx + eyy * ny + eyz * nz,
       exz * nx + eyz * ny + ezz * nz);
  bc_element(p, pix, ib, dk, ns - 1, delta, b, &Cacc);
#undef SETD
  *C = Cacc;
}

void orc_femat(const orc_problem* p, const int32_t* pix, const int32_t* ib,
               const double* rod, double* cmod, double* dk, double* b, double* C) {
  orc_cmod(p, rod, cmod);
  orc_dk(p, cmod, dk);
  orc_femat_bc(p, pix, ib, dk, b, C);
}

void orc_affine_u(const orc_problem* p, double* u) {
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  const size_t ns = (size_t)nx * ny * nz;
#pragma omp parallel for collapse(2) schedule(guided)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t m = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
        const double x = i, y = j, z = k;
        u[m] = x * p->exx + y * p->exy + z * p->exz;
        u[m + ns] = x * p->exy + y * p->eyy + z * p->eyz;
        u[m + 2 * ns] = x * p->exz + y * p->eyz + z * p->ezz;
      }
}

/* Stencil for one node, three rows (src/elas3dxtal_pcg.f90:1592-1878). */
static inline void stencil_node(const nbr_terms* terms, int np, const int32_t* pix,
                                const int32_t* ib, const double* dk, const double* x,
                                size_t ns, size_t m, double out[3]) {
  int ibl[27], pl[8];
  for (int n = 0; n < 27; ++n) ibl[n] = ib[m + ns * n];
  for (int e = 0; e < 8; ++e) pl[e] = pix[ibl[ELEM_NBR[e]]] - 1;
  static const int LOCAL_OF_M[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  for (int j = 0; j < 3; ++j) {
    double s = 0.0;
    for (int n = 0; n < 3; ++n)
      for (int q = 0; q < 27; ++q) {
        const nbr_terms* t = &terms[q];
        double coef = 0.0;
        for (int c = 0; c < t->count; ++c) {
          const int e = t->e[c];
          coef += dk[DK(np, pl[e], LOCAL_OF_M[e], j, t->b[c], n)];
        }
        s += x[(size_t)ibl[q] + ns * n] * coef;
      }
    out[j] = s;
  }
}

void orc_apply(const orc_problem* p, const int32_t* pix, const int32_t* ib,
               const double* dk, const double* x, double* y) {
  nbr_terms terms[27];
  build_terms(terms);
  const size_t ns = (size_t)p->nx * p->ny * p->nz;
  const size_t bs = p->block_size > 0 ? (size_t)p->block_size : 8192;
  for (size_t L1 = 0; L1 < ns; L1 += bs) {
    const size_t L2 = (L1 + bs < ns) ? L1 + bs : ns;
#pragma omp parallel for schedule(guided)
    for (size_t m = L1; m < L2; ++m) {
      double o[3];
      stencil_node(terms, p->nphase, pix, ib, dk, x, ns, m, o);
      y[m] = o[0];
      y[m + ns] = o[1];
      y[m + 2 * ns] = o[2];
    }
  }
}

/* Deterministic dot product over n values: fixed-size chunk partials summed in order. */
static double ddot(const double* a, const double* b, size_t n) {
  const size_t nc = (n + RCHUNK - 1) / RCHUNK;
  double* part = (double*)malloc(sizeof(double) * (nc ? nc : 1));
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    const size_t lo = c * RCHUNK, hi = (lo + RCHUNK < n) ? lo + RCHUNK : n;
    double s = 0.0;
    for (size_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0.0;
  for (size_t c = 0; c < nc; ++c) s += part[c];
  free(part);
  return s;
}

void orc_energy(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                const double* dk, const double* b, double C, const double* u,
                double* gb, double* utot) {
  const size_t ns = (size_t)p->nx * p->ny * p->nz;
  orc_apply(p, pix, ib, dk, u, gb);
  /* utot = C + sum(0.5 u.gb + b.u); gb += b  (src/elas3dxtal_pcg.f90:1332-1340) */
  const size_t n = 3 * ns;
  const size_t nc = (n + RCHUNK - 1) / RCHUNK;
  double* part = (double*)malloc(sizeof(double) * (nc ? nc : 1));
#pragma omp parallel for schedule(static)
  for (size_t c = 0; c < nc; ++c) {
    const size_t lo = c * RCHUNK, hi = (lo + RCHUNK < n) ? lo + RCHUNK : n;
    double s = 0.0;
    for (size_t i = lo; i < hi; ++i) {
      s += 0.5 * u[i] * gb[i] + b[i] * u[i];
      gb[i] = gb[i] + b[i];
    }
    part[c] = s;
  }
  double s = C;
  for (size_t c = 0; c < nc; ++c) s += part[c];
  free(part);
  *utot = s;
}

void orc_invert3x3(const double* a, double* ainv) {
#define A(i, j) a[(i - 1) + 3 * (j - 1)]
#define AI(i, j) ainv[(i - 1) + 3 * (j - 1)]
  const double c11 = A(2, 2) * A(3, 3) - A(2, 3) * A(3, 2);
  const double c21 = -A(2, 1) * A(3, 3) + A(2, 3) * A(3, 1);
  const double c31 = A(2, 1) * A(3, 2) - A(2, 2) * A(3, 1);
  const double det = A(1, 1) * c11 + A(1, 2) * c21 + A(1, 3) * c31;
  if (fabs(det) < 1e-14) {
    for (int i = 0; i < 9; ++i) ainv[i] = 0.0;
    return;
  }
  const double inv_det = 1.0 / det;
  const double c12 = -A(1, 2) * A(3, 3) + A(1, 3) * A(3, 2);
  const double c22 = A(1, 1) * A(3, 3) - A(1, 3) * A(3, 1);
  const double c32 = -A(1, 1) * A(3, 2) + A(1, 2) * A(3, 1);
  const double c13 = A(1, 2) * A(2, 3) - A(1, 3) * A(2, 2);
  const double c23 = -A(1, 1) * A(2, 3) + A(1, 3) * A(2, 1);
  const double c33 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
  AI(1, 1) = c11 * inv_det;
  AI(2, 1) = c21 * inv_det;
  AI(3, 1) = c31 * inv_det;
  AI(1, 2) = c12 * inv_det;
  AI(2, 2) = c22 * inv_det;
  AI(3, 2) = c32 * inv_det;
  AI(1, 3) = c13 * inv_det;
  AI(2, 3) = c23 * inv_det;
  AI(3, 3) = c33 * inv_det;
#undef A
#undef AI
}

void orc_block_jacobi(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                      const double* dk, double* minv) {
  const size_t ns = (size_t)p->nx * p->ny * p->nz;
  const int np = p->nphase;
#pragma omp parallel for schedule(guided)
  for (size_t m = 0; m < ns; ++m) {
    int pl[8];
    for (int e = 0; e < 8; ++e) pl[e] = pix[ib[m + ns * ELEM_NBR[e]]] - 1;
    double M[9], Mi[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = dk[DK(np, pl[0], 0, i, 0, j)] + dk[DK(np, pl[1], 1, i, 1, j)];
        s += dk[DK(np, pl[2], 2, i, 2, j)] + dk[DK(np, pl[3], 3, i, 3, j)];
        s += dk[DK(np, pl[4], 4, i, 4, j)] + dk[DK(np, pl[5], 5, i, 5, j)];
        s += dk[DK(np, pl[6], 6, i, 6, j)] + dk[DK(np, pl[7], 7, i, 7, j)];
        M[i + 3 * j] = s;
      }
    orc_invert3x3(M, Mi);
    for (int i = 0; i < 9; ++i) minv[m + ns * i] = Mi[i];
  }
}

static void precond(const double* minv, const double* g, double* z, size_t ns) {
#pragma omp parallel for schedule(guided)
  for (size_t m = 0; m < ns; ++m)
    for (int i = 0; i < 3; ++i)
      z[m + ns * i] = minv[m + ns * (i + 0)] * g[m] + minv[m + ns * (i + 3)] * g[m + ns] +
                      minv[m + ns * (i + 6)] * g[m + 2 * ns];
}

/* State of one PCG solve (dembx_OpenMP, src/elas3dxtal_pcg.f90:1356-2043),
 * split into set-up, iterations and tear-down so that a caller can time the
 * iterations alone and run them in several calls without restarting the
 * search direction.  u, gb and h stay caller-owned. */
struct orc_pcg {
  const orc_problem* p;
  const int32_t *pix, *ib;
  const double* dk;
  double *u, *gb, *h, *Ah, *z, *minv, *history;
  double gg, gg0_eff, rel_res_prev;
  int32_t L, resets, reason, done;
};

orc_pcg* orc_pcg_begin(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                       const double* dk, double* u, double* gb, double* h, int32_t kkk,
                       double gg0, double* history) {
  const size_t ns = (size_t)p->nx * p->ny * p->nz, n3 = 3 * ns;
  orc_pcg* s = (orc_pcg*)calloc(1, sizeof(orc_pcg));
  if (!s) return NULL;
  s->p = p, s->pix = pix, s->ib = ib, s->dk = dk, s->u = u, s->gb = gb, s->h = h, s->history = history;
  s->Ah = (double*)malloc(sizeof(double) * n3);
  s->z = (double*)malloc(sizeof(double) * n3);
  s->minv = (double*)malloc(sizeof(double) * 9 * ns);
  if (!s->Ah || !s->z || !s->minv) {
    orc_pcg_end(s, NULL, NULL, NULL);
    return NULL;
  }
  /* kkk == 1 builds the preconditioner (src/elas3dxtal_pcg.f90:1498-1520);
   * kmax = 1 in the reference so it is always built here.  precond == 1 is the
   * unpreconditioned CG of applications/sec3_1/cg/n_100x100x100/elas3dxtal_cg.f90:
   * 1011-1060 (z = g, no divergence reset). */
  if (p->precond == 1) {
    memset(s->minv, 0, sizeof(double) * 9 * ns);
    for (size_t m = 0; m < ns; ++m) s->minv[m] = s->minv[m + 4 * ns] = s->minv[m + 8 * ns] = 1.0;
  } else {
    orc_block_jacobi(p, pix, ib, dk, s->minv);
  }
  precond(s->minv, gb, s->z, ns);
  s->gg = ddot(s->z, gb, n3);
  if (kkk == 1) memcpy(h, s->z, sizeof(double) * n3);
  s->gg0_eff = (p->criterion == 1) ? s->gg : gg0;
  s->rel_res_prev = sqrt(s->gg / s->gg0_eff);
  s->reason = 2;
  return s;
}

int32_t orc_pcg_iterate(orc_pcg* s, int32_t nsteps) {
  const orc_problem* p = s->p;
  const size_t ns = (size_t)p->nx * p->ny * p->nz, n3 = 3 * ns;
  double *u = s->u, *gb = s->gb, *h = s->h, *Ah = s->Ah, *z = s->z;
  const double tol = (double)p->tol;
  for (int32_t k = 0; k < nsteps && !s->done; ++k) {
    if (s->L >= p->ldemb) { /* ldemb iterations done (:1574) */
      s->reason = 2;
      s->done = 1;
      break;
    }
    s->L++;
    orc_apply(p, s->pix, s->ib, s->dk, h, Ah);
    const double hAh = ddot(h, Ah, n3);
    if (fabs(hAh) < 1e-14) {
      s->reason = 1;
      s->done = 1;
      break;
    }
    const double lambda = s->gg / hAh;
#pragma omp parallel for schedule(guided)
    for (size_t i = 0; i < n3; ++i) {
      u[i] = u[i] - lambda * h[i];
      gb[i] = gb[i] - lambda * Ah[i];
    }
    precond(s->minv, gb, z, ns);
    const double gglast = s->gg;
    s->gg = ddot(z, gb, n3);
    const double rel_res = sqrt(s->gg / s->gg0_eff);
    if (s->history) s->history[s->L - 1] = rel_res;
    if (p->divergence_reset && rel_res > 10.0 * s->rel_res_prev && s->L > 1) {
      memcpy(h, z, sizeof(double) * n3);
      s->resets++;
    } else {
      const double gamma = s->gg / gglast;
#pragma omp parallel for schedule(guided)
      for (size_t i = 0; i < n3; ++i) h[i] = z[i] + gamma * h[i];
    }
    s->rel_res_prev = rel_res;
    if (rel_res < tol) {
      s->reason = 0;
      s->done = 1;
      break;
    }
  }
  if (!s->done && s->L >= p->ldemb) {
    s->reason = 2;
    s->done = 1;
  }
  return s->done ? s->reason : -1;
}

void orc_pcg_end(orc_pcg* s, int32_t* lstep, double* gg_out, int32_t* reset_count) {
  if (!s) return;
  if (lstep) *lstep = s->L;
  if (gg_out) *gg_out = s->gg;
  if (reset_count) *reset_count = s->resets;
  free(s->Ah);
  free(s->z);
  free(s->minv);
  free(s);
}

int32_t orc_dembx(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                  const double* dk, double* u, double* gb, double* h, int32_t kkk,
                  double gg0, int32_t max_steps, int32_t* lstep, double* gg_out,
                  double* history, int32_t* reset_count) {
  orc_pcg* s = orc_pcg_begin(p, pix, ib, dk, u, gb, h, kkk, gg0, history);
  if (!s) return -1;
  const int32_t limit = (max_steps > 0 && max_steps < p->ldemb) ? max_steps : p->ldemb;
  int32_t reason = orc_pcg_iterate(s, limit);
  if (reason < 0) reason = 2;
  orc_pcg_end(s, lstep, gg_out, reset_count);
  return reason;
}

/* Gather the 8 nodal displacements of voxel (i,j,k) with the periodic jump
 * (src/elas3dxtal_pcg.f90:2269-2323).  uu is [8][3] in reference local order. */
static void gather_voxel(const orc_problem* p, const double* u, int i, int j, int k,
                         double uu[8][3]) {
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  const size_t ns = (size_t)nx * ny * nz;
  for (int a = 0; a < 8; ++a) {
    int i1 = i + LOX[a], j1 = j + LOY[a], k1 = k + LOZ[a];
    if (i1 >= nx) i1 -= nx;
    if (j1 >= ny) j1 -= ny;
    if (k1 >= nz) k1 -= nz;
    const size_t mm = (size_t)i1 + (size_t)nx * ((size_t)j1 + (size_t)ny * k1);
    for (int c = 0; c < 3; ++c) uu[a][c] = u[mm + ns * c];
  }
  if (i == nx - 1) {
    const int nodes[4] = {1, 2, 5, 6};
    for (int t = 0; t < 4; ++t) {
      uu[nodes[t]][0] += p->exx * (double)nx;
      uu[nodes[t]][1] += p->exy * (double)nx;
      uu[nodes[t]][2] += p->exz * (double)nx;
    }
  }
  if (j == ny - 1) {
    const int nodes[4] = {2, 3, 6, 7};
    for (int t = 0; t < 4; ++t) {
      uu[nodes[t]][0] += p->exy * (double)ny;
      uu[nodes[t]][1] += p->eyy * (double)ny;
      uu[nodes[t]][2] += p->eyz * (double)ny;
    }
  }
  if (k == nz - 1) {
    const int nodes[4] = {4, 5, 6, 7};
    for (int t = 0; t < 4; ++t) {
      uu[nodes[t]][0] += p->exz * (double)nz;
      uu[nodes[t]][1] += p->eyz * (double)nz;
      uu[nodes[t]][2] += p->ezz * (double)nz;
    }
  }
}

/* Centre-point B matrix (src/elas3dxtal_pcg.f90:2224-2238). */
static void centre_es(double es[6][8][3]) {
  static const double dndx[8] = {-0.25, 0.25, 0.25, -0.25, -0.25, 0.25, 0.25, -0.25};
  static const double dndy[8] = {-0.25, -0.25, 0.25, 0.25, -0.25, -0.25, 0.25, 0.25};
  static const double dndz[8] = {-0.25, -0.25, -0.25, -0.25, 0.25, 0.25, 0.25, 0.25};
  memset(es, 0, sizeof(double) * 144);
  for (int n = 0; n < 8; ++n) {
    es[0][n][0] = dndx[n];
    es[1][n][1] = dndy[n];
    es[2][n][2] = dndz[n];
    es[3][n][0] = dndz[n];
    es[3][n][2] = dndx[n];
    es[4][n][1] = dndz[n];
    es[4][n][2] = dndy[n];
    es[5][n][0] = dndy[n];
    es[5][n][1] = dndx[n];
  }
}

void orc_stress(const orc_problem* p, const int32_t* pix, const double* cmod,
                const double* u, double* strav, double* epsav) {
  const int nx = p->nx, ny = p->ny, nz = p->nz, np = p->nphase;
  const size_t ns = (size_t)nx * ny * nz;
  double es[6][8][3];
  centre_es(es);
  /* Deterministic reduction: one partial per (j,k) row, summed in order. */
  const size_t nrows = (size_t)ny * nz;
  double* part = (double*)malloc(sizeof(double) * 12 * nrows);
#pragma omp parallel for schedule(guided)
  for (size_t row = 0; row < nrows; ++row) {
    const int j = (int)(row % ny), k = (int)(row / ny);
    double acc[12] = {0};
    for (int i = 0; i < nx; ++i) {
      double uu[8][3];
      gather_voxel(p, u, i, j, k, uu);
      const size_t m = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
      const int ph = pix[m] - 1;
      double st[6] = {0}, s[6] = {0};
      for (int n3 = 0; n3 < 3; ++n3)
        for (int n8 = 0; n8 < 8; ++n8) {
          for (int r = 0; r < 6; ++r) s[r] += es[r][n8][n3] * uu[n8][n3];
          for (int n = 0; n < 6; ++n)
            for (int r = 0; r < 6; ++r)
              st[r] += cmod[ph + np * (r + 6 * n)] * es[n][n8][n3] * uu[n8][n3];
        }
      for (int r = 0; r < 6; ++r) {
        acc[r] += st[r];
        acc[6 + r] += s[r];
      }
    }
    for (int t = 0; t < 12; ++t) part[12 * row + t] = acc[t];
  }
  double tot[12] = {0};
  for (size_t row = 0; row < nrows; ++row)
    for (int t = 0; t < 12; ++t) tot[t] += part[12 * row + t];
  free(part);
  for (int r = 0; r < 6; ++r) {
    strav[r] = tot[r] / (double)ns;
    epsav[r] = tot[6 + r] / (double)ns;
  }
}

void orc_stress_fullfield(const orc_problem* p, const int32_t* pix,
                          const double* cmod, const double* u, double* sigma,
                          double* vm) {
  const int nx = p->nx, ny = p->ny, nz = p->nz, np = p->nphase;
  const size_t ns = (size_t)nx * ny * nz;
  double es[6][8][3];
  centre_es(es);
#pragma omp parallel for collapse(2) schedule(guided)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double uu[8][3];
        gather_voxel(p, u, i, j, k, uu);
        const size_t m = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
        double eps[6] = {0};
        for (int n3 = 0; n3 < 3; ++n3)
          for (int n8 = 0; n8 < 8; ++n8)
            for (int r = 0; r < 6; ++r) eps[r] += es[r][n8][n3] * uu[n8][n3];
        const int ph = pix[m] - 1;
        double s6[6];
        for (int r = 0; r < 6; ++r) {
          double s = 0.0;
          for (int c = 0; c < 6; ++c) s += cmod[ph + np * (r + 6 * c)] * eps[c];
          s6[r] = s;
          sigma[m + ns * r] = s;
        }
        /* von Mises as written at src/elas3dxtal_pcg.f90:2826-2831 */
        vm[m] = sqrt(0.5 * ((s6[0] - s6[1]) * (s6[0] - s6[1]) + (s6[1] - s6[2]) * (s6[1] - s6[2]) +
                            (s6[2] - s6[0]) * (s6[2] - s6[0]) +
                            6.0 * (s6[3] * s6[3] + s6[4] * s6[4] + s6[5] * s6[5])));
      }
}

void orc_assig(const orc_problem* p, const int32_t* pix, double* prob) {
  const size_t ns = (size_t)p->nx * p->ny * p->nz;
  for (int i = 0; i < p->nphase; ++i) prob[i] = 0.0;
  for (size_t m = 0; m < ns; ++m)
    if (pix[m] >= 1 && pix[m] <= p->nphase) prob[pix[m] - 1] += 1.0;
  for (int i = 0; i < p->nphase; ++i) prob[i] /= (double)ns;
}

int32_t orc_run(const orc_problem* p, const int32_t* pix, const double* rod,
                double* u, double* history, orc_result* res) {
  const size_t ns = (size_t)p->nx * p->ny * p->nz, n3 = 3 * ns;
  const int np = p->nphase;
  int32_t* ib = (int32_t*)malloc(sizeof(int32_t) * 27 * ns);
  double* cmod = (double*)malloc(sizeof(double) * 36 * (size_t)np);
  double* dk = (double*)malloc(sizeof(double) * 576 * (size_t)np);
  double* b = (double*)malloc(sizeof(double) * n3);
  double* gb = (double*)malloc(sizeof(double) * n3);
  double* h = (double*)calloc(n3, sizeof(double));
  if (!ib || !cmod || !dk || !b || !gb || !h) {
    free(ib), free(cmod), free(dk), free(b), free(gb), free(h);
    return -1;
  }
  memset(res, 0, sizeof *res);
  orc_build_ib(p->nx, p->ny, p->nz, ib);
  double t0 = wtime();
  double C;
  orc_femat(p, pix, ib, rod, cmod, dk, b, &C);
  res->C = C;
  double t1 = wtime();
  orc_affine_u(p, u);
  double utot;
  orc_energy(p, pix, ib, dk, b, C, u, gb, &utot);
  res->utot0 = utot;
  const double gg0 = ddot(gb, gb, n3);
  res->gg0 = gg0;
  double t2 = wtime();
  int32_t L = 0, resets = 0;
  double gg = 0.0;
  res->exit_reason = orc_dembx(p, pix, ib, dk, u, gb, h, 1, gg0, 0, &L, &gg, history, &resets);
  double t3 = wtime();
  orc_energy(p, pix, ib, dk, b, C, u, gb, &utot);
  double t4 = wtime();
  orc_stress(p, pix, cmod, u, res->strav, res->epsav);
  double t5 = wtime();
  res->utot = utot;
  res->gg = gg;
  res->lstep = L;
  res->reset_count = resets;
  res->rel_res = sqrt(gg / gg0);
  res->t_femat = t1 - t0;
  res->t_energy = (t2 - t1) + (t4 - t3);
  res->t_pcg = t3 - t2;
  res->t_stress = t5 - t4;
  free(ib), free(cmod), free(dk), free(b), free(gb), free(h);
  return 0;
}
