/*
 * e3d_oracle.h -- CPU oracle for the ELAS3D-Xtal voxel-FE PCG solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C/OpenMP restatement of the
 * reference's algorithm (src/elas3dxtal_pcg.f90) that the tests compare the
 * CUDA library against, and the timed CPU baseline.  Nothing in the product library
 * links, loads or calls it.
 *
 * Parity status: UNPINNED by reference outputs.  The reference ships no tests,
 * golden vectors or result files, and it cannot be compiled here (Fortran +
 * HDF5).  The oracle is pinned instead by analytical known-answer tests
 * (homogeneous medium, rigid translation, symmetry, PSD element matrices,
 * orientation invariance at Zener ratio 1, volume-average identities) and by an
 * independent scipy sparse-assembly restatement (oracle/np_ref.py).
 *
 * Data layout follows the reference exactly (Fortran column-major, 1-based
 * phase ids):
 *   node m (0-based)   = i + nx*(j + ny*k)
 *   u, gb, b, h (ns,3) = x[c*ns + m]
 *   dk(nphase,8,3,8,3) = dk[p + np*(a + 8*(i + 3*(b + 8*j)))]   (0-based p,a,i,b,j)
 *   cmod(nphase,6,6)   = cmod[p + np*(i + 6*j)]
 *   ib(ns,27)          = ib[m + ns*n]
 *   Minv(ns,3,3)       = minv[m + ns*(i + 3*j)]
 *   pix(ns)            = phase id in [1, nphase]
 */
#ifndef E3D_ORACLE_H
#define E3D_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem {
  int32_t nx, ny, nz;      /* nodes per direction (fully periodic: ns = nx*ny*nz) */
  int32_t nphase;          /* grains + 1 (last phase = inclusion / pore)          */
  int32_t flag_m;          /* 0: isotropic matrix, 1: rotated cubic polycrystal   */
  double c11, c12, c44;    /* cubic single-crystal constants (Pa)                 */
  double e1, nu1;          /* inclusion Young's modulus and Poisson ratio         */
  double exx, eyy, ezz, exz, eyz, exy;   /* applied macro strain (tensor comps)  */
  float tol;               /* convergence tolerance, single precision as in ref  */
  int32_t ldemb;           /* max PCG iterations                                  */
  int32_t criterion;       /* 0 = reference sqrt(z.g/|g0|^2), 1 = sqrt(z.g/z0.g0) */
  int32_t divergence_reset;/* 1 = reset h = z when rel_res jumps > 10x           */
  int32_t block_size;      /* apply chunk (reference: 8192)                       */
  int32_t precond;         /* 0 block-Jacobi, 1 none (applications/sec3_1/cg)     */
} orc_problem;

/* Rodrigues -> Bond-rotated cubic stiffness, row-major 36 per grain
 * (rotatestiffnessby, src/elas3dxtal_pcg.f90:2470-2637). */
void orc_rotate_stiffness(int32_t ngrains, const double* rod, double c11,
                          double c12, double c44, double* rotated);

/* Phase stiffness table cmod(nphase,6,6) (src/elas3dxtal_pcg.f90:295-317, 655-705). */
void orc_cmod(const orc_problem* p, const double* rod, double* cmod);

/* Element stiffness dk(nphase,8,3,8,3) by 3x3x3 Simpson (src/elas3dxtal_pcg.f90:713-805). */
void orc_dk(const orc_problem* p, const double* cmod, double* dk);

/* Periodic neighbour table ib(ns,27) (src/elas3dxtal_pcg.f90:326-369). */
void orc_build_ib(int32_t nx, int32_t ny, int32_t nz, int32_t* ib);

/* Periodic-jump force b(ns,3) and constant C (src/elas3dxtal_pcg.f90:815-1100). */
void orc_femat_bc(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                  const double* dk, double* b, double* C);

/* Full femat: cmod, dk, b, C (femat_OpenMP, src/elas3dxtal_pcg.f90:555-1104). */
void orc_femat(const orc_problem* p, const int32_t* pix, const int32_t* ib,
               const double* rod, double* cmod, double* dk, double* b, double* C);

/* Affine initial guess u = E.x (src/elas3dxtal_pcg.f90:423-438). */
void orc_affine_u(const orc_problem* p, double* u);

/* y = K x, 27-point stencil (src/elas3dxtal_pcg.f90:1176-1321, 1585-1883). */
void orc_apply(const orc_problem* p, const int32_t* pix, const int32_t* ib,
               const double* dk, const double* x, double* y);

/* gb = K u + b, utot = C + sum(0.5 u.Ku + b.u) (energy_OpenMP, :1107-1353). */
void orc_energy(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                const double* dk, const double* b, double C, const double* u,
                double* gb, double* utot);

/* 3x3 block inverse, zero if |det| < 1e-14 (invert3x3, :2046-2147).
 * a and ainv are column-major 3x3. */
void orc_invert3x3(const double* a, double* ainv);

/* Block-Jacobi inverse blocks Minv(ns,3,3) (:1498-1520). */
void orc_block_jacobi(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                      const double* dk, double* minv);

/* PCG solve (dembx_OpenMP, :1356-2043).  u, gb, h are in/out.  history
 * (length ldemb) receives rel_res per iteration.  Returns the exit reason:
 * 0 converged, 1 hAh guard, 2 max iterations.  max_steps <= 0 means ldemb. */
int32_t orc_dembx(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                  const double* dk, double* u, double* gb, double* h,
                  int32_t kkk, double gg0, int32_t max_steps, int32_t* lstep,
                  double* gg_out, double* history, int32_t* reset_count);

/* The same solve in three steps: set-up (block-Jacobi build, z0, gg,
 * h = z0), nsteps iterations per orc_pcg_iterate call (the search direction
 * carries over between calls), and tear-down.  orc_pcg_iterate returns the
 * exit reason once the solve has ended and -1 while it is still running. */
typedef struct orc_pcg orc_pcg;
orc_pcg* orc_pcg_begin(const orc_problem* p, const int32_t* pix, const int32_t* ib,
                       const double* dk, double* u, double* gb, double* h,
                       int32_t kkk, double gg0, double* history);
int32_t orc_pcg_iterate(orc_pcg* s, int32_t nsteps);
void orc_pcg_end(orc_pcg* s, int32_t* lstep, double* gg_out, int32_t* reset_count);

/* Volume-averaged stress and engineering strain, Voigt xx,yy,zz,xz,yz,xy
 * (stress_OpenMP, :2149-2408). */
void orc_stress(const orc_problem* p, const int32_t* pix, const double* cmod,
                const double* u, double* strav, double* epsav);

/* Per-voxel stress(ns,6) and von Mises(ns) (stress_fullfield_OpenMP, :2723-2833). */
void orc_stress_fullfield(const orc_problem* p, const int32_t* pix,
                          const double* cmod, const double* u, double* sigma,
                          double* vm);

/* Phase volume fractions prob(nphase) (assig, :2410-2468). */
void orc_assig(const orc_problem* p, const int32_t* pix, double* prob);

/* Whole driver (program elas3d, :186-552) without file I/O.  Outputs the
 * initial energy, final energy, gg0, final gg, iteration count and the
 * averaged stress/strain.  u receives the converged displacement. */
typedef struct orc_result {
  double utot0, utot, gg0, gg, rel_res;
  int32_t lstep, exit_reason, reset_count;
  double strav[6], epsav[6];
  double C;
  double t_femat, t_energy, t_pcg, t_stress;   /* seconds */
} orc_result;

int32_t orc_run(const orc_problem* p, const int32_t* pix, const double* rod,
                double* u, double* history, orc_result* res);

int32_t orc_num_threads(void);

/* Length of the chunks whose partial sums make every dot product (default
 * 4096; n <= 0 restores it).  Another length gives another, equally valid,
 * FP64 summation order. */
void orc_set_reduction_chunk(int64_t n);

#ifdef __cplusplus
}
#endif
#endif
