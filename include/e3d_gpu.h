/*
 * e3d_gpu.h -- C ABI of the GB300 (sm_103a) voxel-FE elasticity solver.
 *
 * Drop-in boundary for the hot path of ELAS3D-Xtal (src/elas3dxtal_pcg.f90).
 * The reference exposes no library: its "API" is five Fortran subroutines
 * called by `program elas3d` on a shared derived type `e3d`.  Each entry
 * point below replaces one of them and keeps its meaning; the reference
 * subroutine is cited beside it.  Plain C types only (int32_t, int64_t,
 * double*, opaque handle), so Fortran binds it through iso_c_binding, Python
 * through ctypes and C++ directly.
 *
 * Conventions (same as the reference's arrays, src/elas3dxtal_pcg.f90:155-181):
 *  - grid of nx*ny*nz nodes, fully periodic, node/voxel (i,j,k) (0-based) has
 *    linear index m = i + nx*(j + ny*k)  (Fortran column order);
 *  - vectors of 3 dof per node are component-major ("SoA"), i.e. Fortran
 *    u(ns,3): x[c*ns + m];
 *  - phase ids in pix are 1-based, in [1, nphase]; phase nphase is the
 *    inclusion / pore phase (E1, nu1 -- zero stiffness by default);
 *  - orientations are Rodrigues vectors r = q_xyz/q_w, 3 per grain, grains
 *    1..nphase-1 (src/elas3dxtal_pcg.f90:2538);
 *  - strains are TENSOR components (exx, eyy, ezz, exz, eyz, exy), as
 *    e3d%exx.. in the reference; averaged outputs use engineering shear and
 *    Voigt order xx, yy, zz, xz, yz, xy (src/elas3dxtal_pcg.f90:2235-2237).
 *
 * Ownership: host arrays are caller-owned and copied in/out; device state is
 * owned by the handle.  Threading: one handle per host thread; all work runs
 * on the handle's CUDA stream and every call returns after it completes.
 * Errors: every call returns an E3D_* status (the reference `stop`s instead).
 */
#ifndef E3D_GPU_H
#define E3D_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define E3D_OK 0
#define E3D_ERR_INPUT 1     /* bad argument / size / phase id out of range   */
#define E3D_ERR_OOM 2       /* device allocation failed or over hbm_budget    */
#define E3D_ERR_BREAKDOWN 3 /* NaN/Inf in h.Ah or z.g                         */
#define E3D_ERR_MAXITER 4   /* solve stopped at max_iter without converging   */
#define E3D_ERR_TIMEOUT 5   /* a device-side wait exceeded its limit          */
#define E3D_ERR_CUDA 6      /* CUDA runtime error (see e3d_last_cuda_error)   */
#define E3D_ERR_STATE 7     /* call out of order (e.g. solve before energy)   */

/* ---- solve exit reasons (e3d_solve_stats_t.exit_reason) ---- */
#define E3D_EXIT_CONVERGED 0 /* rel_res < tol (src/elas3dxtal_pcg.f90:2007)     */
#define E3D_EXIT_HAH_GUARD 1 /* |h.Ah| < 1e-14 (src/elas3dxtal_pcg.f90:1899)    */
#define E3D_EXIT_MAXITER 2   /* ldemb iterations (src/elas3dxtal_pcg.f90:1574)  */
#define E3D_EXIT_BREAKDOWN 3 /* non-finite scalar                               */
#define E3D_EXIT_TIMEOUT 4   /* device wait limit                               */
#define E3D_EXIT_RUNNING 5   /* iteration budget of an e3d_iterate call used up */

/* ---- stopping criterion ---- */
#define E3D_CRIT_REF 0         /* sqrt(z.g / |g0|^2), the reference's test (:1949, :452) */
#define E3D_CRIT_PRECOND_REL 1 /* sqrt(z.g / z0.g0), true preconditioned relative     */

/* ---- preconditioner ---- */
#define E3D_PRECOND_BLOCK_JACOBI 0 /* 3x3 point-block Jacobi (dembx_OpenMP, :1498-1535)       */
#define E3D_PRECOND_NONE 1         /* identity: the plain CG variant (applications/sec3_1/cg) */

/* ---- arithmetic ---- */
#define E3D_PREC_FP64 0  /* FP64 everywhere (the reference's arithmetic)           */
#define E3D_PREC_MIXED 1 /* FP32 stencil + preconditioner inside FP64 refinement   */

typedef struct e3d_problem {
  int32_t nx, ny, nz;       /* nodes per direction, ns = nx*ny*nz (md in the ref)  */
  int32_t nphase;           /* grains + 1                                           */
  int32_t flag_m;           /* 0 isotropic matrix, 1 rotated cubic polycrystal     */
  int32_t criterion;        /* E3D_CRIT_*                                          */
  int32_t precision;        /* E3D_PREC_*                                          */
  int32_t divergence_reset; /* 1: h = z when rel_res grows > 10x (:1961-1981)      */
  int32_t max_iter;         /* ldemb (:141)                                        */
  int32_t device;           /* CUDA device ordinal                                 */
  float tol;                /* single precision, as `real :: tol` (:148)           */
  int32_t refine_every;     /* MIXED: FP64 residual replacement period (0 = 50)    */
  int32_t preconditioner;   /* E3D_PRECOND_*                                       */
  int32_t refine_decades;   /* MIXED: also replace once the FP32 residual has fallen
                               this many decades below the last FP64 one (0: never) */
  double c11, c12, c44;     /* cubic constants, Pa (:100-102)                      */
  double e1, nu1;           /* inclusion Young's modulus / Poisson ratio (:114-115)*/
  double strain[6];         /* exx, eyy, ezz, exz, eyz, exy (tensor) (:394-399)    */
  int64_t hbm_budget;       /* bytes the handle may allocate; 0 = unlimited        */
} e3d_problem_t;

typedef struct e3d_solve_stats {
  int32_t iterations;  /* Lstep (:1575)                                          */
  int32_t exit_reason; /* E3D_EXIT_*                                             */
  int32_t resets;      /* divergence resets (:1978)                              */
  int32_t refinements; /* MIXED: FP64 residual replacements performed            */
  double gg;           /* final z.g (gg returned by dembx_OpenMP)                */
  double gg0;          /* denominator of the criterion                           */
  double rel_res;      /* sqrt(gg/gg0), the criterion value at exit              */
  double true_rel;     /* |g| / |g0| from the recurrence residual                */
  double ms_setup;     /* block-Jacobi build + initial z, milliseconds           */
  double ms_iter;      /* PCG iterations, milliseconds                           */
} e3d_solve_stats_t;

typedef struct e3d_handle e3d_handle_t;

/* Fills p with the reference's defaults (src/elas3dxtal_pcg.f90:77-148):
 * C11/C12/C44 = 206/133/119 GPa, E1 = nu1 = 0, ezz = 1e-3, tol = 1e-8 (float),
 * ldemb = 10000, flag_m = 1, REF criterion, FP64, divergence reset on. */
void e3d_problem_defaults(e3d_problem_t* p, int32_t nx, int32_t ny, int32_t nz,
                          int32_t nphase);

/* Allocates the device state of one problem (the allocate() block of
 * `program elas3d`, src/elas3dxtal_pcg.f90:242-256).  The neighbour table ib
 * (:326-369) is not stored: kernels compute periodic neighbours. */
int32_t e3d_create(e3d_handle_t** h, const e3d_problem_t* p);
int32_t e3d_destroy(e3d_handle_t* h);

/* Phase map + orientations, as read by ppixel_hdf5 (:2879-2990): pix has ns
 * entries in [1, nphase] (checked as at :2986-2989, on the device after one
 * copy of the map; a pinned pix buffer copies fastest), rodrigues has
 * 3*(nphase-1) entries (ignored when flag_m == 0, may be NULL then).  On
 * E3D_ERR_INPUT the handle holds no phase map until the next upload. */
int32_t e3d_upload(e3d_handle_t* h, const int32_t* pix, const double* rodrigues);

/* e3d_upload with the phase map already in device memory (d_pix: ns int32 on
 * the handle's device, e.g. from e3d_micro_grains_device); rodrigues is on the
 * host.  The range check runs on the device; E3D_ERR_INPUT if it fails. */
int32_t e3d_upload_device(e3d_handle_t* h, const int32_t* d_pix, const double* rodrigues);

/* femat_OpenMP (:555-1104): cmod (rotatestiffnessby, :2470-2637), element
 * stiffness dk, periodic-jump force b and constant C, all on the device. */
int32_t e3d_femat(e3d_handle_t* h);

/* Affine initial guess u = E.x (driver, :423-438). */
int32_t e3d_init_affine(e3d_handle_t* h);

/* energy_OpenMP (:1107-1353): gb = K u + b and utot = C + sum(u.Ku/2 + b.u).
 * Also returns gg = sum(gb^2), which the driver stores as gg0 (:452-453);
 * the handle keeps it as the REF criterion denominator for e3d_solve. */
int32_t e3d_energy(e3d_handle_t* h, double* utot, double* gg);

/* dembx_OpenMP with kkk = 1 (:1356-2043): block-Jacobi build (:1498-1520,
 * invert3x3 :2046-2147), then PCG on u and gb until the criterion, the hAh
 * guard or max_iter.  Returns E3D_OK (converged or hAh guard),
 * E3D_ERR_MAXITER, E3D_ERR_BREAKDOWN or E3D_ERR_TIMEOUT; st may be NULL. */
int32_t e3d_solve(e3d_handle_t* h, e3d_solve_stats_t* st);

/* Split form of e3d_solve for callers that interleave work or time single
 * iterations: e3d_solve_begin does the setup, e3d_iterate runs at most n
 * iterations (exit_reason E3D_EXIT_RUNNING when the budget ran out). */
int32_t e3d_solve_begin(e3d_handle_t* h);
int32_t e3d_iterate(e3d_handle_t* h, int32_t n, e3d_solve_stats_t* st);

/* stress_OpenMP (:2149-2408): volume-averaged stress (Pa) and engineering
 * strain, Voigt xx, yy, zz, xz, yz, xy. */
int32_t e3d_stress(e3d_handle_t* h, double strav[6], double epsav[6]);

/* stress_fullfield_OpenMP compute part (:2723-2833): sigma(ns,6) (SoA) and
 * von Mises vm(ns).  Either pointer may be NULL.  The HDF5 write is left to
 * the caller. */
int32_t e3d_stress_field(e3d_handle_t* h, double* sigma, double* vm);

/* The whole driver flow of `program elas3d` without file I/O (:417-514):
 * femat, affine guess, energy, gg0, dembx, energy, stress.  out6[0..5] =
 * strav, out6[6..11] = epsav; utot[0] initial energy, utot[1] final energy. */
int32_t e3d_run(e3d_handle_t* h, double utot[2], double out12[12], e3d_solve_stats_t* st);

/* Matrix-free y = K x (the stencil of :1585-1883 without b), host buffers of
 * 3*ns doubles.  e3d_apply_device takes device pointers instead. */
int32_t e3d_apply(e3d_handle_t* h, const double* x, double* y);
int32_t e3d_apply_device(e3d_handle_t* h, const double* d_x, double* d_y);

/* State transfer (3*ns doubles each unless noted). */
int32_t e3d_set_u(e3d_handle_t* h, const double* u);
int32_t e3d_get_u(e3d_handle_t* h, double* u);
int32_t e3d_get_g(e3d_handle_t* h, double* g);
int32_t e3d_get_b(e3d_handle_t* h, double* b);
int32_t e3d_get_C(e3d_handle_t* h, double* C);
/* cmod(nphase,6,6) and dk(nphase,8,3,8,3) in the reference's Fortran layout. */
int32_t e3d_get_cmod(e3d_handle_t* h, double* cmod);
int32_t e3d_get_dk(e3d_handle_t* h, double* dk);
/* Block-Jacobi inverses in the reference's M_block_inv(ns,3,3) layout (9*ns). */
int32_t e3d_get_minv(e3d_handle_t* h, double* minv);
/* Per-iteration rel_res history of the last solve (cgitr file, :2019-2021);
 * copies min(n, iterations) values, returns the count through *count. */
int32_t e3d_get_history(e3d_handle_t* h, double* hist, int32_t n, int32_t* count);

/* Checkpoint / resume of a solve in progress.  The reference's only resumable
 * state is e3d%u, gb, h carried across its kkk restart loop
 * (src/elas3dxtal_pcg.f90:470-508, 2024-2031); here the whole PCG state
 * (u, g, z, the search direction, scalars, rel_res history; for the mixed form
 * its FP32 inner state) is written to `path`, so a long solve can stop and
 * continue in another process.  Save needs a started solve (e3d_solve_begin);
 * load needs e3d_upload + e3d_femat with the same problem, rebuilds the
 * preconditioner and continues with e3d_iterate exactly where save stopped. */
int32_t e3d_checkpoint_save(e3d_handle_t* h, const char* path);
int32_t e3d_checkpoint_load(e3d_handle_t* h, const char* path);

/* Device pointers of the state vectors (3*ns doubles each, SoA), for callers
 * that keep inputs resident in HBM. */
int32_t e3d_device_ptrs(e3d_handle_t* h, double** d_u, double** d_g, double** d_b);

/* Bytes of device memory the handle holds. */
int64_t e3d_device_bytes(const e3d_handle_t* h);

/* Number of kernel launches issued by the handle so far. */
int64_t e3d_launch_count(const e3d_handle_t* h);

/* Which inner stencil the solve runs: E3D_PATH_FP64 (plain FP64 form),
 * E3D_PATH_F32 (mixed form, per-thread loads: the default) or
 * E3D_PATH_F32_TMA (mixed form, node planes staged in shared memory by TMA;
 * when the environment sets E3D_TMA=1 as the handle is created and
 * nx % 4 == 0). */
enum { E3D_PATH_FP64 = 0, E3D_PATH_F32 = 1, E3D_PATH_F32_TMA = 2 };
int32_t e3d_stencil_path(const e3d_handle_t* h);

/* No counterpart in the reference.  y = K x, the same matrix-free stencil as
 * e3d_apply_device, for callers that must not allocate device memory: a host
 * framework that owns every device allocation and forbids library-side
 * cudaMalloc (which also synchronises the device), or a serving loop that
 * admits work under a fixed HBM budget.  Nothing is allocated: the caller
 * passes device pointers to its inputs and output --
 *   d_pix  ns int32 phase ids, 1-based, in [1, nphase] (checked),
 *   d_cmod 36*nphase doubles, cmod(nphase,6,6) in the reference layout
 *          (e3d_get_cmod returns it),
 *   d_x, d_y 3*ns doubles (SoA), in separate buffers (overlapping ones are
 *          refused with E3D_ERR_INPUT: y is written while x is still read),
 * and the scaled stiffness table and tile halos live in one static device
 * array of E3D_NOALLOC_SCRATCH_BYTES per GPU, held from library load to
 * process exit.  A grid whose scratch (about 41*3*ns/256 doubles of halos plus
 * 126*(nphase+1) doubles of table -- e.g. 128^3 with up to 8600 phases) does
 * not fit is rejected with E3D_ERR_INPUT and e3d_last_cuda_error() says why.
 * Runs on `stream` (a cudaStream_t, NULL = legacy default) of the current
 * device; each call copies a phase-check flag back to host memory and waits
 * for `stream` before it returns, so y is complete on return.  Every
 * rejection leaves its reason in e3d_last_cuda_error().  The first call on each device looks
 * up the array's device address (make it before any stream capture).  Calls
 * share the array: calls that overlap on the GPU race. */
#define E3D_NOALLOC_SCRATCH_BYTES (16LL * 1024 * 1024)
int32_t e3d_apply_noalloc(int32_t nx, int32_t ny, int32_t nz, int32_t nphase,
                          const int32_t* d_pix, const double* d_cmod,
                          const double* d_x, double* d_y, void* stream);

/* Measured FP64 and FP32 FMA throughput of the device (TFLOP/s, FMA = 2
 * flops), the compute roofline denominators of the stencil. */
int32_t e3d_probe_peaks(int32_t device, double* fp64_tflops, double* fp32_tflops);

/* Test hook (no counterpart in the reference): runs one kernel whose device
 * wait can never be satisfied -- which = 0: a grid barrier whose partner block
 * never arrives; which = 1: an mbarrier phase expecting bytes no copy delivers
 * -- with a wall-clock limit of timeout_s seconds (at most 10).  Returns
 * E3D_ERR_TIMEOUT when the wait ran out and was reported through the error flag
 * (the context stays usable), any other status otherwise. */
int32_t e3d_selftest_timeout(int32_t device, int32_t which, double timeout_s);

/* Bounds-checked debug build (no counterpart in the reference; the library
 * compiled with -DE3D_BOUNDS, build recipe option bounds=True): reads and
 * clears the record of the indices that the checked kernels found outside
 * their buffers since the last call, on the current device.  report = {count,
 * unit, line, index, limit}: the number of such indices (0 in a clean run)
 * and, for the first one, the translation unit (0 solver, 1 batch and serve
 * engine, 2 allocation-free apply), the source line of the check, the index
 * and the buffer's length.  A checked kernel uses element 0 in place of a bad
 * index, so nothing is read or written outside a buffer.  Returns
 * E3D_ERR_STATE (report zeroed) in a library built without the checks. */
int32_t e3d_debug_bounds(int64_t report[5]);

/* Test hook of the checked build: one kernel hands the check an index past
 * the end of its 32-element buffer, which must be counted and redirected to
 * element 0.  Clears the record first.  Returns E3D_OK when e3d_debug_bounds
 * then reports exactly that index, E3D_ERR_STATE in a library built without
 * the checks (no kernel runs there). */
int32_t e3d_selftest_bounds(int32_t device);

const char* e3d_strerror(int32_t status);
/* Text of the last CUDA error seen by any handle in this thread. */
const char* e3d_last_cuda_error(void);

#ifdef __cplusplus
}
#endif
#endif
