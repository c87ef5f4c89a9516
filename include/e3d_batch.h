/*
 * e3d_batch.h -- batched effective-stiffness ensembles and the serving loop.
 *
 * No single counterpart in the reference: its driver solves one RVE under one
 * load case per run (`program elas3d`, src/elas3dxtal_pcg.f90:186-552, with
 * the load in compile-time constants aml_* at :125-131).  These entry points
 * run many such solves -- each the same femat / energy / dembx / stress chain
 * -- concurrently on one GPU:
 *
 *  - e3d_batch_*: many RVEs of uneven size, each under the six unit macro-strain
 *    load cases, in one persistent launch replayed from a CUDA graph; output the
 *    6x6 effective stiffness of each RVE (column j = <sigma> / strain for unit
 *    engineering strain in Voigt slot j, order xx yy zz xz yz xy).
 *  - e3d_serve_*: a continuous-batching server: requests (one RVE, one load
 *    case) are admitted while others run, as slots and HBM budget free up; their
 *    PCG state stays resident between rounds of the persistent engine.
 *
 * Every solve uses the mixed form (FP32 stencil and block-Jacobi inside FP64
 * residual replacement; FP64 energy and stress) and the reference's stopping
 * test unless opts.criterion says otherwise.
 */
#ifndef E3D_BATCH_H
#define E3D_BATCH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct e3d_rve {
  int32_t nx, ny, nz;       /* nodes per direction (fully periodic)              */
  int32_t ngrains;          /* phases 1..ngrains are grains, ngrains+1 the pores */
  double c11, c12, c44;     /* cubic constants of this RVE, Pa                   */
  const int32_t* pix;       /* nx*ny*nz phase ids in [1, ngrains+1]              */
  const double* rodrigues;  /* 3*ngrains Rodrigues vectors                       */
} e3d_rve_t;

typedef struct e3d_batch_opts {
  int32_t device;
  int32_t max_iter;         /* per solve (ldemb)                                 */
  int32_t refine_every;     /* FP64 residual replacement period (0 = 50)         */
  int32_t criterion;        /* E3D_CRIT_* of e3d_gpu.h                           */
  int32_t divergence_reset; /* 1: h = z when rel_res grows > 10x                 */
  float tol;                /* single precision, as the reference's tol          */
  int32_t load_cases;       /* bitmask of the six unit load cases (0 = all six)  */
  int32_t parts;            /* blocks per solve (<= 64): 0 = autotune            */
  int32_t pad;
  double strain;            /* magnitude of the unit load cases (1e-3)           */
  double e1, nu1;           /* inclusion phase modulus / Poisson ratio           */
  int64_t hbm_budget;       /* bytes; 0 = unlimited                              */
} e3d_batch_opts_t;

typedef struct e3d_job_result {
  int32_t rve, load_case;   /* load_case 0..5 (xx yy zz xz yz xy), -1 for served requests */
  int32_t status;           /* E3D_EXIT_* of e3d_gpu.h                           */
  int32_t iterations, refinements, resets;
  int32_t parts;             /* blocks that ran the solve                         */
  int32_t tile_z;            /* element planes per tile (autotuned tile shape)    */
  double utot0, utot;       /* initial / final energy                            */
  double rel_res, true_rel; /* criterion value and |g|/|g0| at exit              */
  double strav[6], epsav[6];
  double seconds;           /* served requests: arrival to completion            */
} e3d_job_result_t;

typedef struct e3d_batch e3d_batch_t;

void e3d_batch_opts_defaults(e3d_batch_opts_t* o);

/* Uploads the RVEs, builds every phase table (femat element part) and
 * block-Jacobi inverse, allocates all solve state (within hbm_budget), picks
 * the blocks per solve and the tile shape (autotuner when opts->parts == 0) and captures the
 * solve into a CUDA graph. */
int32_t e3d_batch_create(e3d_batch_t** b, const e3d_rve_t* rves, int32_t n, const e3d_batch_opts_t* opts);

/* Runs every solve (one graph launch: one persistent kernel).  ceff receives
 * 36 doubles per RVE, row-major C[i][j] in Pa (may be NULL); seconds the
 * device time of the launch (may be NULL). */
int32_t e3d_batch_solve(e3d_batch_t* b, double* ceff, double* seconds);

/* Per-solve results of the last e3d_batch_solve (n*popcount(load_cases)). */
int32_t e3d_batch_results(e3d_batch_t* b, e3d_job_result_t* out, int32_t capacity, int32_t* count);

/* Blocks per solve chosen for each solve (same order as the results). */
int32_t e3d_batch_parts(e3d_batch_t* b, int32_t* parts, int32_t capacity);

int32_t e3d_batch_destroy(e3d_batch_t* b);

/* ---- serving ----------------------------------------------------------- */
typedef struct e3d_server e3d_server_t;

typedef struct e3d_serve_opts {
  int32_t device;
  int32_t max_iter, refine_every, criterion, divergence_reset;
  float tol;
  int32_t max_active;       /* concurrent solves on the device (slots)           */
  int32_t round_iters;      /* PCG iterations per solve per engine round          */
  int32_t parts;            /* blocks per solve (<= 64): 0 = by size              */
  int32_t round_balance;    /* 1: a solve with fewer nodes per block runs up to
                               8x round_iters per round (same results, fewer
                               rounds); 0 (default): round_iters for every solve */
  double e1, nu1;
  int64_t hbm_budget;       /* bytes of device memory the server may hold        */
} e3d_serve_opts_t;

void e3d_serve_opts_defaults(e3d_serve_opts_t* o);
int32_t e3d_serve_create(e3d_server_t** s, const e3d_serve_opts_t* opts);

/* Queues one request: an RVE under a macro strain (tensor exx eyy ezz exz eyz
 * exy).  Inputs are copied; returns the request id through *id.  Phase ids
 * outside [1, ngrains + 1] are refused with E3D_ERR_INPUT, and a request larger
 * than the HBM budget with E3D_ERR_OOM. */
int32_t e3d_serve_submit(e3d_server_t* s, const e3d_rve_t* rve, const double strain[6], int64_t* id);

/* One scheduling round: admits queued requests while slots and HBM allow,
 * advances every active solve by round_iters iterations in one engine launch,
 * and retires finished solves (their memory is freed for the next admission).
 * Returns the number of requests still queued or active through *pending. */
int32_t e3d_serve_step(e3d_server_t* s, int32_t* pending);

/* Result of a finished request (E3D_ERR_STATE while it is not finished). */
int32_t e3d_serve_result(e3d_server_t* s, int64_t id, e3d_job_result_t* out);

/* Cancels a request between rounds: a queued request leaves the queue, an
 * active one gives its slot and device memory back before the next round.  Its
 * result then has status E3D_EXIT_CANCELLED (iterations done so far).
 * E3D_ERR_STATE if the request already finished, E3D_ERR_INPUT for an unknown
 * id. */
#define E3D_EXIT_CANCELLED 6
int32_t e3d_serve_cancel(e3d_server_t* s, int64_t id);

/* Bytes of device memory held now / at most so far. */
int32_t e3d_serve_memory(e3d_server_t* s, int64_t* now, int64_t* peak);

int32_t e3d_serve_destroy(e3d_server_t* s);

#ifdef __cplusplus
}
#endif
#endif
