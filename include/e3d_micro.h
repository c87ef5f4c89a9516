/*
 * e3d_micro.h -- seeded synthetic microstructures for the voxel-FE solver.
 *
 * The reference builds its inputs with MATLAB + MTEX (src/microstructure_gen.m)
 * and stores them as HDF5 /pix (int32, 1-based phase per voxel) and
 * /orientation (float64, one Rodrigues vector per grain)
 * (src/microstructure_gen.m:866-892).  These host routines write the same two
 * arrays, deterministically from a 64-bit seed, so that every workload can be
 * regenerated on any machine instead of being shipped as a file.
 *
 * Grid convention: nodes == voxels (fully periodic), voxel (i,j,k) has centre
 * (i+0.5, j+0.5, k+0.5) in a box of side (nx, ny, nz) voxels, linear index
 * m = i + nx*(j + ny*k).  Grains are phases 1..ngrains; the pore phase is
 * ngrains+1 (zero stiffness in the solver).
 */
#ifndef E3D_MICRO_H
#define E3D_MICRO_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Periodic Voronoi (laguerre_sigma == 0) or Laguerre/power-Voronoi
 * (laguerre_sigma > 0: grain volumes ~ lognormal(sigma)) tessellation.
 * Seeds are uniform in the box; each voxel centre takes the grain of the
 * nearest seed under the minimum-image distance (power distance for Laguerre);
 * ties go to the lower grain id.  Orientations are uniform on SO(3): an
 * isotropic unit quaternion with q_w >= 0, stored as Rodrigues r = q_xyz/q_w
 * (the reference's convention, src/microstructure_gen.m:774-800).
 * pix: nx*ny*nz int32; rod: 3*ngrains doubles.  Returns 0 on success. */
int32_t e3d_micro_grains(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                         double laguerre_sigma, uint64_t seed, int32_t* pix,
                         double* rod);

/* Adds periodic spherical pores (radius ~ lognormal(log_mu, log_sigma) voxels,
 * uniform centres) until at least target_frac of the voxels carry pore_phase.
 * Returns the number of pores placed (< 0 on error). */
int32_t e3d_micro_spherical_pores(int32_t nx, int32_t ny, int32_t nz,
                                  double target_frac, double log_mu,
                                  double log_sigma, int32_t pore_phase,
                                  uint64_t seed, int32_t* pix);

/* Adds periodic ellipsoidal voids with semi-axes (aspect*a, a, a), a ~
 * lognormal(log_mu, log_sigma) voxels, uniformly random orientation, until at
 * least target_frac of the voxels carry pore_phase.  Returns the count. */
int32_t e3d_micro_ellipsoidal_pores(int32_t nx, int32_t ny, int32_t nz,
                                    double target_frac, double aspect,
                                    double log_mu, double log_sigma,
                                    int32_t pore_phase, uint64_t seed,
                                    int32_t* pix);

/* Raw microstructure container (.e3d), the stand-in for the reference's HDF5
 * input input_structure_poly.h5 (/pix int32 ns, /orientation float64
 * 3*ngrains; ppixel_hdf5, src/elas3dxtal_pcg.f90:2879-2990) where libhdf5 is
 * absent.  Little-endian: 8-byte magic "E3DMICRO", int32 version (1), nx, ny,
 * nz, ngrains, int32 reserved, then pix (ns int32) and rodrigues (3*ngrains
 * float64).  The reader applies the reference's checks: the sizes must match
 * (:2939-2942, :2966-2969) and every phase id must lie in [1, ngrains+1]
 * (:2986-2989).  Return 0 on success, -1 on I/O errors, -2 on a bad file. */
int32_t e3d_micro_write(const char* path, int32_t nx, int32_t ny, int32_t nz,
                        int32_t ngrains, const int32_t* pix, const double* rod);
int32_t e3d_micro_read_header(const char* path, int32_t* nx, int32_t* ny,
                              int32_t* nz, int32_t* ngrains);
int32_t e3d_micro_read(const char* path, int32_t nx, int32_t ny, int32_t nz,
                       int32_t ngrains, int32_t* pix, double* rod);

/* HDF5 files without libhdf5: a minimal reader and writer of the subset the
 * HDF5 library writes by default (version-0/1 superblock, version-1 object
 * headers, symbol-table root group, contiguous or compact datasets; chunked or
 * filtered storage is refused).  Return 0 on success, -1 on I/O errors, -2 on
 * a bad or unsupported file, -3 on a size mismatch, -4 on a phase id out of
 * range; the reason is left in e3d_last_cuda_error (include/e3d_gpu.h).
 *
 * e3d_h5_micro_info: element counts of the datasets "pix" and "orientation"
 * of a microstructure file and the int32 attribute "dimensions" of "pix"
 * (Nx, Ny, Nz, as the reference's MATLAB generator stores it; zeros when
 * absent).  dims may be NULL. */
int32_t e3d_h5_micro_info(const char* path, int64_t* npix, int64_t* norient,
                          int32_t dims[3]);

/* ppixel_hdf5 (src/elas3dxtal_pcg.f90:2879-2990): reads "pix" (ns values,
 * any integer type) and "orientation" (3*ngrains values, any float type) with
 * the reference's checks -- the sizes must match (:2939-2942, :2966-2969)
 * and every phase id must lie in [1, ngrains+1] (:2986-2989). */
int32_t e3d_h5_micro_read(const char* path, int64_t ns, int32_t ngrains,
                          int32_t* pix, double* rod);

/* The input file of the reference's MATLAB generator
 * (src/microstructure_gen.m:876-889): "pix" int32 (1 x ns, with the int32
 * attribute "dimensions" = Nx, Ny, Nz) and "orientation" float64
 * (1 x 3*ngrains, attribute "dimensions" = 3*ngrains, 1). */
int32_t e3d_h5_micro_write(const char* path, int32_t nx, int32_t ny, int32_t nz,
                           int32_t ngrains, const int32_t* pix, const double* rod);

/* fullfield_poly.h5 of stress_fullfield_OpenMP (src/elas3dxtal_pcg.f90:
 * 2840-2874): "pix" int32 (ns), "vm" float64 (ns) and "stress_tensor" float64
 * (6 x ns in the file, i.e. the reference's stress_field(ns,6): component-major,
 * the layout e3d_stress_field returns). */
int32_t e3d_h5_fullfield_write(const char* path, int64_t ns, const int32_t* pix,
                               const double* vm, const double* sigma);

/* Any dataset of the root group by name: its element count, rank and
 * dimensions (HDF5 order, slowest first; dims may be NULL, at most 8 filled),
 * and its values converted to int32 / float64 (n must equal the count; -3 on a
 * mismatch or an integer outside the int32 range). */
int32_t e3d_h5_dataset_size(const char* path, const char* name, int64_t* count,
                            int32_t* rank, int64_t dims[8]);
int32_t e3d_h5_read_i32(const char* path, const char* name, int64_t n, int32_t* out);
int32_t e3d_h5_read_f64(const char* path, const char* name, int64_t n, double* out);

/* GPU versions of the three generators above: the same microstructures, bit
 * for bit, written to device memory.  d_pix: nx*ny*nz int32 on CUDA device
 * `device` (caller-owned; the pore routines read and update it in place);
 * rod: 3*ngrains doubles on the host.  For the grains the host draws the seeds
 * and builds the per-block candidate lists and the GPU does the per-voxel
 * nearest-seed search; the pores are drawn on the host and painted on the GPU
 * in the host's order.  Temporary device buffers are allocated and freed
 * inside; calls are synchronous.  Return values as the host routines, and -3
 * on a CUDA error (text in e3d_last_cuda_error). */
int32_t e3d_micro_grains_device(int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                double laguerre_sigma, uint64_t seed, int32_t device,
                                int32_t* d_pix, double* rod);
int32_t e3d_micro_spherical_pores_device(int32_t nx, int32_t ny, int32_t nz,
                                         double target_frac, double log_mu,
                                         double log_sigma, int32_t pore_phase,
                                         uint64_t seed, int32_t device, int32_t* d_pix);
int32_t e3d_micro_ellipsoidal_pores_device(int32_t nx, int32_t ny, int32_t nz,
                                           double target_frac, double aspect,
                                           double log_mu, double log_sigma,
                                           int32_t pore_phase, uint64_t seed,
                                           int32_t device, int32_t* d_pix);

/* Bunge Euler angles (phi1, Phi, phi2; radians) -> Rodrigues vectors, for
 * callers whose orientation files hold Euler angles.  n orientations. */
void e3d_euler_to_rodrigues(int32_t n, const double* euler, double* rod);

#ifdef __cplusplus
}
#endif
#endif
