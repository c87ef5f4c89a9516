! elas3d_gpu_mod.f90 -- iso_c_binding interface to libe3d_gpu.so (include/e3d_gpu.h)
!
! Lets the reference's Fortran driver (`program elas3d`, src/elas3dxtal_pcg.f90)
! replace femat_OpenMP / energy_OpenMP / dembx_OpenMP / stress_OpenMP /
! stress_fullfield_OpenMP with the GB300 library while keeping its own arrays:
! u(ns,3), pix(ns) and orientation(3*(nphase-1)) are passed as they are.
!
! Build (where a Fortran compiler exists):
!   gfortran -c elas3d_gpu_mod.f90
!   gfortran ... elas3dxtal_pcg.f90 elas3d_gpu_mod.o -L<pkg>/_build -le3d_gpu
      module elas3d_gpu_mod
        use, intrinsic :: iso_c_binding
        implicit none

        integer(c_int32_t), parameter :: E3D_OK = 0
        integer(c_int32_t), parameter :: E3D_ERR_INPUT = 1, E3D_ERR_OOM = 2, E3D_ERR_BREAKDOWN = 3
        integer(c_int32_t), parameter :: E3D_ERR_MAXITER = 4, E3D_ERR_TIMEOUT = 5, E3D_ERR_CUDA = 6
        integer(c_int32_t), parameter :: E3D_ERR_STATE = 7
        integer(c_int32_t), parameter :: E3D_EXIT_CONVERGED = 0, E3D_EXIT_HAH_GUARD = 1
        integer(c_int32_t), parameter :: E3D_EXIT_MAXITER = 2, E3D_EXIT_BREAKDOWN = 3
        integer(c_int32_t), parameter :: E3D_EXIT_TIMEOUT = 4, E3D_EXIT_RUNNING = 5
        integer(c_int32_t), parameter :: E3D_CRIT_REF = 0, E3D_CRIT_PRECOND_REL = 1
        integer(c_int32_t), parameter :: E3D_PRECOND_BLOCK_JACOBI = 0, E3D_PRECOND_NONE = 1
        integer(c_int32_t), parameter :: E3D_PREC_FP64 = 0, E3D_PREC_MIXED = 1

        ! mirrors e3d_problem_t (field order and padding identical)
        type, bind(C) :: e3d_problem_t
          integer(c_int32_t) :: nx, ny, nz, nphase
          integer(c_int32_t) :: flag_m, criterion, precision, divergence_reset
          integer(c_int32_t) :: max_iter, device
          real(c_float)      :: tol
          integer(c_int32_t) :: refine_every
          integer(c_int32_t) :: preconditioner, refine_decades
          real(c_double)     :: c11, c12, c44, e1, nu1
          real(c_double)     :: strain(6)      ! exx eyy ezz exz eyz exy (tensor)
          integer(c_int64_t) :: hbm_budget
        end type

        type, bind(C) :: e3d_solve_stats_t
          integer(c_int32_t) :: iterations, exit_reason, resets, refinements
          real(c_double)     :: gg, gg0, rel_res, true_rel, ms_setup, ms_iter
        end type

        interface
          subroutine e3d_problem_defaults(p, nx, ny, nz, nphase) bind(C, name="e3d_problem_defaults")
            import :: e3d_problem_t, c_int32_t
            type(e3d_problem_t), intent(out) :: p
            integer(c_int32_t), value :: nx, ny, nz, nphase
          end subroutine
          integer(c_int32_t) function e3d_create(h, p) bind(C, name="e3d_create")
            import :: c_ptr, c_int32_t, e3d_problem_t
            type(c_ptr), intent(out) :: h
            type(e3d_problem_t), intent(in) :: p
          end function
          integer(c_int32_t) function e3d_destroy(h) bind(C, name="e3d_destroy")
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
          end function
          integer(c_int32_t) function e3d_upload(h, pix, rod) bind(C, name="e3d_upload")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), intent(in) :: pix(*)
            real(c_double), intent(in) :: rod(*)
          end function
          integer(c_int32_t) function e3d_femat(h) bind(C, name="e3d_femat")
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
          end function
          integer(c_int32_t) function e3d_init_affine(h) bind(C, name="e3d_init_affine")
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
          end function
          integer(c_int32_t) function e3d_solve_begin(h) bind(C, name="e3d_solve_begin")
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
          end function
          integer(c_int32_t) function e3d_iterate(h, n, st) bind(C, name="e3d_iterate")
            import :: c_ptr, c_int32_t, e3d_solve_stats_t
            type(c_ptr), value :: h
            integer(c_int32_t), value :: n
            type(e3d_solve_stats_t), intent(out) :: st
          end function
          integer(c_int32_t) function e3d_run(h, utot, out12, st) bind(C, name="e3d_run")
            import :: c_ptr, c_int32_t, c_double, e3d_solve_stats_t
            type(c_ptr), value :: h
            real(c_double), intent(out) :: utot(2), out12(12)
            type(e3d_solve_stats_t), intent(out) :: st
          end function
          ! path: a C string, e.g. trim(name)//c_null_char
          integer(c_int32_t) function e3d_checkpoint_save(h, path) bind(C, name="e3d_checkpoint_save")
            import :: c_ptr, c_int32_t, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
          end function
          integer(c_int32_t) function e3d_checkpoint_load(h, path) bind(C, name="e3d_checkpoint_load")
            import :: c_ptr, c_int32_t, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
          end function
          type(c_ptr) function e3d_strerror(status) bind(C, name="e3d_strerror")
            import :: c_ptr, c_int32_t
            integer(c_int32_t), value :: status
          end function
          integer(c_int32_t) function e3d_set_u(h, u) bind(C, name="e3d_set_u")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(in) :: u(*)
          end function
          integer(c_int32_t) function e3d_get_u(h, u) bind(C, name="e3d_get_u")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: u(*)
          end function
          integer(c_int32_t) function e3d_energy(h, utot, gg) bind(C, name="e3d_energy")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: utot, gg
          end function
          integer(c_int32_t) function e3d_solve(h, st) bind(C, name="e3d_solve")
            import :: c_ptr, c_int32_t, e3d_solve_stats_t
            type(c_ptr), value :: h
            type(e3d_solve_stats_t), intent(out) :: st
          end function
          integer(c_int32_t) function e3d_stress(h, strav, epsav) bind(C, name="e3d_stress")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: strav(6), epsav(6)
          end function
          integer(c_int32_t) function e3d_stress_field(h, sigma, vm) bind(C, name="e3d_stress_field")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: sigma(*), vm(*)
          end function
          integer(c_int32_t) function e3d_get_history(h, hist, n, cnt) bind(C, name="e3d_get_history")
            import :: c_ptr, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: hist(*)
            integer(c_int32_t), value :: n
            integer(c_int32_t), intent(out) :: cnt
          end function
          ! HDF5 files without libhdf5 (include/e3d_micro.h): ppixel_hdf5 and the
          ! fullfield_poly.h5 writer become two calls, so the Fortran driver
          ! needs no HDF5 library.  Status 0, -1 I/O error, -2 bad or
          ! unsupported file, -3 size mismatch, -4 phase id out of range.
          integer(c_int32_t) function e3d_h5_micro_read(path, ns, ngrains, pix, rod) &
              bind(C, name="e3d_h5_micro_read")
            import :: c_int32_t, c_int64_t, c_double, c_char
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int64_t), value :: ns
            integer(c_int32_t), value :: ngrains
            integer(c_int32_t), intent(out) :: pix(*)
            real(c_double), intent(out) :: rod(*)
          end function
          integer(c_int32_t) function e3d_h5_fullfield_write(path, ns, pix, vm, sigma) &
              bind(C, name="e3d_h5_fullfield_write")
            import :: c_int32_t, c_int64_t, c_double, c_char
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int64_t), value :: ns
            integer(c_int32_t), intent(in) :: pix(*)
            real(c_double), intent(in) :: vm(*), sigma(*)
          end function
        end interface
      end module elas3d_gpu_mod
