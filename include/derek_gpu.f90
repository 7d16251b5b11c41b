! Fortran 2003 iso_c_binding interface to libderek_gpu (include/derek_gpu.h).
!
! A DEReK maintainer compiles this module ahead of Source/electronic.f90 and
! links with -L<repo>/derek_gb300 -lderek_gpu -lcudart.  The calls replace
! the reference's stubs: electronic_scf (Source/electronic.f90:86),
! pot_apply_wfn (Source/pot.f90:344), density_calculate
! (Source/density.f90:101) and the wave_dot_* family (Source/wave.f90:929).
!
! Conventions:
! * every entry point returns an integer(c_int) status, 0 on success
!   (DEREK_OK); derek_gpu_strerror / derek_gpu_last_error give the text as a
!   C string (type(c_ptr));
! * the handle is a type(c_ptr) passed by value;
! * complex arrays are complex(c_double_complex), the C side's interleaved
!   (re, im) doubles;
! * arguments C accepts as NULL are type(c_ptr), value: pass c_loc(x) or
!   c_null_ptr;
! * strings are NUL-terminated: path = "run.den" // c_null_char.
! Derived types mirror the C structs member for member.
module derek_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: DEREK_OK = 0, DEREK_ERR_BAD_ARG = 1, DEREK_ERR_OOM = 2, &
       DEREK_ERR_CUDA = 3, DEREK_ERR_NOT_CONVERGED = 4, DEREK_ERR_CHOLESKY = 5, &
       DEREK_ERR_NAN = 6, DEREK_ERR_TIMEOUT = 7, DEREK_ERR_UNSUPPORTED = 8
  integer(c_int), parameter :: DEREK_PREC_FP64 = 0, DEREK_PREC_MIXED = 1
  integer(c_int), parameter :: DEREK_GRID_REFERENCE = 0, DEREK_GRID_SMOOTH23 = 1
  integer(c_int), parameter :: DEREK_TUNE_RETUNE = 1

  type, bind(C) :: derek_sys_desc
     real(c_double)    :: cell(9), inv_cell(9), ecut, g_fine_scale
     integer(c_int)    :: n_fine(3), grid_policy, nk
     type(c_ptr)       :: kpts, wk
     integer(c_int)    :: nbands, nspinor
     real(c_double)    :: nelec, kT
     type(c_ptr)       :: vext
     integer(c_int)    :: nwells
     type(c_ptr)       :: wells
  end type derek_sys_desc

  type, bind(C) :: derek_scf_opts
     integer(c_int)     :: precision
     real(c_double)     :: mix_alpha, kerker_q0
     integer(c_int)     :: pulay_history, cheb_degree, first_passes, first_degree
     integer(c_int64_t) :: seed
     integer(c_int)     :: use_graph, use_tensor_cores
     real(c_double)     :: density_tol
     integer(c_int)     :: buffer_bands, etol_per_electron, init_vectors
  end type derek_scf_opts

  type, bind(C) :: derek_scf_report
     real(c_double) :: energy, free_energy, delta, efermi, entropy
     real(c_double) :: e_band, e_hartree, e_xc, e_dc, residual
     integer(c_int) :: iterations, converged
  end type derek_scf_report

  type, bind(C) :: derek_info
     integer(c_int)         :: check, debugging, n_electrons, max_scf, conduction_bands, nbands, &
                               iprint, random_seed
     integer(c_int)         :: write_wvfn, soc, write_density, write_potential, write_state, &
                               write_spec, write_memory, write_formatted_potential, write_potex, &
                               write_formatted_density, restart, write_formatted_potex, write_xsf
     integer(c_int)         :: kpt_mp_grid(3), periodic_pot_grid(3), dos_kpt_mp_grid(3)
     real(c_double)         :: energy_tol, cut_off_energy, g_fine_scale
     real(c_double)         :: electronic_temp
     real(c_double)         :: finite_barrier_height, finite_barrier_width(3), periodic_pot_amp
     real(c_double)         :: ext_efield(3), ext_bfield(3)
     character(kind=c_char) :: xc_functional(32), task(32), scf_method(32), external_pot(32), &
                               output_level(32), unit_energy(32), unit_length(32), unit_efield(32), &
                               unit_bfield(32), out_energy_unit(32), out_len_unit(32), &
                               out_efield_unit(32), out_bfield_unit(32)
     real(c_double)         :: cell(9)
     integer(c_int)         :: n_pots
     real(c_double)         :: pot_centres(192), pot_heights(64), pot_widths(64)
     integer(c_int)         :: n_corrected
  end type derek_info

  interface
     ! ---- handle
     subroutine derek_gpu_default_opts(opts) bind(C, name="derek_gpu_default_opts")
       import :: derek_scf_opts
       type(derek_scf_opts), intent(out) :: opts
     end subroutine
     type(c_ptr) function derek_gpu_strerror(status) bind(C, name="derek_gpu_strerror")
       import :: c_ptr, c_int
       integer(c_int), value :: status
     end function
     type(c_ptr) function derek_gpu_last_error(h) bind(C, name="derek_gpu_last_error")
       import :: c_ptr
       type(c_ptr), value :: h
     end function
     integer(c_int) function derek_gpu_create(h, sys, nsys, opts) bind(C, name="derek_gpu_create")
       import :: c_ptr, c_int, derek_sys_desc, derek_scf_opts
       type(c_ptr), intent(out)         :: h
       type(derek_sys_desc), intent(in) :: sys(*)
       integer(c_int), value            :: nsys
       type(derek_scf_opts), intent(in) :: opts
     end function
     integer(c_int) function derek_gpu_destroy(h) bind(C, name="derek_gpu_destroy")
       import :: c_ptr, c_int
       type(c_ptr), value :: h
     end function

     ! ---- sizes and tables
     integer(c_int) function derek_gpu_grid(h, sys, n_fine, n_std) bind(C, name="derek_gpu_grid")
       import :: c_ptr, c_int
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       integer(c_int), intent(out) :: n_fine(3), n_std(3)
     end function
     integer(c_int) function derek_gpu_bands(h, sys, nbands, nbands_internal) bind(C, name="derek_gpu_bands")
       import :: c_ptr, c_int
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       integer(c_int), intent(out) :: nbands, nbands_internal
     end function
     integer(c_int) function derek_gpu_npw(h, sys, k, npw) bind(C, name="derek_gpu_npw")
       import :: c_ptr, c_int
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys, k
       integer(c_int), intent(out) :: npw
     end function
     ! box_rows (0-based rows of the standard box), fft_index, kinetic: each
     ! npw long, or c_null_ptr
     integer(c_int) function derek_gpu_gsphere(h, sys, k, box_rows, fft_index, kinetic) &
          bind(C, name="derek_gpu_gsphere")
       import :: c_ptr, c_int
       type(c_ptr), value    :: h
       integer(c_int), value :: sys, k
       type(c_ptr), value    :: box_rows, fft_index, kinetic
     end function

     ! ---- FFT, potentials, wavefunctions, H.psi, density, overlaps
     integer(c_int) function derek_gpu_fft3d(h, sys, inout, dir) bind(C, name="derek_gpu_fft3d")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                       :: h
       integer(c_int), value                    :: sys
       complex(c_double_complex), intent(inout) :: inout(*)
       integer(c_int), value                    :: dir
     end function
     integer(c_int) function derek_gpu_set_vloc(h, sys, vloc) bind(C, name="derek_gpu_set_vloc")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value         :: h
       integer(c_int), value      :: sys
       real(c_double), intent(in) :: vloc(*)
     end function
     integer(c_int) function derek_gpu_get_vloc(h, sys, vloc) bind(C, name="derek_gpu_get_vloc")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: vloc(*)
     end function
     integer(c_int) function derek_gpu_set_wfn(h, sys, k, psi) bind(C, name="derek_gpu_set_wfn")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                    :: h
       integer(c_int), value                 :: sys, k
       complex(c_double_complex), intent(in) :: psi(*)
     end function
     integer(c_int) function derek_gpu_get_wfn(h, sys, k, psi) bind(C, name="derek_gpu_get_wfn")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                     :: h
       integer(c_int), value                  :: sys, k
       complex(c_double_complex), intent(out) :: psi(*)
     end function
     integer(c_int) function derek_gpu_apply_h(h, sys, k, hpsi) bind(C, name="derek_gpu_apply_h")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                     :: h
       integer(c_int), value                  :: sys, k
       complex(c_double_complex), intent(out) :: hpsi(*)
     end function
     integer(c_int) function derek_gpu_density(h, sys, occ, rho) bind(C, name="derek_gpu_density")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(in)  :: occ(*)
       real(c_double), intent(out) :: rho(*)
     end function
     integer(c_int) function derek_gpu_set_nc_pot(h, sys, nc_pot) bind(C, name="derek_gpu_set_nc_pot")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                    :: h
       integer(c_int), value                 :: sys
       complex(c_double_complex), intent(in) :: nc_pot(*)
     end function
     integer(c_int) function derek_gpu_get_nc_pot(h, sys, nc_pot) bind(C, name="derek_gpu_get_nc_pot")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                     :: h
       integer(c_int), value                  :: sys
       complex(c_double_complex), intent(out) :: nc_pot(*)
     end function
     integer(c_int) function derek_gpu_get_nc_ext(h, sys, nc_pot) bind(C, name="derek_gpu_get_nc_ext")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                     :: h
       integer(c_int), value                  :: sys
       complex(c_double_complex), intent(out) :: nc_pot(*)
     end function
     ! rho (nr) and mag (3 nr) may each be c_null_ptr
     integer(c_int) function derek_gpu_density_spinor(h, sys, occ, rho, mag) bind(C, name="derek_gpu_density_spinor")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value         :: h
       integer(c_int), value      :: sys
       real(c_double), intent(in) :: occ(*)
       type(c_ptr), value         :: rho, mag
     end function
     integer(c_int) function derek_gpu_get_magnetisation(h, sys, mag) bind(C, name="derek_gpu_get_magnetisation")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: mag(*)
     end function
     ! mag: 3 nr values, or c_null_ptr for a zero start
     integer(c_int) function derek_gpu_set_start_magnetisation(h, sys, mag) &
          bind(C, name="derek_gpu_set_start_magnetisation")
       import :: c_ptr, c_int
       type(c_ptr), value    :: h
       integer(c_int), value :: sys
       type(c_ptr), value    :: mag
     end function
     integer(c_int) function derek_gpu_xc_lsda(h, n, rho_up, rho_down, exc, v_up, v_down) &
          bind(C, name="derek_gpu_xc_lsda")
       import :: c_ptr, c_long, c_double
       type(c_ptr), value          :: h
       integer(c_long), value      :: n
       real(c_double), intent(in)  :: rho_up(*), rho_down(*)
       real(c_double), intent(out) :: exc(*), v_up(*), v_down(*)
     end function
     integer(c_int) function derek_gpu_xc_lda(h, n, rho, exc, vxc) bind(C, name="derek_gpu_xc_lda")
       import :: c_ptr, c_long, c_double
       type(c_ptr), value          :: h
       integer(c_long), value      :: n
       real(c_double), intent(in)  :: rho(*)
       real(c_double), intent(out) :: exc(*), vxc(*)
     end function
     integer(c_int) function derek_gpu_overlap(h, sys, k, s) bind(C, name="derek_gpu_overlap")
       import :: c_ptr, c_int, c_double_complex
       type(c_ptr), value                     :: h
       integer(c_int), value                  :: sys, k
       complex(c_double_complex), intent(out) :: s(*)
     end function
     ! device pointers and a cudaStream_t (c_null_ptr: the default stream)
     integer(c_int) function derek_gpu_overlap_noalloc(x, y, nb, npw, ld, precision, s, stream) &
          bind(C, name="derek_gpu_overlap_noalloc")
       import :: c_ptr, c_int, c_long
       type(c_ptr), value     :: x, y
       integer(c_int), value  :: nb, npw
       integer(c_long), value :: ld
       integer(c_int), value  :: precision
       type(c_ptr), value     :: s, stream
     end function

     ! ---- SCF and the frozen-potential solver
     integer(c_int) function derek_gpu_scf_iterate(h, rep) bind(C, name="derek_gpu_scf_iterate")
       import :: c_ptr, c_int, derek_scf_report
       type(c_ptr), value                  :: h
       type(derek_scf_report), intent(out) :: rep(*)
     end function
     integer(c_int) function derek_gpu_scf_run(h, max_scf, etol, rep) bind(C, name="derek_gpu_scf_run")
       import :: c_ptr, c_int, c_double, derek_scf_report
       type(c_ptr), value                  :: h
       integer(c_int), value               :: max_scf
       real(c_double), value               :: etol
       type(derek_scf_report), intent(out) :: rep(*)
     end function
     integer(c_int) function derek_gpu_set_vext(h, sys, vext) bind(C, name="derek_gpu_set_vext")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value         :: h
       integer(c_int), value      :: sys
       real(c_double), intent(in) :: vext(*)
     end function
     integer(c_int) function derek_gpu_get_vext(h, sys, vext) bind(C, name="derek_gpu_get_vext")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: vext(*)
     end function
     type(c_ptr) function derek_gpu_stream(h) bind(C, name="derek_gpu_stream")
       import :: c_ptr
       type(c_ptr), value :: h
     end function
     integer(c_long_long) function derek_gpu_launch_count() bind(C, name="derek_gpu_launch_count")
       import :: c_long_long
     end function
     integer(c_int) function derek_gpu_time_apply_h(h, nrep, ms_apply, ms_stage) bind(C, name="derek_gpu_time_apply_h")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: nrep
       real(c_double), intent(out) :: ms_apply, ms_stage(3)
     end function
     integer(c_int) function derek_gpu_autotune(h, cache_path, flags) bind(C, name="derek_gpu_autotune")
       import :: c_ptr, c_int, c_char
       type(c_ptr), value                 :: h
       character(kind=c_char), intent(in) :: cache_path(*)
       integer(c_int), value              :: flags
     end function
     integer(c_int) function derek_gpu_plan(h, buf, len) bind(C, name="derek_gpu_plan")
       import :: c_ptr, c_int, c_char
       type(c_ptr), value                  :: h
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_int), value               :: len
     end function
     integer(c_int) function derek_host_tune_cache_normalise(text, out, len) &
         bind(C, name="derek_host_tune_cache_normalise")
       import :: c_int, c_char
       character(kind=c_char), intent(in)  :: text(*)
       character(kind=c_char), intent(out) :: out(*)
       integer(c_int), value               :: len
     end function
     integer(c_int) function derek_host_radix_candidates(n, out, len) bind(C, name="derek_host_radix_candidates")
       import :: c_int, c_char
       integer(c_int), value               :: n
       character(kind=c_char), intent(out) :: out(*)
       integer(c_int), value               :: len
     end function
     integer(c_int) function derek_gpu_set_wait_limit(iterations) bind(C, name="derek_gpu_set_wait_limit")
       import :: c_int, c_long
       integer(c_long), value :: iterations
     end function
     integer(c_int) function derek_gpu_grad_wells(h, sys, grad) bind(C, name="derek_gpu_grad_wells")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: grad(*)
     end function
     integer(c_int) function derek_gpu_grad_density_loss(h, sys, n_target, loss, grad, max_iter, tol) &
          bind(C, name="derek_gpu_grad_density_loss")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(in)  :: n_target(*)
       real(c_double), intent(out) :: loss, grad(*)
       integer(c_int), value       :: max_iter
       real(c_double), value       :: tol
     end function
     integer(c_int) function derek_gpu_get_eigenvalues(h, sys, eig) bind(C, name="derek_gpu_get_eigenvalues")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: eig(*)
     end function
     integer(c_int) function derek_gpu_get_occupations(h, sys, occ) bind(C, name="derek_gpu_get_occupations")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: occ(*)
     end function
     integer(c_int) function derek_gpu_get_density(h, sys, rho) bind(C, name="derek_gpu_get_density")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value          :: h
       integer(c_int), value       :: sys
       real(c_double), intent(out) :: rho(*)
     end function
     ! iterations: an integer(c_int) target, or c_null_ptr
     integer(c_int) function derek_gpu_nscf_run(h, max_iter, eig_tol, nconv, iterations) bind(C, name="derek_gpu_nscf_run")
       import :: c_ptr, c_int, c_double
       type(c_ptr), value    :: h
       integer(c_int), value :: max_iter
       real(c_double), value :: eig_tol
       integer(c_int), value :: nconv
       type(c_ptr), value    :: iterations
     end function
     ! rho: nr values, or c_null_ptr for the uniform start
     integer(c_int) function derek_gpu_set_start_density(h, sys, rho) bind(C, name="derek_gpu_set_start_density")
       import :: c_ptr, c_int
       type(c_ptr), value    :: h
       integer(c_int), value :: sys
       type(c_ptr), value    :: rho
     end function

     ! ---- the reference's files
     integer(c_int) function derek_io_write_den(path, n_std, nr, charge, spin) bind(C, name="derek_io_write_den")
       import :: c_char, c_int, c_long_long, c_double_complex, c_ptr
       character(kind=c_char), intent(in)    :: path(*)
       integer(c_int), intent(in)            :: n_std(3)
       integer(c_long_long), value           :: nr
       complex(c_double_complex), intent(in) :: charge(*)
       type(c_ptr), value                    :: spin
     end function
     integer(c_int) function derek_io_read_den(path, n_std, nr, charge, spin) bind(C, name="derek_io_read_den")
       import :: c_char, c_int, c_long_long, c_double_complex
       character(kind=c_char), intent(in)     :: path(*)
       integer(c_int), intent(in)             :: n_std(3)
       integer(c_long_long), value            :: nr
       complex(c_double_complex), intent(out) :: charge(*), spin(*)
     end function
     integer(c_int) function derek_io_write_pot(path, n_std, nr, nc_pot) bind(C, name="derek_io_write_pot")
       import :: c_char, c_int, c_long_long, c_double_complex
       character(kind=c_char), intent(in)    :: path(*)
       integer(c_int), intent(in)            :: n_std(3)
       integer(c_long_long), value           :: nr
       complex(c_double_complex), intent(in) :: nc_pot(*)
     end function
     integer(c_int) function derek_io_read_pot(path, n_std, nr, nc_pot) bind(C, name="derek_io_read_pot")
       import :: c_char, c_int, c_long_long, c_double_complex
       character(kind=c_char), intent(in)     :: path(*)
       integer(c_int), intent(in)             :: n_std(3)
       integer(c_long_long), value            :: nr
       complex(c_double_complex), intent(out) :: nc_pot(*)
     end function
     integer(c_int) function derek_io_write_wvfn(path, n_std, nbox, nk, nb, nspinor, coeff) &
          bind(C, name="derek_io_write_wvfn")
       import :: c_char, c_int, c_long_long, c_double_complex
       character(kind=c_char), intent(in)    :: path(*)
       integer(c_int), intent(in)            :: n_std(3)
       integer(c_long_long), value           :: nbox
       integer(c_int), value                 :: nk, nb, nspinor
       complex(c_double_complex), intent(in) :: coeff(*)
     end function
     integer(c_int) function derek_io_read_wvfn(path, n_std, nbox, nk, nb, nspinor, coeff) &
          bind(C, name="derek_io_read_wvfn")
       import :: c_char, c_int, c_long_long, c_double_complex
       character(kind=c_char), intent(in)     :: path(*)
       integer(c_int), intent(in)             :: n_std(3)
       integer(c_long_long), value            :: nbox
       integer(c_int), value                  :: nk, nb, nspinor
       complex(c_double_complex), intent(out) :: coeff(*)
     end function
     integer(c_int) function derek_io_write_xsf(path, cell, n_fine, data) bind(C, name="derek_io_write_xsf")
       import :: c_char, c_int, c_double
       character(kind=c_char), intent(in) :: path(*)
       real(c_double), intent(in)         :: cell(9)
       integer(c_int), intent(in)         :: n_fine(3)
       real(c_double), intent(in)         :: data(*)
     end function
     integer(c_int) function derek_io_write_fden(path, n_fine, charge, spin) bind(C, name="derek_io_write_fden")
       import :: c_char, c_int, c_double, c_ptr
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int), intent(in)         :: n_fine(3)
       real(c_double), intent(in)         :: charge(*)
       type(c_ptr), value                 :: spin
     end function
     integer(c_int) function derek_io_write_fpot(path, n_fine, nc_pot) bind(C, name="derek_io_write_fpot")
       import :: c_char, c_int, c_double_complex
       character(kind=c_char), intent(in)    :: path(*)
       integer(c_int), intent(in)            :: n_fine(3)
       complex(c_double_complex), intent(in) :: nc_pot(*)
     end function
     integer(c_int) function derek_io_set_subrecord_limit(bytes) bind(C, name="derek_io_set_subrecord_limit")
       import :: c_int, c_long_long
       integer(c_long_long), value :: bytes
     end function
     integer(c_int) function derek_info_read(path, params, message, message_len) bind(C, name="derek_info_read")
       import :: c_char, c_int, derek_info
       character(kind=c_char), intent(in)  :: path(*)
       type(derek_info), intent(out)       :: params
       character(kind=c_char), intent(out) :: message(*)
       integer(c_int), value               :: message_len
     end function

     ! ---- host-only helpers
     integer(c_int) function derek_host_prime_fact(n) bind(C, name="derek_host_prime_fact")
       import :: c_int
       integer(c_int), value :: n
     end function
     integer(c_int) function derek_host_grid_sizes(cell, ecut, g_fine_scale, grid_policy, n_std, n_fine) &
          bind(C, name="derek_host_grid_sizes")
       import :: c_int, c_double
       real(c_double), intent(in)  :: cell(9)
       real(c_double), value       :: ecut, g_fine_scale
       integer(c_int), value       :: grid_policy
       integer(c_int), intent(out) :: n_std(3), n_fine(3)
     end function
     integer(c_int) function derek_host_gsphere(inv_cell, ecut, kfrac, n_std, capacity, box_rows, npw) &
          bind(C, name="derek_host_gsphere")
       import :: c_int, c_int32_t, c_double
       real(c_double), intent(in)       :: inv_cell(9)
       real(c_double), value            :: ecut
       real(c_double), intent(in)       :: kfrac(3)
       integer(c_int), intent(in)       :: n_std(3)
       integer(c_int), value            :: capacity
       integer(c_int32_t), intent(out)  :: box_rows(*)
       integer(c_int), intent(out)      :: npw
     end function
  end interface
end module derek_gpu
