! ISO_C_BINDING interface to libmld_gpu (include/mld_gpu.h) for the MILADY Fortran host.
!
! A MILADY build links this module and libmld_gpu.so in place of the reference's own
! descriptor, row-fill, solve and prediction routines.  Arrays keep the reference's
! column-major shapes (pos_cart(3,nat), cell(3,3), force(3,nat), stress(6), energy(dim,nat),
! Amat(D,M)) and are passed with c_loc, so no copies are made on the host side.
module mld_gpu_mod
  use iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: MLD_OK = 0
  integer(c_int), parameter, public :: MLD_PRECISION_PLAIN_FP64 = 0
  integer(c_int), parameter, public :: MLD_PRECISION_MIXED = 1
  integer, parameter, public :: MLD_MAX_ELEMENTS = 8

  type, bind(C), public :: mld_gpu_config
    integer(c_int) :: descriptor_type
    real(c_double) :: j_max
    real(c_double) :: r_cut
    real(c_double) :: inv_r0_input
    integer(c_int) :: weighted
    integer(c_int) :: weighted_3ch
    integer(c_int) :: n_elements
    real(c_double) :: weight_per_element(MLD_MAX_ELEMENTS)
    real(c_double) :: weight_per_element_3ch(MLD_MAX_ELEMENTS)
    real(c_double) :: r_cut_pair_in(MLD_MAX_ELEMENTS * MLD_MAX_ELEMENTS)
    real(c_double) :: r_cut_width_in
    integer(c_int) :: desc_forces
    integer(c_int) :: ml_type
    integer(c_int) :: mld_order
    real(c_double) :: lambda_krr
    real(c_double) :: svd_rcond
    real(c_double) :: sign_stress
    real(c_double) :: sign_stress_big_box
    integer(c_int) :: imm_neigh
    integer(c_int) :: precision
    integer(c_int) :: kernel_type
    real(c_double) :: kernel_power
    real(c_double) :: length_kernel
    real(c_double) :: sigma_kernel
  end type mld_gpu_config

  public :: mld_gpu_config_defaults, mld_gpu_create, mld_gpu_destroy, mld_gpu_dims, &
            mld_gpu_set_structures, mld_gpu_set_labels, mld_gpu_descriptors, mld_gpu_num_rows, &
            mld_gpu_design_matrix, mld_gpu_gram, mld_gpu_solve, mld_gpu_fit, mld_gpu_predict, mld_gpu_evaluate, &
            mld_gpu_set_kernel_points, mld_gpu_solve_info, mld_gpu_gram_rows, &
            mld_gpu_server_create, mld_gpu_server_destroy, mld_gpu_server_submit, &
            mld_gpu_server_progress, mld_gpu_server_result, mld_gpu_server_wait, mld_gpu_server_stats, &
            mld_gpu_server_admission, &
            mld_gpu_descriptor_derivatives, mld_gpu_last_error, mld_gpu_server_last_error, &
            mld_gpu_set_profiling, mld_gpu_profile, mld_gpu_timer_start, mld_gpu_timer_stop, &
            mld_gpu_work_counts, mld_gpu_peak_flops, mld_gpu_descriptors_noalloc, mld_gpu_test_pipeline_timeout, mld_gpu_tuning, &
            mld_gpu_synchronize

  interface
    subroutine mld_gpu_config_defaults(cfg) bind(C, name="mld_gpu_config_defaults")
      import :: mld_gpu_config
      type(mld_gpu_config), intent(out) :: cfg
    end subroutine

    integer(c_int) function mld_gpu_create(cfg, h) bind(C, name="mld_gpu_create")
      import :: c_int, c_ptr, mld_gpu_config
      type(mld_gpu_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function

    subroutine mld_gpu_destroy(h) bind(C, name="mld_gpu_destroy")
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine

    integer(c_int) function mld_gpu_dims(h, k, dim_desc, dim_design_line) bind(C, name="mld_gpu_dims")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: k, dim_desc, dim_design_line
    end function

    integer(c_int) function mld_gpu_set_structures(h, nstruct, nat, pos, cell, types) &
        bind(C, name="mld_gpu_set_structures")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nstruct
      type(c_ptr), value :: nat, pos, cell, types
    end function

    integer(c_int) function mld_gpu_set_labels(h, energy, force, stress, has_efs, w_efs) &
        bind(C, name="mld_gpu_set_labels")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, energy, force, stress, has_efs, w_efs
    end function

    integer(c_int) function mld_gpu_descriptors(h, b_out, n_neigh_out) bind(C, name="mld_gpu_descriptors")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, b_out, n_neigh_out
    end function

    integer(c_int) function mld_gpu_num_rows(h, m) bind(C, name="mld_gpu_num_rows")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), intent(out) :: m
    end function

    integer(c_int) function mld_gpu_design_matrix(h, a, y, w) bind(C, name="mld_gpu_design_matrix")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, a, y, w
    end function

    integer(c_int) function mld_gpu_gram(h, g, rhs) bind(C, name="mld_gpu_gram")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, g, rhs
    end function

    integer(c_int) function mld_gpu_solve(h, g, rhs, d, w, rank) bind(C, name="mld_gpu_solve")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, g, rhs, w, rank
      integer(c_int), value :: d
    end function

    integer(c_int) function mld_gpu_fit(h, w_params, rmse_efs) bind(C, name="mld_gpu_fit")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, w_params, rmse_efs
    end function

    integer(c_int) function mld_gpu_predict(h, w_params, e, f, s) bind(C, name="mld_gpu_predict")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, w_params, e, f, s
    end function

    integer(c_int) function mld_gpu_evaluate(h, w_params, e, f, s) bind(C, name="mld_gpu_evaluate")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, w_params, e, f, s
    end function

    integer(c_int) function mld_gpu_set_kernel_points(h, nk, z_raw) bind(C, name="mld_gpu_set_kernel_points")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, z_raw
      integer(c_int), value :: nk
    end function

    integer(c_int) function mld_gpu_synchronize(h) bind(C, name="mld_gpu_synchronize")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function mld_gpu_solve_info(h, pcg_iterations, pcg_residual, precond_shift, chol_retries) &
        bind(C, name="mld_gpu_solve_info")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, pcg_iterations, pcg_residual, precond_shift, chol_retries
    end function

    integer(c_int) function mld_gpu_gram_rows(method, x, x_is_fp32, m, d, ldx, w, y, g, rhs, stream, err, err_len) &
        bind(C, name="mld_gpu_gram_rows")
      import :: c_int, c_long_long, c_ptr
      integer(c_int), value :: method, x_is_fp32, d, ldx, err_len
      integer(c_long_long), value :: m
      type(c_ptr), value :: x, w, y, g, rhs, stream, err
    end function

    ! returns a NUL-terminated C string owned by the handle (c_f_pointer to read it)
    type(c_ptr) function mld_gpu_last_error(h) bind(C, name="mld_gpu_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function

    type(c_ptr) function mld_gpu_server_last_error(srv) bind(C, name="mld_gpu_server_last_error")
      import :: c_ptr
      type(c_ptr), value :: srv
    end function

    integer(c_int) function mld_gpu_descriptor_derivatives(h, p_inout, nbr_out, u_out, db_out) &
        bind(C, name="mld_gpu_descriptor_derivatives")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h, nbr_out, u_out, db_out
      integer(c_long_long), intent(inout) :: p_inout
    end function

    integer(c_int) function mld_gpu_set_profiling(h, on) bind(C, name="mld_gpu_set_profiling")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: on
    end function

    integer(c_int) function mld_gpu_profile(h, ms, launches, calls, reset) bind(C, name="mld_gpu_profile")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, ms, launches, calls
      integer(c_int), value :: reset
    end function

    integer(c_int) function mld_gpu_timer_start(h) bind(C, name="mld_gpu_timer_start")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function mld_gpu_timer_stop(h, ms) bind(C, name="mld_gpu_timer_stop")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: ms
    end function

    integer(c_int) function mld_gpu_work_counts(h, counts) bind(C, name="mld_gpu_work_counts")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, counts
    end function

    integer(c_int) function mld_gpu_peak_flops(h, precision, tflops) bind(C, name="mld_gpu_peak_flops")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: precision
      real(c_double), intent(out) :: tflops
    end function

    integer(c_int) function mld_gpu_descriptors_noalloc(cfg, nat, pos, cell, types, b, stream, err, err_len) &
        bind(C, name="mld_gpu_descriptors_noalloc")
      import :: c_int, c_ptr, mld_gpu_config
      type(mld_gpu_config), intent(in) :: cfg
      integer(c_int), value :: nat, err_len
      type(c_ptr), value :: pos, cell, types, b, stream, err
    end function

    ! serving loop: one server per GPU, continuous batching over n_slots evaluation slots
    integer(c_int) function mld_gpu_server_create(cfg, w_params, n_slots, max_batch_atoms, hbm_fraction, srv) &
        bind(C, name="mld_gpu_server_create")
      import :: c_int, c_long_long, c_double, c_ptr, mld_gpu_config
      type(mld_gpu_config), intent(in) :: cfg
      type(c_ptr), value :: w_params
      integer(c_int), value :: n_slots
      integer(c_long_long), value :: max_batch_atoms
      real(c_double), value :: hbm_fraction
      type(c_ptr), intent(out) :: srv
    end function

    subroutine mld_gpu_server_destroy(srv) bind(C, name="mld_gpu_server_destroy")
      import :: c_ptr
      type(c_ptr), value :: srv
    end subroutine

    integer(c_int) function mld_gpu_server_submit(srv, nat, pos, cell, types, ticket) bind(C, name="mld_gpu_server_submit")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: srv, pos, cell, types
      integer(c_int), value :: nat
      integer(c_long_long), intent(out) :: ticket
    end function

    integer(c_int) function mld_gpu_server_progress(srv, n_busy, n_queued) bind(C, name="mld_gpu_server_progress")
      import :: c_int, c_ptr
      type(c_ptr), value :: srv
      integer(c_int), intent(out) :: n_busy, n_queued
    end function

    integer(c_int) function mld_gpu_server_result(srv, ticket, e, f, s, latency_ms, ready) &
        bind(C, name="mld_gpu_server_result")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: srv, e, f, s, latency_ms
      integer(c_long_long), value :: ticket
      integer(c_int), intent(out) :: ready
    end function

    integer(c_int) function mld_gpu_server_wait(srv, ticket, e, f, s, latency_ms, timeout_ms) &
        bind(C, name="mld_gpu_server_wait")
      import :: c_int, c_ptr, c_long_long, c_double
      type(c_ptr), value :: srv, e, f, s, latency_ms
      integer(c_long_long), value :: ticket
      real(c_double), value :: timeout_ms
    end function

    integer(c_int) function mld_gpu_server_stats(srv, batches, atoms_done, budget_bytes) &
        bind(C, name="mld_gpu_server_stats")
      import :: c_int, c_ptr, c_long_long, c_double
      type(c_ptr), value :: srv
      integer(c_long_long), intent(out) :: batches, atoms_done
      real(c_double), intent(out) :: budget_bytes
    end function

    integer(c_int) function mld_gpu_tuning(h, mode, shape, ncand, ms) bind(C, name="mld_gpu_tuning")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: mode
      integer(c_int), intent(out) :: shape(4)
      integer(c_int), intent(inout) :: ncand
      real(c_double), intent(out) :: ms(*)
    end function

    integer(c_int) function mld_gpu_test_pipeline_timeout(skip_loads, wait_limit_clocks) &
        bind(C, name="mld_gpu_test_pipeline_timeout")
      import :: c_int, c_long_long
      integer(c_int), value :: skip_loads
      integer(c_long_long), value :: wait_limit_clocks
    end function

    integer(c_int) function mld_gpu_server_admission(srv, peak_bytes_in_flight, share_bytes, largest_batch_bytes) &
        bind(C, name="mld_gpu_server_admission")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: srv
      real(c_double), intent(out) :: peak_bytes_in_flight, share_bytes, largest_batch_bytes
    end function
  end interface
end module mld_gpu_mod
