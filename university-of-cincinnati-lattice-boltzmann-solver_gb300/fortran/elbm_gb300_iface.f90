! ISO_C_BINDING interface to libelbm_gb300 (include/elbm_gb300.h).
!
! The reference's per-level driver (looping/timestepping/loop.f95:94-147) keeps
! its calls streaming(level_step,fine,lvl), calculate_flow_variables(...),
! collision(...) and damp_it(...).  With this module their bodies become one
! call of elbm_level_step per level and sub-cycle, after the level's boxes
! were registered (from_scratch, amr/modules/amr_processes.f95:383-476) and
! their FABs uploaded.  No Fortran compiler is available where this library is
! built, so this file is shipped as source; the same entry points are
! exercised from Python (ctypes) by the library's tests.
module elbm_gb300_iface
  use iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: ELBM_OK = 0, ELBM_E_ARG = -1, ELBM_E_CUDA = -2, &
    ELBM_E_UNSUPPORTED = -3, ELBM_E_STATE = -4, ELBM_E_NUMERIC = -5
  integer(c_int), parameter, public :: ELBM_ST_NAN = 1, ELBM_ST_NEWTON_FALLBACK = 2, ELBM_ST_NEG_POP = 4, &
    ELBM_ST_DH_TOL = 8, ELBM_ST_COPY_TIMEOUT = 16
  integer(c_int), parameter, public :: ELBM_KERNEL_VARIANTS = 10, ELBM_MLP_PARAMS = 6017, ELBM_MLP_RECORD = 29
  integer(c_int), parameter, public :: ELBM_D3Q27 = 27, ELBM_D3Q39 = 39
  integer(c_int), parameter, public :: ELBM_STORE_FP64 = 0, ELBM_STORE_FP32_DEV = 1
  integer(c_int), parameter, public :: ELBM_ALPHA_FIXED2 = 0, ELBM_ALPHA_NEWTON = 1, ELBM_ALPHA_LEARNED = 2

  type, bind(c), public :: elbm_d3q27_params
    real(c_double) :: nu, tol_alpha, tol_dH
    integer(c_int32_t) :: max_newton, alpha_mode, check_dH, record_alpha
    integer(c_int32_t) :: outlet_type(8)
    real(c_double) :: fs_feq(27)
    real(c_double) :: inl_feq(27, 8)   ! C layout inl_feq[8][27]
    real(c_double) :: outl_feq(27, 8)
    integer(c_int32_t) :: damp, pad_damp
  end type

  type, bind(c), public :: elbm_d3q39_params
    integer(c_int32_t) :: shifted, primary_flow_dir, turbulent, lvl, startup_timesteps, max_lm_iters
    integer(c_int32_t) :: periodic, timestep, damp, pad
    real(c_double) :: gama, t_ref, rho_ref, p_ref, mu_ref, kappa_ref, gas_const_R, const_vol, &
      const_press, molec_weight
    real(c_double) :: dt, elbm_epsilon, init_beta_1, init_beta_2, beta_1_scaling, beta_2_scaling
    real(c_double) :: su_lm(13)   ! su_chi .. su_lambda_z
  end type

  type, bind(c), public :: elbm_d3q39_bc
    integer(c_int32_t) :: inlet_type(8), outlet_type(8)
    real(c_double) :: fs_fieq(39), fs_gieq(39)
    real(c_double) :: inl_fieq(39, 8), inl_gieq(39, 8)    ! C layout [8][39]
    real(c_double) :: outl_fieq(39, 8), outl_gieq(39, 8)
    real(c_double) :: fs_u, fs_v, fs_w, fs_temp
  end type

  type, bind(c), public :: elbm_plot3d_header
    real(c_double) :: mach, reynolds, time, gama, t_ref, stag_temperature, const_vol, const_press, non_dim_R
  end type

  type, bind(c), public :: elbm_stats
    integer(c_int64_t) :: node_updates, newton_iters, exact_path_nodes, fallbacks
    integer(c_int32_t) :: status, pad
    real(c_double) :: max_abs_dH
    integer(c_int64_t) :: dh_over_tol, guess_misses
    real(c_double) :: kernel_ms
  end type

  public :: elbm_create, elbm_destroy, elbm_level_register, elbm_set_d3q27_params, elbm_set_links, &
    elbm_upload_level, elbm_download_level, elbm_download_alpha, elbm_level_step, elbm_sync, &
    elbm_set_d3q39_params, elbm_upload_level39, elbm_download_level39, elbm_mark_triangles, &
    elbm_upload_level_noalloc, elbm_autotune, elbm_set_kernel_variant, elbm_alpha_harvest, &
    elbm_alpha_mlp_train, elbm_set_alpha_mlp, elbm_interlevel_setup, elbm_fill_fine_ghosts, &
    elbm_average_down, elbm_amr_run, elbm_damp_level, elbm_set_links39, elbm_upload_macro39, &
    elbm_init_level39, elbm_d3q39_equilibrium, elbm_checkpoint_write, elbm_checkpoint_read, elbm_ggm_tags, elbm_ggm_tags_pgs, &
    elbm_write_plot3d, elbm_mic_sample, elbm_mark_triangles_gpu, elbm_last_error_string, &
    elbm_alpha_mlp_grad, elbm_alpha_mlp_infer, elbm_links39_tables, elbm_error_message, &
    elbm_mark_triangles39, elbm_mark_triangles39_gpu

  interface
    integer(c_int) function elbm_create(device, ctx) bind(c, name="elbm_create")
      import :: c_int, c_ptr
      integer(c_int), value :: device
      type(c_ptr) :: ctx
    end function
    subroutine elbm_destroy(ctx) bind(c, name="elbm_destroy")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function elbm_level_register(ctx, lvl, lattice, storage, nbox, lo_hi, ngrow) &
        bind(c, name="elbm_level_register")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, lattice, storage, nbox, ngrow
      integer(c_int32_t), intent(in) :: lo_hi(6, *)   ! mfi%validbox() lo/hi, 0-based
    end function
    integer(c_int) function elbm_set_d3q27_params(ctx, lvl, p) bind(c, name="elbm_set_d3q27_params")
      import :: c_int, c_ptr, elbm_d3q27_params
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      type(elbm_d3q27_params), intent(in) :: p
    end function
    integer(c_int) function elbm_set_links(ctx, lvl, box, state, ngrow_state) bind(c, name="elbm_set_links")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box, ngrow_state
      integer(c_int32_t), intent(in) :: state(*)      ! mfstate(lvl)%dataptr(mfi)
    end function
    integer(c_int) function elbm_upload_level(ctx, lvl, box, fout) bind(c, name="elbm_upload_level")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(in) :: fout(*)           ! mffout(lvl)%dataptr(mfi)
    end function
    integer(c_int) function elbm_download_level(ctx, lvl, box, fout) bind(c, name="elbm_download_level")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(out) :: fout(*)
    end function
    integer(c_int) function elbm_download_alpha(ctx, lvl, box, alpha) bind(c, name="elbm_download_alpha")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(out) :: alpha(*)
    end function
    integer(c_int) function elbm_level_step(ctx, lvl, nsteps, stats) bind(c, name="elbm_level_step")
      import :: c_int, c_ptr, elbm_stats
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, nsteps
      type(elbm_stats), intent(out) :: stats
    end function
    integer(c_int) function elbm_sync(ctx) bind(c, name="elbm_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function elbm_set_d3q39_params(ctx, lvl, p) bind(c, name="elbm_set_d3q39_params")
      import :: c_int, c_ptr, elbm_d3q39_params
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      type(elbm_d3q39_params), intent(in) :: p
    end function
    integer(c_int) function elbm_upload_level39(ctx, lvl, box, fout, gout, lm, w_vel) &
        bind(c, name="elbm_upload_level39")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(in) :: fout(*), gout(*), lm(*), w_vel(*)
    end function
    integer(c_int) function elbm_ggm_tags(ctx, lvl, box, variable, scheme, limit, tags, ggm, ntagged) &
        bind(c, name="elbm_ggm_tags")
      import :: c_int, c_ptr, c_double, c_int64_t, c_int8_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box, variable, scheme
      real(c_double), value :: limit
      integer(c_int8_t), intent(out) :: tags(*)
      type(c_ptr), value :: ggm            ! c_loc(ggm values) or c_null_ptr
      integer(c_int64_t), intent(out) :: ntagged
    end function
    integer(c_int) function elbm_ggm_tags_pgs(ctx, lvl, box, variable, scheme, limit, pgs_sensitivity, pgs_reach, &
        tags, ggm, ntagged) bind(c, name="elbm_ggm_tags_pgs")
      import :: c_int, c_ptr, c_double, c_int64_t, c_int8_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box, variable, scheme, pgs_reach
      real(c_double), value :: limit, pgs_sensitivity
      integer(c_int8_t), intent(out) :: tags(*)
      type(c_ptr), value :: ggm            ! c_loc(ggm values) or c_null_ptr
      integer(c_int64_t), intent(out) :: ntagged
    end function
    integer(c_int) function elbm_mark_triangles_gpu(ctx, nx, ny, nz, origin, dx, ntri, tri, state) &
        bind(c, name="elbm_mark_triangles_gpu")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: nx, ny, nz, ntri
      real(c_double), intent(in) :: origin(3), tri(9, *)
      real(c_double), value :: dx
      integer(c_int32_t), intent(inout) :: state(*)
    end function
    integer(c_int) function elbm_mark_triangles39(nx, ny, nz, origin, dx, ntri, tri, shifted, primary_flow_dir, &
        periodic, state) bind(c, name="elbm_mark_triangles39")
      import :: c_int, c_double, c_int32_t
      integer(c_int), value :: nx, ny, nz, ntri, shifted, primary_flow_dir, periodic
      real(c_double), intent(in) :: origin(3), tri(9, *)
      real(c_double), value :: dx
      integer(c_int32_t), intent(inout) :: state(*)
    end function
    integer(c_int) function elbm_mark_triangles39_gpu(ctx, nx, ny, nz, origin, dx, ntri, tri, shifted, &
        primary_flow_dir, periodic, state) bind(c, name="elbm_mark_triangles39_gpu")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: nx, ny, nz, ntri, shifted, primary_flow_dir, periodic
      real(c_double), intent(in) :: origin(3), tri(9, *)
      real(c_double), value :: dx
      integer(c_int32_t), intent(inout) :: state(*)
    end function
    integer(c_int) function elbm_write_plot3d(ctx, lvl, grid_path, data_path, origin, dx, hdr) &
        bind(c, name="elbm_write_plot3d")
      import :: c_int, c_ptr, c_char, c_double, elbm_plot3d_header
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      character(kind=c_char), intent(in) :: grid_path(*), data_path(*)   ! NUL-terminated
      real(c_double), intent(in) :: origin(3)
      real(c_double), value :: dx
      type(elbm_plot3d_header), intent(in) :: hdr
    end function
    integer(c_int) function elbm_mic_sample(ctx, lvl, box, nmic, nodes, weights, values) &
        bind(c, name="elbm_mic_sample")
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box, nmic
      integer(c_int32_t), intent(in) :: nodes(8, *)
      real(c_double), intent(in) :: weights(8, *)
      real(c_double), intent(out) :: values(6, *)
    end function
    integer(c_int) function elbm_checkpoint_write(ctx, lvl, path) bind(c, name="elbm_checkpoint_write")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
    end function
    integer(c_int) function elbm_checkpoint_read(ctx, lvl, path) bind(c, name="elbm_checkpoint_read")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function elbm_init_level39(ctx, lvl, box, macro, lm_start, capped) &
        bind(c, name="elbm_init_level39")
      import :: c_int, c_ptr, c_double, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(in) :: macro(*), lm_start(13)
      integer(c_int64_t), intent(out) :: capped
    end function
    integer(c_int) function elbm_d3q39_equilibrium(ctx, p, macro, lm, fieq, gieq) &
        bind(c, name="elbm_d3q39_equilibrium")
      import :: c_int, c_ptr, c_double, elbm_d3q39_params
      type(c_ptr), value :: ctx
      type(elbm_d3q39_params), intent(in) :: p
      real(c_double), intent(in) :: macro(5)
      real(c_double), intent(inout) :: lm(13)
      real(c_double), intent(out) :: fieq(39), gieq(39)
    end function
    integer(c_int) function elbm_upload_macro39(ctx, lvl, box, macro) bind(c, name="elbm_upload_macro39")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(in) :: macro(*)   ! rho, u_vel, v_vel, w_vel, temp as one 5-component FAB
    end function
    integer(c_int) function elbm_download_level39(ctx, lvl, box, fout, gout, lm, w_vel, alpha, macro) &
        bind(c, name="elbm_download_level39")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      type(c_ptr), value :: fout, gout, lm, w_vel, alpha, macro  ! c_loc(...) or c_null_ptr
    end function
    integer(c_int) function elbm_mark_triangles(nx, ny, nz, origin, dx, ntri, tri, state) &
        bind(c, name="elbm_mark_triangles")
      import :: c_int, c_double, c_int32_t
      integer(c_int), value :: nx, ny, nz, ntri
      real(c_double), intent(in) :: origin(3)
      real(c_double), value :: dx
      real(c_double), intent(in) :: tri(9, *)          ! vertex coordinates of each triangle
      integer(c_int32_t), intent(inout) :: state(*)   ! 27 components of nx*ny*nz (no ghosts)
    end function
    integer(c_int) function elbm_upload_level_noalloc(ctx, lvl, box, fout) bind(c, name="elbm_upload_level_noalloc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box
      real(c_double), intent(in) :: fout(*)
    end function
    integer(c_int) function elbm_autotune(ctx, lvl, reps, chosen, ms_per_variant) bind(c, name="elbm_autotune")
      import :: c_int, c_ptr, c_double, ELBM_KERNEL_VARIANTS
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, reps
      integer(c_int), intent(out) :: chosen
      real(c_double), intent(out) :: ms_per_variant(ELBM_KERNEL_VARIANTS)
    end function
    integer(c_int) function elbm_set_kernel_variant(ctx, lvl, variant) bind(c, name="elbm_set_kernel_variant")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, variant
    end function
    integer(c_int) function elbm_alpha_harvest(ctx, lvl, nsteps, stride, records, capacity, count) &
        bind(c, name="elbm_alpha_harvest")
      import :: c_int, c_ptr, c_float, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, nsteps, stride
      real(c_float), intent(out) :: records(29, *)
      integer(c_int64_t), value :: capacity
      integer(c_int64_t), intent(out) :: count
    end function
    integer(c_int) function elbm_alpha_mlp_train(ctx, records, n, epochs, batch, lr, seed, weights, loss_per_epoch) &
        bind(c, name="elbm_alpha_mlp_train")
      import :: c_int, c_ptr, c_float, c_int64_t, c_double
      type(c_ptr), value :: ctx
      real(c_float), intent(in) :: records(29, *)
      integer(c_int64_t), value :: n, seed
      integer(c_int), value :: epochs, batch
      real(c_float), value :: lr
      real(c_float), intent(inout) :: weights(6017)
      real(c_double), intent(out) :: loss_per_epoch(*)
    end function
    integer(c_int) function elbm_set_alpha_mlp(ctx, lvl, weights) bind(c, name="elbm_set_alpha_mlp")
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      real(c_float), intent(in) :: weights(6017)
    end function
    integer(c_int) function elbm_interlevel_setup(ctx, lvl) bind(c, name="elbm_interlevel_setup")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
    end function
    integer(c_int) function elbm_fill_fine_ghosts(ctx, lvl, repaired) bind(c, name="elbm_fill_fine_ghosts")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      integer(c_int64_t), intent(out) :: repaired
    end function
    integer(c_int) function elbm_average_down(ctx, lvl) bind(c, name="elbm_average_down")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
    end function
    integer(c_int) function elbm_amr_run(ctx, nlev, ncycles, stats) bind(c, name="elbm_amr_run")
      import :: c_int, c_ptr, elbm_stats
      type(c_ptr), value :: ctx
      integer(c_int), value :: nlev, ncycles
      type(elbm_stats), intent(out) :: stats
    end function
    integer(c_int) function elbm_damp_level(ctx, lvl, repaired) bind(c, name="elbm_damp_level")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl
      integer(c_int64_t), intent(out) :: repaired
    end function
    integer(c_int) function elbm_set_links39(ctx, lvl, box, state, ngrow_state, bc) bind(c, name="elbm_set_links39")
      import :: c_int, c_ptr, c_int32_t, elbm_d3q39_bc
      type(c_ptr), value :: ctx
      integer(c_int), value :: lvl, box, ngrow_state
      integer(c_int32_t), intent(in) :: state(*)      ! mfstate(lvl)%dataptr(mfi), 39 comps
      type(elbm_d3q39_bc), intent(in) :: bc
    end function
    ! The message of the last error on the context (a NUL-terminated C string owned by the
    ! library, valid until the next call on the context); elbm_error_message copies it.
    type(c_ptr) function elbm_last_error_string(ctx) bind(c, name="elbm_last_error_string")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function elbm_alpha_mlp_grad(ctx, weights, records, n, grad, loss) &
        bind(c, name="elbm_alpha_mlp_grad")
      import :: c_int, c_ptr, c_float, c_int64_t, c_double
      type(c_ptr), value :: ctx
      real(c_float), intent(in) :: weights(6017), records(29, *)
      integer(c_int64_t), value :: n
      real(c_float), intent(out) :: grad(6017)
      real(c_double), intent(out) :: loss
    end function
    integer(c_int) function elbm_alpha_mlp_infer(ctx, weights, x, n, out, status) &
        bind(c, name="elbm_alpha_mlp_infer")
      import :: c_int, c_ptr, c_float, c_int64_t, c_int32_t
      type(c_ptr), value :: ctx
      real(c_float), intent(in) :: weights(6017), x(27, *)
      integer(c_int64_t), value :: n
      real(c_float), intent(out) :: out(*)
      integer(c_int32_t), intent(out) :: status
    end function
    integer(c_int) function elbm_links39_tables(nx, ny, nz, state, ngrow_state, periodic, shifted, &
        primary_flow_dir, inlet_type, outlet_type, ntype, rec_node, words, capacity, nrec) &
        bind(c, name="elbm_links39_tables")
      import :: c_int, c_int32_t, c_int8_t, c_int64_t
      integer(c_int), value :: nx, ny, nz, ngrow_state, periodic, shifted, primary_flow_dir
      integer(c_int32_t), intent(in) :: state(*), inlet_type(8), outlet_type(8)
      integer(c_int8_t), intent(out) :: ntype(*)
      integer(c_int32_t), intent(out) :: rec_node(*), words(39, *)   ! words: uint32 link words
      integer(c_int64_t), value :: capacity
      integer(c_int64_t), intent(out) :: nrec
    end function
  end interface

contains

  ! The last error message of a context as a Fortran string (the C string copied up to its NUL,
  ! blank-padded or cut to len(msg)), for the reference's error_out
  ! (general/background_calcs/error_out.f95:12-14) to print before it stops.
  subroutine elbm_error_message(ctx, msg)
    type(c_ptr), value :: ctx
    character(len=*), intent(out) :: msg
    character(kind=c_char), pointer :: cs(:)
    type(c_ptr) :: p
    integer :: i
    msg = ' '
    p = elbm_last_error_string(ctx)
    if (.not. c_associated(p)) return
    call c_f_pointer(p, cs, [len(msg)])
    do i = 1, len(msg)
      if (cs(i) == c_null_char) exit
      msg(i:i) = cs(i)
    end do
  end subroutine
end module elbm_gb300_iface

! Example body of the reference's per-level collide-stream call with the
! library (all boxes of the level registered at once; `ctx` created once with
! elbm_create):
!
!   subroutine collision(level_step, fine, lvl)
!     use elbm_gb300_iface
!     ...
!     if (.not. level_step(lvl)) return
!     rc = elbm_level_step(ctx, lvl, 1, stats)
!     if (rc /= ELBM_OK .or. iand(stats%status, 1) /= 0) call error_out
!   end subroutine
