!-----------------------------------------------------------------------------!
! channel_gpu.f90 -- Fortran binding of libchannel_gpu (include/channel_gpu.h)
!
! Module channel_gpu: ISO_C_BINDING interfaces of every function the C header
! declares, the cf_params record and the header's constants.
! Module channel_gpu_dropin: subroutines with the names and dummy arguments of
! the reference's hot-path subroutines (the ones time_integration.f90 calls),
! forwarding to the library on the device-resident state, and a
! compute_time_step_RK3 that issues them in the order of
! time_integration.f90:89-173.
!
! Status: not compiled in this build image, which has no Fortran compiler.
! The interfaces are checked against include/channel_gpu.h by
! tests/test_fortran_binding.py (names, argument counts and order, kinds,
! pass-by-value attributes, the cf_params layout); the call order of
! channel_gpu_dropin is the one the C driver tests/c_driver/rk3_mirror.c
! runs on the GPU against cf_time_step_rk3.
!
! Arrays: host arrays are passed as assumed-size Real(c_double) in the
! reference's layout and extents (U(nx,nyg,nzg) etc.); device arrays (the
! learned wall-stress and no-allocation entry points) as Type(c_ptr) by value.
! Strings are NUL-terminated Character(c_char) arrays: pass
! Trim(name)//c_null_char.
!-----------------------------------------------------------------------------!
Module channel_gpu

  Use, Intrinsic :: iso_c_binding
  Implicit None

  ! return codes and precision selectors (channel_gpu.h)
  Integer(c_int), Parameter :: CF_OK = 0, CF_ERR_INVALID = 1, CF_ERR_CUDA = 2, &
                               CF_ERR_UNSUPPORTED = 3, CF_ERR_IO = 4, CF_ERR_NAN = 5
  Integer(c_int), Parameter :: CF_PREC_FP64 = 0, CF_PREC_SPLIT = 1
  Integer(c_int), Parameter :: CF_MLP_NPARAM = 4481
  Integer(c_int), Parameter :: CF_NOALLOC_MAX_PLANES = 4096
  Integer(c_int), Parameter :: CF_ENS_TUNE_CANDIDATES = 8

  ! the scalars of read_input_parameters (input_output.f90:21-133) plus the
  ! library's options; field order and kinds are those of the C struct
  Type, Bind(C) :: cf_params
     Real(c_double)    :: nu
     Real(c_double)    :: CFL
     Real(c_double)    :: dPdx
     Real(c_double)    :: dPdz
     Real(c_double)    :: Rossby_plus
     Real(c_double)    :: freq_mult
     Integer(c_int)    :: Retau_int
     Integer(c_int)    :: x_mass_cte
     Integer(c_int)    :: y_mass_cte
     Integer(c_int)    :: LES_model
     Integer(c_int)    :: iwall_model
     Integer(c_int)    :: Dirichlet_nu_t
     Integer(c_int)    :: jref_eqwm
     Integer(c_int)    :: precision
     Integer(c_int)    :: eqwm_ncv
     Real(c_double)    :: eqwm_stretch
     Integer(c_int)    :: sgs_recompute
     Integer(c_int)    :: dsm_unfused
     Integer(c_int)    :: cfl_corrected
  End Type cf_params

  Interface

     !---------------------------------------------------- parameters, lifetime
     Subroutine cf_default_params(p) Bind(C, name="cf_default_params")
       Import :: cf_params
       Type(cf_params) :: p
     End Subroutine cf_default_params

     Integer(c_int) Function cf_create(nx, ny, nz, x, y, z, p, device, out) Bind(C, name="cf_create")
       Import :: c_int, c_double, c_ptr, cf_params
       Integer(c_int), Value :: nx, ny, nz
       Real(c_double)        :: x(*), y(*), z(*)
       Type(cf_params)       :: p
       Integer(c_int), Value :: device
       Type(c_ptr)           :: out
     End Function cf_create

     Integer(c_int) Function cf_destroy(ctx) Bind(C, name="cf_destroy")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_destroy

     ! returns a C string (const char *): convert with c_f_pointer
     Type(c_ptr) Function cf_last_error(ctx) Bind(C, name="cf_last_error")
       Import :: c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_last_error

     !--------------------------------------------------------- state transfer
     Integer(c_int) Function cf_upload_fields(ctx, U, V, W) Bind(C, name="cf_upload_fields")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: U(*), V(*), W(*)
     End Function cf_upload_fields

     Integer(c_int) Function cf_download_fields(ctx, U, V, W, P, nu_t) Bind(C, name="cf_download_fields")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: U(*), V(*), W(*), P(*), nu_t(*)
     End Function cf_download_fields

     Integer(c_int) Function cf_download_wall(ctx, alpha_x, alpha_z, tau) Bind(C, name="cf_download_wall")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: alpha_x(*), alpha_z(*), tau(*)
     End Function cf_download_wall

     Integer(c_int) Function cf_upload_wall(ctx, alpha_x, alpha_z, tau) Bind(C, name="cf_upload_wall")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: alpha_x(*), alpha_z(*), tau(*)
     End Function cf_upload_wall

     Integer(c_int) Function cf_set_scalars(ctx, t, dt, rk_step, dPdx, dPdy) Bind(C, name="cf_set_scalars")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: ctx
       Real(c_double), Value :: t, dt
       Integer(c_int), Value :: rk_step
       Real(c_double), Value :: dPdx, dPdy
     End Function cf_set_scalars

     Integer(c_int) Function cf_get_scalars(ctx, t, dt, rk_step, dPdx, dPdy) Bind(C, name="cf_get_scalars")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: t, dt
       Integer(c_int)     :: rk_step
       Real(c_double)     :: dPdx, dPdy
     End Function cf_get_scalars

     Integer(c_int) Function cf_init_mass_flow(ctx, Qflow_x_0) Bind(C, name="cf_init_mass_flow")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: Qflow_x_0
     End Function cf_init_mass_flow

     !----------------------- mirrors of the subroutines time_integration.f90 calls
     Integer(c_int) Function cf_compute_dt(ctx, dt) Bind(C, name="cf_compute_dt")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: dt
     End Function cf_compute_dt

     Integer(c_int) Function cf_compute_eddy_viscosity(ctx) Bind(C, name="cf_compute_eddy_viscosity")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_compute_eddy_viscosity

     Integer(c_int) Function cf_compute_wall_model(ctx) Bind(C, name="cf_compute_wall_model")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_compute_wall_model

     Integer(c_int) Function cf_compute_rhs_u(ctx, slot) Bind(C, name="cf_compute_rhs_u")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: slot
     End Function cf_compute_rhs_u

     Integer(c_int) Function cf_compute_rhs_v(ctx, slot) Bind(C, name="cf_compute_rhs_v")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: slot
     End Function cf_compute_rhs_v

     Integer(c_int) Function cf_compute_rhs_w(ctx, slot) Bind(C, name="cf_compute_rhs_w")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: slot
     End Function cf_compute_rhs_w

     Integer(c_int) Function cf_rk_update(ctx, substep) Bind(C, name="cf_rk_update")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: substep
     End Function cf_rk_update

     Integer(c_int) Function cf_apply_boundary_conditions(ctx) Bind(C, name="cf_apply_boundary_conditions")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_apply_boundary_conditions

     Integer(c_int) Function cf_compute_projection_step(ctx) Bind(C, name="cf_compute_projection_step")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_compute_projection_step

     Integer(c_int) Function cf_compute_dPx_for_constant_mass_flow(ctx, dPdx) &
          Bind(C, name="cf_compute_dPx_for_constant_mass_flow")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: dPdx
     End Function cf_compute_dPx_for_constant_mass_flow

     Integer(c_int) Function cf_compute_dPy_for_constant_mass_flow(ctx, dPdy) &
          Bind(C, name="cf_compute_dPy_for_constant_mass_flow")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: dPdy
     End Function cf_compute_dPy_for_constant_mass_flow

     Integer(c_int) Function cf_compute_dPx_for_constant_Ucenterline(ctx, dPdx) &
          Bind(C, name="cf_compute_dPx_for_constant_Ucenterline")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: dPdx
     End Function cf_compute_dPx_for_constant_Ucenterline

     Integer(c_int) Function cf_check_divergence(ctx, maxdiv, maxabsdiv) Bind(C, name="cf_check_divergence")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: maxdiv, maxabsdiv
     End Function cf_check_divergence

     Integer(c_int) Function cf_compute_pressure(ctx) Bind(C, name="cf_compute_pressure")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_compute_pressure

     Integer(c_int) Function cf_apply_mass_flow_correction(ctx, comp, value) &
          Bind(C, name="cf_apply_mass_flow_correction")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: comp
       Real(c_double), Value :: value
     End Function cf_apply_mass_flow_correction

     Integer(c_int) Function cf_save_old_state(ctx) Bind(C, name="cf_save_old_state")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_save_old_state

     Integer(c_int) Function cf_download_rhs(ctx, comp, slot, out) Bind(C, name="cf_download_rhs")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: comp, slot
       Real(c_double)        :: out(*)
     End Function cf_download_rhs

     Integer(c_int) Function cf_download_avg_nu_t(ctx, out) Bind(C, name="cf_download_avg_nu_t")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: out(*)
     End Function cf_download_avg_nu_t

     ! u_les: device array (Type(c_ptr)) of cap doubles, or c_null_ptr to query npts
     Integer(c_int) Function cf_wall_model_inputs(ctx, u_les, cap, npts, h_wm, nu) Bind(C, name="cf_wall_model_inputs")
       Import :: c_int, c_long, c_double, c_ptr
       Type(c_ptr), Value     :: ctx, u_les
       Integer(c_long), Value :: cap
       Integer(c_long)        :: npts
       Real(c_double)         :: h_wm, nu
     End Function cf_wall_model_inputs

     Integer(c_int) Function cf_get_eqwm_counters(ctx, n_nan, n_iter) Bind(C, name="cf_get_eqwm_counters")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int)     :: n_nan, n_iter
     End Function cf_get_eqwm_counters

     Integer(c_int) Function cf_copy_wait_expired(ctx, expired) Bind(C, name="cf_copy_wait_expired")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int)     :: expired
     End Function cf_copy_wait_expired

     Integer(c_int) Function cf_test_skip_plane_copy(ctx, on) Bind(C, name="cf_test_skip_plane_copy")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: on
     End Function cf_test_skip_plane_copy

     !-------------------------------------------------------------- fast path
     Integer(c_int) Function cf_time_step_rk3(ctx, nsteps, sync) Bind(C, name="cf_time_step_rk3")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: nsteps, sync
     End Function cf_time_step_rk3

     Integer(c_int) Function cf_set_fixed_dt(ctx, dt) Bind(C, name="cf_set_fixed_dt")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: ctx
       Real(c_double), Value :: dt
     End Function cf_set_fixed_dt

     Integer(c_int) Function cf_synchronize(ctx) Bind(C, name="cf_synchronize")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_synchronize

     Type(c_ptr) Function cf_get_stream(ctx) Bind(C, name="cf_get_stream")
       Import :: c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_get_stream

     Integer(c_int) Function cf_launches_per_step(ctx) Bind(C, name="cf_launches_per_step")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
     End Function cf_launches_per_step

     ! names: max_names rows of 48 characters
     Integer(c_int) Function cf_profile_steps(ctx, nsteps, max_names, names, total_ms, counts, n_names) &
          Bind(C, name="cf_profile_steps")
       Import :: c_int, c_double, c_char, c_ptr
       Type(c_ptr), Value     :: ctx
       Integer(c_int), Value  :: nsteps, max_names
       Character(kind=c_char) :: names(*)
       Real(c_double)         :: total_ms(*)
       Integer(c_int)         :: counts(*)
       Integer(c_int)         :: n_names
     End Function cf_profile_steps

     Integer(c_int) Function cf_profile_graph_steps(ctx, nsteps, max_names, names, total_ms, counts, n_names) &
          Bind(C, name="cf_profile_graph_steps")
       Import :: c_int, c_double, c_char, c_ptr
       Type(c_ptr), Value     :: ctx
       Integer(c_int), Value  :: nsteps, max_names
       Character(kind=c_char) :: names(*)
       Real(c_double)         :: total_ms(*)
       Integer(c_int)         :: counts(*)
       Integer(c_int)         :: n_names
     End Function cf_profile_graph_steps

     Integer(c_int) Function cf_autotune(ctx, reps, report) Bind(C, name="cf_autotune")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: ctx
       Integer(c_int), Value :: reps
       Real(c_double)        :: report(*)
     End Function cf_autotune

     !------------------------------------------------------------ statistics
     Integer(c_int) Function cf_compute_statistics(ctx, out) Bind(C, name="cf_compute_statistics")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: out(*)
     End Function cf_compute_statistics

     Integer(c_int) Function cf_output_monitor(ctx, out) Bind(C, name="cf_output_monitor")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: out(*)
     End Function cf_output_monitor

     !------------------------------------- input_parameters and snapshot format
     ! filein, fileout: 200 characters each
     Integer(c_int) Function cf_read_input_parameters(path, p, grid, filein, fileout, ints, ints2) &
          Bind(C, name="cf_read_input_parameters")
       Import :: c_int, c_char, cf_params
       Character(kind=c_char) :: path(*)
       Type(cf_params)        :: p
       Integer(c_int)         :: grid(3)
       Character(kind=c_char) :: filein(*), fileout(*)
       Integer(c_int)         :: ints(4), ints2(2)
     End Function cf_read_input_parameters

     Integer(c_int) Function cf_read_snapshot(path, nx, ny, nz, x, y, z, U, V, W) Bind(C, name="cf_read_snapshot")
       Import :: c_int, c_double, c_char
       Character(kind=c_char) :: path(*)
       Integer(c_int), Value  :: nx, ny, nz
       Real(c_double)         :: x(*), y(*), z(*), U(*), V(*), W(*)
     End Function cf_read_snapshot

     Integer(c_int) Function cf_write_snapshot(path, nx, ny, nz, x, y, z, U, V, W, P, nu_t) &
          Bind(C, name="cf_write_snapshot")
       Import :: c_int, c_double, c_char
       Character(kind=c_char) :: path(*)
       Integer(c_int), Value  :: nx, ny, nz
       Real(c_double)         :: x(*), y(*), z(*), U(*), V(*), W(*), P(*), nu_t(*)
     End Function cf_write_snapshot

     Integer(c_int) Function cf_write_statistics(path, t, nu, nx, ny, nz, istep, y, stats) &
          Bind(C, name="cf_write_statistics")
       Import :: c_int, c_double, c_char
       Character(kind=c_char) :: path(*)
       Real(c_double), Value  :: t, nu
       Integer(c_int), Value  :: nx, ny, nz, istep
       Real(c_double)         :: y(*), stats(*)
     End Function cf_write_statistics

     Integer(c_int) Function cf_statistics_file_name(fileout, istep, nstep_init, name, cap) &
          Bind(C, name="cf_statistics_file_name")
       Import :: c_int, c_char
       Character(kind=c_char) :: fileout(*)
       Integer(c_int), Value  :: istep, nstep_init
       Character(kind=c_char) :: name(*)
       Integer(c_int), Value  :: cap
     End Function cf_statistics_file_name

     !----------------------------- learned wall-stress model (device pointers)
     Integer(c_int) Function cf_eqwm_solve_batch(n, u, h, nu, ncv, stretch, tau_init, tau, iters, stream) &
          Bind(C, name="cf_eqwm_solve_batch")
       Import :: c_int, c_double, c_ptr
       Integer(c_int), Value :: n
       Type(c_ptr), Value    :: u, h, nu
       Integer(c_int), Value :: ncv
       Real(c_double), Value :: stretch, tau_init
       Type(c_ptr), Value    :: tau, iters, stream
     End Function cf_eqwm_solve_batch

     Integer(c_int) Function cf_mlp_create(seed, ncv, stretch, out) Bind(C, name="cf_mlp_create")
       Import :: c_int, c_double, c_ptr
       Integer(c_int), Value :: seed, ncv
       Real(c_double), Value :: stretch
       Type(c_ptr)           :: out
     End Function cf_mlp_create

     Integer(c_int) Function cf_mlp_destroy(m) Bind(C, name="cf_mlp_destroy")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: m
     End Function cf_mlp_destroy

     Integer(c_int) Function cf_mlp_fit_normalisation(m, n, u, h, nu, tau, stream) &
          Bind(C, name="cf_mlp_fit_normalisation")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: n
       Type(c_ptr), Value    :: u, h, nu, tau, stream
     End Function cf_mlp_fit_normalisation

     ! loss_out: host array of `epochs` values (or c_null_ptr)
     Integer(c_int) Function cf_mlp_train(m, n, u, h, nu, tau, epochs, batch, lr, seed, loss_out, stream) &
          Bind(C, name="cf_mlp_train")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: n
       Type(c_ptr), Value    :: u, h, nu, tau
       Integer(c_int), Value :: epochs, batch
       Real(c_double), Value :: lr
       Integer(c_int), Value :: seed
       Type(c_ptr), Value    :: loss_out, stream
     End Function cf_mlp_train

     ! grad: device array; loss: host double
     Integer(c_int) Function cf_mlp_gradient(m, n, u, h, nu, tau, grad, loss, stream) &
          Bind(C, name="cf_mlp_gradient")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: n
       Type(c_ptr), Value    :: u, h, nu, tau, grad
       Real(c_double)        :: loss
       Type(c_ptr), Value    :: stream
     End Function cf_mlp_gradient

     Integer(c_int) Function cf_mlp_set_train_tensor_cores(m, on) Bind(C, name="cf_mlp_set_train_tensor_cores")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: on
     End Function cf_mlp_set_train_tensor_cores

     Integer(c_int) Function cf_mlp_predict(m, n, u, h, nu, tau, inside, use_tensor_cores, stream) &
          Bind(C, name="cf_mlp_predict")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: n
       Type(c_ptr), Value    :: u, h, nu, tau, inside
       Integer(c_int), Value :: use_tensor_cores
       Type(c_ptr), Value    :: stream
     End Function cf_mlp_predict

     ! host arrays: params (CF_MLP_NPARAM floats), norm (8), envelope (6)
     Integer(c_int) Function cf_mlp_get(m, params, norm, envelope) Bind(C, name="cf_mlp_get")
       Import :: c_int, c_float, c_double, c_ptr
       Type(c_ptr), Value :: m
       Real(c_float)      :: params(*)
       Real(c_double)     :: norm(*), envelope(*)
     End Function cf_mlp_get

     Integer(c_int) Function cf_mlp_set(m, params, norm, envelope) Bind(C, name="cf_mlp_set")
       Import :: c_int, c_float, c_double, c_ptr
       Type(c_ptr), Value :: m
       Real(c_float)      :: params(*)
       Real(c_double)     :: norm(*), envelope(*)
     End Function cf_mlp_set

     Integer(c_int) Function cf_mlp_wait_expired(m, expired) Bind(C, name="cf_mlp_wait_expired")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: m
       Integer(c_int)     :: expired
     End Function cf_mlp_wait_expired

     Integer(c_int) Function cf_mlp_test_skip_mma(m, on) Bind(C, name="cf_mlp_test_skip_mma")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: m
       Integer(c_int), Value :: on
     End Function cf_mlp_test_skip_mma

     Integer(c_int) Function cf_set_wall_mlp(ctx, m, check_every) Bind(C, name="cf_set_wall_mlp")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: ctx, m
       Integer(c_int), Value :: check_every
     End Function cf_set_wall_mlp

     Integer(c_int) Function cf_get_wall_mlp_log(ctx, out) Bind(C, name="cf_get_wall_mlp_log")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double)     :: out(*)
     End Function cf_get_wall_mlp_log

     !------------------------------------------ ensembles of independent channels
     ! members: n contexts (Type(c_ptr) array)
     Integer(c_int) Function cf_ensemble_create(n, members, out) Bind(C, name="cf_ensemble_create")
       Import :: c_int, c_ptr
       Integer(c_int), Value :: n
       Type(c_ptr)           :: members(*)
       Type(c_ptr)           :: out
     End Function cf_ensemble_create

     Integer(c_int) Function cf_ensemble_destroy(e) Bind(C, name="cf_ensemble_destroy")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: e
     End Function cf_ensemble_destroy

     Integer(c_int) Function cf_ensemble_step(e, nsteps, sync) Bind(C, name="cf_ensemble_step")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: e
       Integer(c_int), Value :: nsteps, sync
     End Function cf_ensemble_step

     Type(c_ptr) Function cf_ensemble_stream(e) Bind(C, name="cf_ensemble_stream")
       Import :: c_ptr
       Type(c_ptr), Value :: e
     End Function cf_ensemble_stream

     Integer(c_int) Function cf_ensemble_launches_per_step(e) Bind(C, name="cf_ensemble_launches_per_step")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: e
     End Function cf_ensemble_launches_per_step

     Integer(c_int) Function cf_ensemble_set_batched_tri(e, on) Bind(C, name="cf_ensemble_set_batched_tri")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: e
       Integer(c_int), Value :: on
     End Function cf_ensemble_set_batched_tri

     Integer(c_int) Function cf_ensemble_set_batched_stencils(e, on) Bind(C, name="cf_ensemble_set_batched_stencils")
       Import :: c_int, c_ptr
       Type(c_ptr), Value    :: e
       Integer(c_int), Value :: on
     End Function cf_ensemble_set_batched_stencils

     ! report: 4 doubles (or c_null_ptr); choice (or c_null_ptr)
     Integer(c_int) Function cf_ensemble_autotune(e, steps, report, choice) Bind(C, name="cf_ensemble_autotune")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value    :: e
       Integer(c_int), Value :: steps
       Real(c_double)        :: report(*)
       Integer(c_int)        :: choice
     End Function cf_ensemble_autotune

     !--------------------------- divergence check without device allocation
     ! every array argument is a device pointer
     Integer(c_int) Function cf_check_divergence_noalloc(nx, ny, nz, U, V, W, x, y, z, out, stream) &
          Bind(C, name="cf_check_divergence_noalloc")
       Import :: c_int, c_ptr
       Integer(c_int), Value :: nx, ny, nz
       Type(c_ptr), Value    :: U, V, W, x, y, z, out, stream
     End Function cf_check_divergence_noalloc

  End Interface

Contains

  ! cf_last_error as a Fortran string (message of ctx, or of the thread's last
  ! context-free failure when ctx is c_null_ptr)
  Function cf_error_message(ctx) Result(msg)
    Type(c_ptr), Intent(In) :: ctx
    Character(len=:), Allocatable :: msg
    Character(kind=c_char), Pointer :: s(:)
    Type(c_ptr) :: p
    Integer :: n
    p = cf_last_error(ctx)
    msg = ''
    If ( .Not. c_associated(p) ) Return
    Call c_f_pointer(p, s, [4096])
    n = 0
    Do While ( n < 4096 )
       If ( s(n+1) == c_null_char ) Exit
       n = n + 1
    End Do
    Allocate(Character(len=n) :: msg)
    msg = Transfer(s(1:n), msg)
  End Function cf_error_message

End Module channel_gpu


!-----------------------------------------------------------------------------!
! Drop-in subroutines: same names and dummy arguments as the reference's, on
! the device-resident state of the context `cf` (created by cf_dropin_start).
! The array dummies are kept so that time_integration.f90 compiles unchanged
! against them; the state they name lives on the GPU, and the host arrays of
! global are refreshed by cf_dropin_download (before output_data, statistics
! written from the host, and so on).  The right-hand-side slot of
! compute_rhs_* is the reference's: Fu1/Fu2/Fu3 at rk_step 1/2/3.
! A maintainer replaces the reference's Use of equations, subgrid, wallmodel,
! boundary_conditions, projection and mass_flow in time_integration.f90 by
! Use channel_gpu_dropin; compute_time_step_RK3 below is then the reference's
! sequence (time_integration.f90:89-173) with its array lines replaced by
! cf_save_old_state, cf_rk_update and cf_apply_mass_flow_correction.
!-----------------------------------------------------------------------------!
Module channel_gpu_dropin

  Use, Intrinsic :: iso_c_binding
  Use, Intrinsic :: iso_fortran_env, Only: error_unit, Int64
  Use channel_gpu
  Use global
  Implicit None

  Type(c_ptr), Save :: cf = c_null_ptr

Contains

  Subroutine cf_check(ierr, what)
    Integer(c_int), Intent(In) :: ierr
    Character(len=*), Intent(In) :: what
    If ( ierr /= CF_OK ) Then
       Write(error_unit,*) 'channel_gpu: ', what, ': ', cf_error_message(cf)
       Stop
    End If
  End Subroutine cf_check

  ! after initialize (initialization.f90:23-536): the context from global's
  ! grids and parameters, the fields of the snapshot and the mass flow
  Subroutine cf_dropin_start(device, precision)
    Integer(c_int), Intent(In) :: device, precision
    Type(cf_params) :: p
    Integer(c_int)  :: ierr
    Real(c_double)  :: q0
    Call cf_default_params(p)
    p%nu = nu ; p%CFL = CFL ; p%dPdx = dPdx ; p%dPdz = dPdz
    ! Omega_z = Rossby_plus*dPdx**0.5/2 (input_output.f90:83-84), read back
    If ( dPdx > 0d0 ) Then
       p%Rossby_plus = 2d0*Omega_z/dPdx**0.5d0
    Else
       p%Rossby_plus = 0d0
    End If
    p%freq_mult = freq_mult ; p%Retau_int = Retau_int
    p%x_mass_cte = x_mass_cte ; p%y_mass_cte = y_mass_cte ; p%LES_model = LES_model
    p%iwall_model = iwall_model ; p%Dirichlet_nu_t = Dirichlet_nu_t ; p%jref_eqwm = jref_eqwm
    p%precision = precision
    ierr = cf_create(Int(nx,c_int), Int(ny,c_int), Int(nz,c_int), x, y, z, p, device, cf)
    Call cf_check(ierr, 'cf_create')
    Call cf_check(cf_upload_fields(cf, U, V, W), 'cf_upload_fields')
    Call cf_check(cf_init_mass_flow(cf, q0), 'cf_init_mass_flow')
    Qflow_x_0 = q0
  End Subroutine cf_dropin_start

  Subroutine cf_dropin_download
    Call cf_check(cf_download_fields(cf, U, V, W, P, nu_t), 'cf_download_fields')
    Call cf_check(cf_download_avg_nu_t(cf, avg_nu_t), 'cf_download_avg_nu_t')
  End Subroutine cf_dropin_download

  Subroutine cf_dropin_stop
    Call cf_check(cf_destroy(cf), 'cf_destroy')
    cf = c_null_ptr
  End Subroutine cf_dropin_stop

  ! the device copies of the module scalars the next call reads
  Subroutine cf_dropin_push_scalars
    Call cf_check(cf_set_scalars(cf, t, dt, Int(rk_step,c_int), dPdx, dPdy), 'cf_set_scalars')
  End Subroutine cf_dropin_push_scalars

  Subroutine compute_dt
    Real(c_double) :: dt_
    Call cf_check(cf_compute_dt(cf, dt_), 'compute_dt')
    dt = dt_
  End Subroutine compute_dt

  Subroutine compute_eddy_viscosity(U_, V_, W_, avg_nu_t_, nu_t_)
    Real(Int64), Dimension(:,:,:), Intent(In)    :: U_, V_, W_
    Real(Int64), Dimension(:,:,:), Intent(InOut) :: avg_nu_t_, nu_t_
    Call cf_check(cf_compute_eddy_viscosity(cf), 'compute_eddy_viscosity')
  End Subroutine compute_eddy_viscosity

  Subroutine compute_wall_model(U_, V_, W_, nu_t_)
    Real(Int64), Dimension(:,:,:), Intent(In) :: U_, V_, W_, nu_t_
    Call cf_check(cf_compute_wall_model(cf), 'compute_wall_model')
  End Subroutine compute_wall_model

  Subroutine compute_rhs_u(U_, V_, W_, rhs_u)
    Real(Int64), Dimension(:,:,:), Intent(In)    :: U_, V_, W_
    Real(Int64), Dimension(:,:,:), Intent(InOut) :: rhs_u
    Call cf_check(cf_compute_rhs_u(cf, Int(rk_step,c_int)), 'compute_rhs_u')
  End Subroutine compute_rhs_u

  Subroutine compute_rhs_v(U_, V_, W_, rhs_v)
    Real(Int64), Dimension(:,:,:), Intent(In)    :: U_, V_, W_
    Real(Int64), Dimension(:,:,:), Intent(InOut) :: rhs_v
    Call cf_check(cf_compute_rhs_v(cf, Int(rk_step,c_int)), 'compute_rhs_v')
  End Subroutine compute_rhs_v

  Subroutine compute_rhs_w(U_, V_, W_, rhs_w)
    Real(Int64), Dimension(:,:,:), Intent(In)    :: U_, V_, W_
    Real(Int64), Dimension(:,:,:), Intent(InOut) :: rhs_w
    Call cf_check(cf_compute_rhs_w(cf, Int(rk_step,c_int)), 'compute_rhs_w')
  End Subroutine compute_rhs_w

  Subroutine apply_boundary_conditions
    Call cf_check(cf_apply_boundary_conditions(cf), 'apply_boundary_conditions')
  End Subroutine apply_boundary_conditions

  Subroutine compute_projection_step
    Call cf_check(cf_compute_projection_step(cf), 'compute_projection_step')
  End Subroutine compute_projection_step

  Subroutine compute_dPx_for_constant_mass_flow(U_, dPdx_)
    Real(Int64), Dimension(:,:,:), Intent(In) :: U_
    Real(Int64), Intent(Out) :: dPdx_
    Real(c_double) :: d
    Call cf_check(cf_compute_dPx_for_constant_mass_flow(cf, d), 'compute_dPx_for_constant_mass_flow')
    dPdx_ = d
  End Subroutine compute_dPx_for_constant_mass_flow

  Subroutine compute_dPy_for_constant_mass_flow(V_, dPdy_)
    Real(Int64), Dimension(:,:,:), Intent(In) :: V_
    Real(Int64), Intent(Out) :: dPdy_
    Real(c_double) :: d
    Call cf_check(cf_compute_dPy_for_constant_mass_flow(cf, d), 'compute_dPy_for_constant_mass_flow')
    dPdy_ = d
  End Subroutine compute_dPy_for_constant_mass_flow

  Subroutine compute_dPx_for_constant_Ucenterline(U_, dPdx_)
    Real(Int64), Dimension(:,:,:), Intent(In) :: U_
    Real(Int64), Intent(Out) :: dPdx_
    Real(c_double) :: d
    Call cf_check(cf_compute_dPx_for_constant_Ucenterline(cf, d), 'compute_dPx_for_constant_Ucenterline')
    dPdx_ = d
  End Subroutine compute_dPx_for_constant_Ucenterline

  Subroutine check_divergence(max_divergence)
    Real(Int64), Intent(Out) :: max_divergence
    Real(c_double) :: d, a
    Call cf_check(cf_check_divergence(cf, d, a), 'check_divergence')
    max_divergence = d
  End Subroutine check_divergence

  Subroutine compute_pressure
    Call cf_check(cf_compute_pressure(cf), 'compute_pressure')
  End Subroutine compute_pressure

  ! compute_time_step_RK3 (time_integration.f90:89-173) through the mirrors:
  ! the array lines U = Uo + dt*(...) become cf_rk_update, Uo = U becomes
  ! cf_save_old_state, and U = U + dPdx becomes cf_apply_mass_flow_correction
  ! (which also sets dPdx = dPdx/dt on the device)
  Subroutine compute_time_step_RK3
    Real(Int64) :: to
    Real(Int64), Parameter :: rk_t_(3) = (/ 8d0/15d0, 2d0/3d0, 1d0 /)
    Integer :: s
    Real(Int64) :: d, t_, dt_, dPdx_, dPdy_
    Integer(c_int) :: rk_

    to = t
    Call cf_check(cf_save_old_state(cf), 'cf_save_old_state')
    Do s = 1, 3
       rk_step = s
       Call cf_dropin_push_scalars
       Call compute_eddy_viscosity(U, V, W, avg_nu_t, nu_t)
       If ( s == 1 ) Then
          Call compute_wall_model(U, V, W, nu_t)
          Call compute_eddy_viscosity(U, V, W, avg_nu_t, nu_t)
       End If
       Call cf_check(cf_compute_rhs_u(cf, Int(s,c_int)), 'compute_rhs_u')
       Call cf_check(cf_compute_rhs_v(cf, Int(s,c_int)), 'compute_rhs_v')
       Call cf_check(cf_compute_rhs_w(cf, Int(s,c_int)), 'compute_rhs_w')
       Call cf_check(cf_rk_update(cf, Int(s,c_int)), 'cf_rk_update')
       t = to + rk_t_(s)*dt
       Call cf_dropin_push_scalars
       Call apply_boundary_conditions
       Call compute_projection_step
       Call apply_boundary_conditions
    End Do

    If ( x_mass_cte == 1 ) Then
       Call compute_dPx_for_constant_mass_flow(U, d)
       Call cf_check(cf_apply_mass_flow_correction(cf, 0_c_int, d), 'cf_apply_mass_flow_correction')
       Call apply_boundary_conditions
    Elseif ( x_mass_cte == 2 ) Then
       Call compute_dPx_for_constant_Ucenterline(U, d)
       Call cf_check(cf_apply_mass_flow_correction(cf, 0_c_int, d), 'cf_apply_mass_flow_correction')
       Call apply_boundary_conditions
    End If
    If ( y_mass_cte == 1 ) Then
       Call compute_dPy_for_constant_mass_flow(V, d)
       Call cf_check(cf_apply_mass_flow_correction(cf, 1_c_int, d), 'cf_apply_mass_flow_correction')
       Call apply_boundary_conditions
    End If
    ! the module scalars the corrections changed on the device (dPdx, dPdy)
    Call cf_check(cf_get_scalars(cf, t_, dt_, rk_, dPdx_, dPdy_), 'cf_get_scalars')
    dPdx = dPdx_
    dPdy = dPdy_
  End Subroutine compute_time_step_RK3

End Module channel_gpu_dropin
