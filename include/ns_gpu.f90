! ns_gpu.f90 -- ISO_C_BINDING interface to libns_gpu.so (include/ns_gpu.h).
!
! The reference's drivers (big_periodic_3D.f90, re_simulation*.f90) use this
! module to run the time-step loop body on a GB300.  Arrays are passed as
! explicit-shape, contiguous real(c_double) arrays in the reference's padded
! shapes: u(nx+1,ny+2,nz+2), v(nx+2,ny+1,nz+2), w(nx+2,ny+2,nz+1),
! p(nx+2,ny+2,nz+2).  Every function returns an integer(c_int) status (0 = ok).
module ns_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: NS_OK = 0, NS_ERR_SHAPE = 1, NS_ERR_CUDA = 2, NS_ERR_NONFINITE = 3, &
                               NS_ERR_TIMEOUT = 4, NS_ERR_UNSUPPORTED_BC = 5, NS_ERR_ARG = 6, NS_ERR_NOMEM = 7, &
                               NS_ERR_IO = 8
  integer(c_int), parameter :: NS_EULER = 0, NS_AB2 = 1, NS_AB2_CN = 2

  type, bind(C) :: ns_config
    integer(c_int) :: nx, ny, nz
    real(c_double) :: lx, ly, lz
    real(c_double) :: nu, dt
    integer(c_int) :: scheme
    integer(c_int) :: bc(3), pbc(3)
    integer(c_int) :: dp_flag, gauge
    real(c_double) :: mean_dp
    integer(c_int) :: cn_periodic_closure, use_graph
    integer(c_int) :: poisson_z
    integer(c_int) :: keep_sweeps   ! AB2-CN: keep u* after the x and y sweeps (per-sweep sub-block faces)
    integer(c_int) :: reserved(6)
  end type ns_config

  type, bind(C) :: ns_diag
    real(c_double) :: max_div, probe
    integer(c_long_long) :: steps_done
    integer(c_int) :: euler_start_pending, reserved
  end type ns_diag

  ! Batched tier (re_simulation_sub_tstep_interBC_combine.f90:415-811 for many sub-blocks at once).
  type, bind(C) :: ns_subdomain
    integer(c_int) :: x0, y0, z0          ! 1-based origin in the parent (idx_xu = x0 + (0..nx))
    integer(c_int) :: nx, ny, nz
    integer(c_int) :: sub_tstep, reserved
  end type ns_subdomain

  type, bind(C) :: ns_batch_config
    integer(c_int) :: scheme, bc, pbc, restart, n_slots, mode, use_graph
    real(c_double) :: nu, dt0, dx, dy, dz
    integer(c_int) :: grid(16)
    integer(c_int) :: using_ustar   ! 1: faces from the parent's u*; 0: from u (+ dt grad p_prev when dp_flag = 0)
    integer(c_int) :: dp_flag       ! 1: incremental pressure; 0: p = dp
    integer(c_int) :: reserved(6)
  end type ns_batch_config

  ! Per-kernel device time of ns_profile (the SYSTEM_CLOCK phases of big_periodic_3D.f90:328-569).
  type, bind(C) :: ns_kernel_time
    character(kind=c_char) :: name(32)
    real(c_double) :: ms
    integer(c_long_long) :: launches
  end type ns_kernel_time

  interface
    integer(c_int) function ns_config_default(cfg, nx, ny, nz) bind(C, name="ns_config_default")
      import :: c_int, ns_config
      type(ns_config), intent(out) :: cfg
      integer(c_int), value :: nx, ny, nz
    end function

    integer(c_int) function ns_create(cfg, h) bind(C, name="ns_create")
      import :: c_int, c_ptr, ns_config
      type(ns_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function

    integer(c_int) function ns_destroy(h) bind(C, name="ns_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    ! C strings: convert with ns_string (below)
    type(c_ptr) function ns_last_error(h) bind(C, name="ns_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function

    type(c_ptr) function ns_status_string(status) bind(C, name="ns_status_string")
      import :: c_ptr, c_int
      integer(c_int), value :: status
    end function

    type(c_ptr) function ns_version() bind(C, name="ns_version")
      import :: c_ptr
    end function

    ! the tile loader's bounded wait on a barrier no copy fills: NS_ERR_TIMEOUT is the expected answer
    integer(c_int) function ns_selftest_wait_timeout(limit_ms, waited_ms) bind(C, name="ns_selftest_wait_timeout")
      import :: c_int, c_double
      real(c_double), value :: limit_ms
      real(c_double), intent(out), optional :: waited_ms
    end function

    integer(c_int) function ns_set_stream(h, stream) bind(C, name="ns_set_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), value :: stream               ! cudaStream_t
    end function

    integer(c_int) function ns_synchronize(h) bind(C, name="ns_synchronize")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function ns_set_state(h, u, v, w, p, rx, ry, rz) bind(C, name="ns_set_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
      real(c_double), intent(in), optional :: rx(*), ry(*), rz(*)   ! absent -> NULL: Euler start
    end function

    integer(c_int) function ns_get_state(h, u, v, w, p, rx, ry, rz) bind(C, name="ns_get_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: u(*), v(*), w(*), p(*), rx(*), ry(*), rz(*)
    end function

    integer(c_int) function ns_set_faces(h, set, faces) bind(C, name="ns_set_faces")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: set
      type(c_ptr), intent(in) :: faces(24)   ! c_loc of bx_u_1 ... bz_p_nz, or c_null_ptr
    end function

    ! mean(dp_sub) of the DCT solve's singular mode (re_simulation_sub_tstep_interBC_combine.f90:766-768)
    integer(c_int) function ns_set_mean_dp(h, mean_dp) bind(C, name="ns_set_mean_dp")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), value :: mean_dp
    end function

    integer(c_int) function ns_step(h, nsteps) bind(C, name="ns_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function

    integer(c_int) function ns_step_host(h, u, v, w, p, rx, ry, rz, uo, vo, wo, po, rxo, ryo, rzo) &
        bind(C, name="ns_step_host")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*)
      real(c_double), intent(in), optional :: p(*), rx(*), ry(*), rz(*)
      real(c_double), intent(out), optional :: uo(*), vo(*), wo(*), po(*), rxo(*), ryo(*), rzo(*)
    end function

    integer(c_int) function ns_get_diag(h, d) bind(C, name="ns_get_diag")
      import :: c_int, c_ptr, ns_diag
      type(c_ptr), value :: h
      type(ns_diag), intent(out) :: d
    end function

    ! u_star, v_star, w_star, dp of the last step (the sources of the sub-block records, big_periodic_3D.f90:664-712)
    integer(c_int) function ns_get_stage(h, us, vs, ws, dp) bind(C, name="ns_get_stage")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: us(*), vs(*), ws(*), dp(*)
    end function

    ! u*, v*, w* after the x sweep and after the y sweep of the last AB2-CN step (cfg%keep_sweeps = 1)
    integer(c_int) function ns_get_sweeps(h, ux, vx, wx, uy, vy, wy) bind(C, name="ns_get_sweeps")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out), optional :: ux(*), vx(*), wx(*), uy(*), vy(*), wy(*)
    end function

    ! TGV (NS_functions.f90:18-50) on the GPU: call ns_tgv(xu, nx+1, yu, ny+2, nz+2, t, nu, u=u) etc.
    integer(c_int) function ns_tgv(x, nx, y, ny, nz, t, nu, u, v, w, p) bind(C, name="ns_tgv")
      import :: c_int, c_double
      integer(c_int), value :: nx, ny, nz
      real(c_double), intent(in) :: x(*), y(*)
      real(c_double), value :: t, nu
      real(c_double), intent(inout), optional :: u(*), v(*), w(*), p(*)
    end function

    integer(c_int) function ns_profile(h, nsteps, out, max_out, n_out) bind(C, name="ns_profile")
      import :: c_int, c_ptr, ns_kernel_time
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps, max_out
      type(ns_kernel_time), intent(out) :: out(*)
      integer(c_int), intent(out) :: n_out
    end function

    integer(c_int) function ns_launch_count(h, launches) bind(C, name="ns_launch_count")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), intent(out) :: launches
    end function

    ! The periodic FFT Poisson solve on caller-owned device arrays, allocating nothing
    integer(c_int) function ns_poisson_fft_noalloc(rhs_dev, dp_dev, nx, ny, nz, lx, ly, lz, stream) &
        bind(C, name="ns_poisson_fft_noalloc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: rhs_dev, dp_dev      ! device addresses (e.g. from a CUDA Fortran or C allocator)
      integer(c_int), value :: nx, ny, nz
      real(c_double), value :: lx, ly, lz
      type(c_ptr), value :: stream               ! cudaStream_t, or c_null_ptr
    end function

    integer(c_int) function ns_cal_conv(h, u, v, w, cx, cy, cz) bind(C, name="ns_cal_conv")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*)
      real(c_double), intent(out) :: cx(*), cy(*), cz(*)
    end function

    integer(c_int) function ns_cal_diff(h, u, v, w, dx, dy, dz) bind(C, name="ns_cal_diff")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*)
      real(c_double), intent(out) :: dx(*), dy(*), dz(*)
    end function

    integer(c_int) function ns_poisson(h, rhs, dp) bind(C, name="ns_poisson")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: rhs(*)
      real(c_double), intent(out) :: dp(*)
    end function

    integer(c_int) function ns_adi(h, us, vs, ws) bind(C, name="ns_adi")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: us(*), vs(*), ws(*)
    end function

    ! vel_bc_staggered (NS_functions.f90:213-310) with the session's bc and face set 0
    integer(c_int) function ns_vel_bc(h, us, vs, ws) bind(C, name="ns_vel_bc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(inout) :: us(*), vs(*), ws(*)
    end function

    ! gauge + correction (big_periodic_3D.f90:562-567): u = u_star - dt0*diff(dp,1,1)/dx ..., p = dp_flag*p + dp
    integer(c_int) function ns_correct(h, us, vs, ws, dp, u, v, w, p) bind(C, name="ns_correct")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: us(*), vs(*), ws(*), dp(*)
      real(c_double), intent(out) :: u(*), v(*), w(*)
      real(c_double), intent(inout) :: p(*)
    end function

    ! --- batched re-simulation --------------------------------------------------
    subroutine ns_batch_config_default(cfg) bind(C, name="ns_batch_config_default")
      import :: ns_batch_config
      type(ns_batch_config), intent(out) :: cfg
    end subroutine

    integer(c_int) function ns_batch_create(cfg, subs, n, b) bind(C, name="ns_batch_create")
      import :: c_int, c_ptr, ns_batch_config, ns_subdomain
      type(ns_batch_config), intent(in) :: cfg
      type(ns_subdomain), intent(in) :: subs(*)
      integer(c_int), value :: n
      type(c_ptr), intent(out) :: b
    end function

    integer(c_int) function ns_batch_destroy(b) bind(C, name="ns_batch_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
    end function

    type(c_ptr) function ns_batch_last_error(b) bind(C, name="ns_batch_last_error")
      import :: c_ptr
      type(c_ptr), value :: b
    end function

    integer(c_int) function ns_batch_set_stream(b, stream) bind(C, name="ns_batch_set_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: b, stream
    end function

    ! Initial sub-block state from host arrays (the u_sub ... groups read at
    ! re_simulation_sub_tstep_interBC_combine.f90:421-433)
    integer(c_int) function ns_batch_set_state(b, i, u, v, w, p, rx, ry, rz) bind(C, name="ns_batch_set_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: i                   ! 0-based subdomain index
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
      real(c_double), intent(in), optional :: rx(*), ry(*), rz(*)
    end function

    ! A snapshot from host faces (the records read at re_simulation_sub_tstep_interBC_combine.f90:455-504,
    ! turned into faces by get_velpr_bc): faces(k) = c_loc of the k-th get_velpr_bc output, or c_null_ptr
    integer(c_int) function ns_batch_set_snapshot(b, slot, t, i, faces, mean_dp) bind(C, name="ns_batch_set_snapshot")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: slot, i
      real(c_double), value :: t, mean_dp
      type(c_ptr), intent(in) :: faces(24)
    end function

    integer(c_int) function ns_batch_get_snapshot(b, slot, i, faces, mean_dp) bind(C, name="ns_batch_get_snapshot")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: slot, i
      type(c_ptr), intent(in) :: faces(24)         ! c_loc of the 24 output arrays, or c_null_ptr
      real(c_double), intent(out), optional :: mean_dp
    end function

    ! AB2-CN batches: the 18 per-sweep faces bx_u_1s ... bz_w_nzs (big_periodic_3D.f90:433-489)
    integer(c_int) function ns_batch_set_sweep_faces(b, slot, i, faces) bind(C, name="ns_batch_set_sweep_faces")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: slot, i
      type(c_ptr), intent(in) :: faces(18)         ! c_loc of each array, or c_null_ptr (zero)
    end function

    integer(c_int) function ns_batch_get_sweep_faces(b, slot, i, faces) bind(C, name="ns_batch_get_sweep_faces")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: slot, i
      type(c_ptr), intent(in) :: faces(18)
    end function

    integer(c_int) function ns_batch_launch_count(b, launches) bind(C, name="ns_batch_launch_count")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: b
      integer(c_long_long), intent(out) :: launches
    end function

    integer(c_int) function ns_batch_autotune(b, reps) bind(C, name="ns_batch_autotune")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: reps
    end function

    integer(c_int) function ns_batch_profile(b, reps, ms_per_stage) bind(C, name="ns_batch_profile")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: reps
      real(c_double), intent(out) :: ms_per_stage(16)
    end function

    integer(c_int) function ns_batch_get_config(b, cfg) bind(C, name="ns_batch_get_config")
      import :: c_int, c_ptr, ns_batch_config
      type(c_ptr), value :: b
      type(ns_batch_config), intent(out) :: cfg
    end function

    ! interp1(knots, y, t, 'spline') weights on the 6-knot window (sub_tstep_BC_combined_interpolation.m:53-64)
    integer(c_int) function ns_spline_weights(knots, n_knots, t, first, w) bind(C, name="ns_spline_weights")
      import :: c_int, c_double
      real(c_double), intent(in) :: knots(*)
      integer(c_int), value :: n_knots
      real(c_double), value :: t
      integer(c_int), intent(out) :: first         ! 0-based index of the window's first knot
      real(c_double), intent(out) :: w(6)
    end function

    integer(c_int) function ns_batch_init_from_parent(b, parent) bind(C, name="ns_batch_init_from_parent")
      import :: c_int, c_ptr
      type(c_ptr), value :: b, parent
    end function

    integer(c_int) function ns_batch_capture(b, parent, slot, t) bind(C, name="ns_batch_capture")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b, parent
      integer(c_int), value :: slot
      real(c_double), value :: t
    end function

    integer(c_int) function ns_batch_advance(b, t0) bind(C, name="ns_batch_advance")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      real(c_double), value :: t0
    end function

    integer(c_int) function ns_batch_get_state(b, i, u, v, w, p, rx, ry, rz) bind(C, name="ns_batch_get_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: i                   ! 0-based subdomain index
      real(c_double), intent(out), optional :: u(*), v(*), w(*), p(*), rx(*), ry(*), rz(*)
    end function

    integer(c_int) function ns_batch_max_div(b, i, max_div) bind(C, name="ns_batch_max_div")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b
      integer(c_int), value :: i
      real(c_double), intent(out) :: max_div
    end function

    ! --- re-simulation error metrics and err_file writer (:813-834, :913-931) ----
    integer(c_int) function ns_error_metrics(h, u_sub, v_sub, w_sub, p_sub, out) bind(C, name="ns_error_metrics")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u_sub(*), v_sub(*), w_sub(*), p_sub(*)
      real(c_double), intent(out) :: out(12)     ! rms_vel(1:4), err_vel(1:8)
    end function

    integer(c_int) function ns_batch_error_metrics(b, parent, out) bind(C, name="ns_batch_error_metrics")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: b, parent
      real(c_double), intent(out) :: out(*)      ! 12 per subdomain
    end function

    integer(c_int) function ns_write_err_csv(path, kind, nrows, rows) bind(C, name="ns_write_err_csv")
      import :: c_int, c_char, c_double
      character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
      integer(c_int), value :: kind, nrows            ! kind 0: err_vel (8 columns), 1: rms_vel (4)
      real(c_double), intent(in) :: rows(*)           ! row-major: rows(col + ncol*j)
    end function

    integer(c_int) function ns_spectrum(h, k, E, count, props) bind(C, name="ns_spectrum")
      import :: c_int, c_ptr, c_double, c_long_long
      type(c_ptr), value :: h
      real(c_double), intent(out) :: k(*), E(*)         ! nx/2 shells (PowerSpec.m)
      integer(c_long_long), intent(out) :: count(*)
      real(c_double), intent(out) :: props(10)          ! SpecProp.m, KolmoScale.m, lambda, Re_lambda
    end function

    ! --- discrete adjoint (no counterpart in the reference) -----------------------
    integer(c_int) function ns_adj_forward(h, nsteps, ckpt_every) bind(C, name="ns_adj_forward")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps, ckpt_every
    end function

    integer(c_int) function ns_adj_backward(h, gu, gv, gw, du0, dv0, dw0, dhx, dhy, dhz) &
        bind(C, name="ns_adj_backward")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: gu(*), gv(*), gw(*)          ! dJ/du(T), dJ/dv(T), dJ/dw(T)
      real(c_double), intent(out) :: du0(*), dv0(*), dw0(*)      ! dJ/du(0) ...
      real(c_double), intent(out), optional :: dhx(*), dhy(*), dhz(*)
    end function

    ! --- HDF5 files of the reference without libhdf5 (big_periodic_3D.f90:593-726) ---
    ! Paths and names are NUL-terminated (trim(name)//c_null_char).  dims in Fortran order.
    integer(c_int) function ns_h5_create(path, overwrite, f) bind(C, name="ns_h5_create")       ! h5fcreate_f
      import :: c_int, c_ptr, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: overwrite
      type(c_ptr), intent(out) :: f
    end function

    integer(c_int) function ns_h5_open(path, writable, f) bind(C, name="ns_h5_open")           ! h5fopen_f
      import :: c_int, c_ptr, c_char
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: writable
      type(c_ptr), intent(out) :: f
    end function

    integer(c_int) function ns_h5_flush(f) bind(C, name="ns_h5_flush")
      import :: c_int, c_ptr
      type(c_ptr), value :: f
    end function

    integer(c_int) function ns_h5_close(f) bind(C, name="ns_h5_close")                        ! h5fclose_f
      import :: c_int, c_ptr
      type(c_ptr), value :: f
    end function

    type(c_ptr) function ns_h5_last_error(f) bind(C, name="ns_h5_last_error")
      import :: c_ptr
      type(c_ptr), value :: f
    end function

    integer(c_int) function ns_h5_group(f, path) bind(C, name="ns_h5_group")                  ! h5gcreate_f
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: path(*)
    end function

    integer(c_int) function ns_h5_attr_int(f, obj, name, value) bind(C, name="ns_h5_attr_int")  ! h5ltset_attribute_int_f
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*)
      integer(c_int), value :: value
    end function

    integer(c_int) function ns_h5_attr_double(f, obj, name, value) bind(C, name="ns_h5_attr_double")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*)
      real(c_double), value :: value
    end function

    integer(c_int) function ns_h5_attr_string(f, obj, name, value) bind(C, name="ns_h5_attr_string")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*), value(*)
    end function

    integer(c_int) function ns_h5_write_double(f, path, rank, dims, data) bind(C, name="ns_h5_write_double")
      import :: c_int, c_ptr, c_char, c_double, c_long_long                           ! h5ltmake_dataset_double_f
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: rank
      integer(c_long_long), intent(in) :: dims(*)
      real(c_double), intent(in) :: data(*)
    end function

    integer(c_int) function ns_h5_dims(f, path, rank, dims) bind(C, name="ns_h5_dims")        ! h5ltget_dataset_info_f
      import :: c_int, c_ptr, c_char, c_long_long
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), intent(out) :: rank
      integer(c_long_long), intent(out) :: dims(32)
    end function

    integer(c_int) function ns_h5_read_double(f, path, rank, dims, out) bind(C, name="ns_h5_read_double")
      import :: c_int, c_ptr, c_char, c_double, c_long_long                           ! h5ltread_dataset_double_f
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: rank
      integer(c_long_long), intent(in) :: dims(*)
      real(c_double), intent(out) :: out(*)
    end function

    integer(c_int) function ns_h5_get_attr_int(f, obj, name, value) bind(C, name="ns_h5_get_attr_int")
      import :: c_int, c_ptr, c_char, c_long_long
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*)
      integer(c_long_long), intent(out) :: value
    end function

    integer(c_int) function ns_h5_get_attr_double(f, obj, name, value) bind(C, name="ns_h5_get_attr_double")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*)
      real(c_double), intent(out) :: value
    end function

    integer(c_int) function ns_h5_get_attr_string(f, obj, name, buf, buflen) bind(C, name="ns_h5_get_attr_string")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: obj(*), name(*)
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_int), value :: buflen
    end function

    integer(c_int) function ns_h5_members(f, group, buf, buflen, needed) bind(C, name="ns_h5_members")
      import :: c_int, c_ptr, c_char, c_long_long
      type(c_ptr), value :: f
      character(kind=c_char), intent(in) :: group(*)
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_long_long), value :: buflen
      integer(c_long_long), intent(out) :: needed
    end function

    ! The session's state as a snapshot in the layout of big_periodic_3D.f90:630-651
    ! (no libhdf5 needed), and the restart of :309-324 from such a file.
    integer(c_int) function ns_h5_write_state(h, path, time, time_step, overwrite) bind(C, name="ns_h5_write_state")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated
      real(c_double), value :: time
      integer(c_int), value :: time_step, overwrite
    end function

    integer(c_int) function ns_h5_read_state(h, path, time, time_step) bind(C, name="ns_h5_read_state")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: h
      character(kind=c_char), intent(in) :: path(*)
      real(c_double), intent(out), optional :: time
      integer(c_int), intent(out), optional :: time_step
    end function
  end interface

contains

  ! A NUL-terminated C string (ns_last_error, ns_status_string, ...) as a Fortran string.
  function ns_string(p) result(s)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: s
    character(kind=c_char), pointer :: c(:)
    integer :: n
    interface
      integer(c_size_t) function c_strlen(q) bind(C, name="strlen")
        import :: c_size_t, c_ptr
        type(c_ptr), value :: q
      end function
    end interface
    if (.not. c_associated(p)) then
      s = ""
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, c, [n])
    allocate(character(len=n) :: s)
    s = transfer(c(1:n), s)
  end function ns_string
end module ns_gpu
