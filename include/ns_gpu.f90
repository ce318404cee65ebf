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
    integer(c_int) :: reserved(7)
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
    integer(c_int) :: grid(16), reserved(8)
  end type ns_batch_config

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
end module ns_gpu
