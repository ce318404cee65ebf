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
                               NS_ERR_TIMEOUT = 4, NS_ERR_UNSUPPORTED_BC = 5, NS_ERR_ARG = 6, NS_ERR_NOMEM = 7
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
    integer(c_int) :: reserved(8)
  end type ns_config

  type, bind(C) :: ns_diag
    real(c_double) :: max_div, probe
    integer(c_long_long) :: steps_done
    integer(c_int) :: euler_start_pending, reserved
  end type ns_diag

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
  end interface
end module ns_gpu
