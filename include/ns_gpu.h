/*
 * ns_gpu.h -- C ABI of libns_gpu.so, the GB300 (sm_103a) FP64 staggered-grid
 * incompressible Navier-Stokes step.
 *
 * This is the drop-in boundary for the time-step loop body of the reference
 * (zzwz02/NS_3D_Staggered_dp):
 *   big_periodic_3D.f90:326-571                       (periodic step)
 *   re_simulation_sub_tstep_interBC_combine.f90:438-804 (sub-block step)
 * and for the NS_functions.f90 / FD_functions.f90 routines it calls.  The
 * Fortran drivers bind it through ISO_C_BINDING (include/ns_gpu.f90).
 *
 * Conventions
 *  - All arrays crossing the boundary are FP64, column-major (Fortran order),
 *    in the reference's exact padded shapes:
 *        u (nx+1, ny+2, nz+2)   v (nx+2, ny+1, nz+2)   w (nx+2, ny+2, nz+1)
 *        p (nx+2, ny+2, nz+2)   rhs_?_previous: same as u / v / w
 *    Pointers are host pointers unless the name ends in _dev.
 *  - Every call returns an int status (NS_OK = 0).  Nothing exits, aborts or
 *    traps; ns_last_error() describes the last failure of a handle.
 *  - One handle owns its device buffers and one CUDA stream.  A handle must
 *    not be used by two host threads at once.  Host pointers are never
 *    retained after a call returns.
 *  - BC codes (NS_functions.f90:219-220): 1 periodic, 2 Dirichlet on the
 *    wall (cell face), 3 Neumann on the wall, 4 Dirichlet on the ghost cell.
 */
#ifndef NS_GPU_H
#define NS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  NS_OK = 0,
  NS_ERR_SHAPE = 1,          /* unsupported / inconsistent grid size            */
  NS_ERR_CUDA = 2,           /* a CUDA runtime call failed                      */
  NS_ERR_NONFINITE = 3,      /* NaN/Inf found by a checked call                 */
  NS_ERR_TIMEOUT = 4,        /* a bounded device wait ran out: the predictor's
                                tile loader gave up on an mbarrier (ns_get_diag
                                reports it; the state is then invalid)           */
  NS_ERR_UNSUPPORTED_BC = 5, /* bc/pbc/scheme combination the step cannot run   */
  NS_ERR_ARG = 6,            /* NULL or out-of-range argument                   */
  NS_ERR_NOMEM = 7,          /* device (or host staging) allocation failed      */
  NS_ERR_IO = 8              /* a file could not be read or written, or is not
                                of the HDF5 subset the ns_h5_* calls handle      */
};

/* Time schemes (big_periodic_3D.f90:350-490). */
enum { NS_EULER = 0, NS_AB2 = 1, NS_AB2_CN = 2 };

/* Boundary-condition codes. */
enum { NS_BC_PERIODIC = 1, NS_BC_DIRICHLET = 2, NS_BC_NEUMANN = 3, NS_BC_GHOST = 4 };

/*
 * Step configuration: the compile-time parameters of the reference drivers
 * (big_periodic_3D.f90:9-13,104-108; re_simulation_sub_tstep_interBC_combine.f90:100-112).
 */
typedef struct ns_config {
  int nx, ny, nz;       /* interior cells per axis                                 */
  double lx, ly, lz;    /* domain lengths; dx = lx/nx etc.                         */
  double nu;            /* kinematic viscosity                                     */
  double dt;            /* time step (dt0)                                         */
  int scheme;           /* NS_EULER, NS_AB2, NS_AB2_CN                             */
  int bc[3];            /* velocity BC per axis: 1, 2 or 4                         */
  int pbc[3];           /* pressure BC per axis: 1, 2, 3 or 4                      */
  int dp_flag;          /* 0: p = dp; 1: incremental (p += dp, -dt*grad p in u*)   */
  int gauge;            /* 1: dp -= dp(1,1,1) after the solve (big_periodic_3D.f90:562) */
  double mean_dp;       /* mean imposed on the singular mode (NS_functions.f90:1576) */
  int cn_periodic_closure; /* 0: reference closure of the periodic normal-component
                              CN row, A(1,n+1) (NS_functions.f90:1273); 1: A(1,n)   */
  int use_graph;        /* 1: replay each step from a captured CUDA graph          */
  int poisson_z;        /* all-periodic boxes, the z stage of the Poisson solve:
                           0: cyclic tridiagonal line solves (Sherman-Morrison),
                           1: z FFT, divide by the eigenvalue, z IFFT            */
  int keep_sweeps;      /* AB2-CN: 1 keeps u*, v*, w* after the x and the y sweep
                           of the last step readable (3 more fields): the
                           per-sweep faces that a parent run records for its
                           sub-blocks (big_periodic_3D.f90:433-489), read by
                           ns_batch_capture and ns_get_sweeps                 */
  int reserved[6];
} ns_config;

/* Diagnostics (big_periodic_3D.f90:572-579). */
typedef struct ns_diag {
  double max_div;          /* max |div u| over the interior                       */
  double probe;            /* u(nx/2, ny/2, nz/2) (Fortran indices)                */
  long long steps_done;    /* steps taken since ns_set_state                       */
  int euler_start_pending; /* 1 if the next step is the Euler start of AB2/AB2-CN  */
  int reserved;
} ns_diag;

typedef struct ns_handle ns_handle;

/* ------------------------------------------------------------------------
 * Session tier: state resident on the GPU between steps.
 * ------------------------------------------------------------------------ */

/* Fill *cfg with the big_periodic_3D defaults for an nx*ny*nz periodic box on
 * [0,2pi]^3 (big_periodic_3D.f90:10-13,104-108). */
int ns_config_default(ns_config* cfg, int nx, int ny, int nz);

/* Create a session: device buffers, stream, CN factors, transform plans.
 * Replaces the driver set-up of big_periodic_3D.f90:158-256 and
 * re_simulation_sub_tstep_interBC_combine.f90:200-354. */
int ns_create(const ns_config* cfg, ns_handle** out);
int ns_destroy(ns_handle* h);
const char* ns_last_error(const ns_handle* h);
const char* ns_status_string(int status);

/* Use an external CUDA stream (cudaStream_t) instead of the handle's own. */
int ns_set_stream(ns_handle* h, void* cuda_stream);
int ns_synchronize(ns_handle* h);

/* Copy the state in.  u, v, w, p are required; the three rhs_?_previous may be
 * NULL, in which case the AB2 history is zero and the next step is the Euler
 * start (big_periodic_3D.f90:296-303 init read, :309-324 restart read). */
int ns_set_state(ns_handle* h, const double* u, const double* v, const double* w, const double* p,
                 const double* rhs_x_prev, const double* rhs_y_prev, const double* rhs_z_prev);

/* Copy the state out (any pointer may be NULL to skip that field).  History
 * entries outside the interior ranges are returned as zero. */
int ns_get_state(ns_handle* h, double* u, double* v, double* w, double* p,
                 double* rhs_x_prev, double* rhs_y_prev, double* rhs_z_prev);

/* One step of a driver that keeps its state on the host: the state in, one
 * step, the state out, in one call (the loop body of
 * big_periodic_3D.f90:326-567 with host arrays).  Transfers run on a copy
 * stream and overlap the step: the AB2 history is copied out while the ADI
 * sweeps and the Poisson solve run.  u, v, w are required; p is read only
 * with dp_flag = 1 (with dp_flag = 0 the step overwrites p with dp); NULL
 * history inputs mean the Euler start.  Any output may be NULL.  The output
 * arrays may be the input arrays.  Equivalent to ns_set_state + ns_step(h, 1)
 * + ns_get_state, bit for bit. */
int ns_step_host(ns_handle* h, const double* u, const double* v, const double* w, const double* p,
                 const double* rhs_x_prev, const double* rhs_y_prev, const double* rhs_z_prev, double* u_out,
                 double* v_out, double* w_out, double* p_out, double* rhs_x_out, double* rhs_y_out, double* rhs_z_out);

/* Boundary faces, in the reference shapes and order of get_velpr_bc's
 * outputs (NS_functions.f90:414-420):
 *   bx_u_1, bx_u_nx, by_u_1, by_u_ny, bz_u_1, bz_u_nz,
 *   bx_v_1, bx_v_nx, by_v_1, by_v_ny, bz_v_1, bz_v_nz,
 *   bx_w_1, bx_w_nx, by_w_1, by_w_ny, bz_w_1, bz_w_nz,
 *   bx_p_1, bx_p_nx, by_p_1, by_p_ny, bz_p_1, bz_p_nz.
 * set == 0: the faces used by vel_bc_staggered and the pressure BC;
 * set == 1, 2, 3: the faces of the x, y, z AB2-CN sweep
 * (vel_bc_staggered_CN2, big_periodic_3D.f90:425,437,462).  A NULL entry
 * means zero.  Faces persist until set again.  The copy is stream-ordered
 * (the next ns_step sees the new faces) and the call returns without waiting
 * for the device; the host arrays may be reused at once. */
int ns_set_faces(ns_handle* h, int set, const double* const faces[24]);

/* The mean imposed on the singular mode of a DCT/DST pressure solve from the
 * next step on (the mean(dp_sub) argument of DCT_poisson_solver,
 * re_simulation_sub_tstep_interBC_combine.f90:766-768, which a re-simulation
 * driver changes every step).  Stream-ordered like ns_set_faces; boxes
 * without a singular mode ignore it. */
int ns_set_mean_dp(ns_handle* h, double mean_dp);

/* Advance nsteps steps (the loop body of big_periodic_3D.f90:326-567). */
int ns_step(ns_handle* h, int nsteps);

/* max|div u| and the probe value of the current state (a synchronous call). */
int ns_get_diag(ns_handle* h, ns_diag* d);

/* The intermediate fields of the last step, in the reference shapes: u*, v*,
 * w* (after the ADI sweeps with AB2-CN) and dp, gauge-shifted as
 * big_periodic_3D.f90:562 shifts it (dp - dp(1,1,1) when cfg.gauge).  These
 * are the u_star_sub, ..., dp_sub that the reference's parent run records
 * for its sub-blocks (big_periodic_3D.f90:664-712).  Any pointer may be
 * NULL.  Valid after ns_step; a synchronous call. */
int ns_get_stage(ns_handle* h, double* u_star, double* v_star, double* w_star, double* dp);

/* u*, v*, w* of the last AB2-CN step after the x sweep (ux, vx, wx) and after
 * the y sweep (uy, vy, wy), reference shapes, any pointer NULL to skip: the
 * fields from which big_periodic_3D.f90:433-458 takes the per-sweep faces
 * bx_?_1s ... by_?_nys.  Needs cfg.keep_sweeps = 1; a synchronous call. */
int ns_get_sweeps(ns_handle* h, double* ux, double* vx, double* wx, double* uy, double* vy, double* wy);

/* TGV (NS_functions.f90:18-50): the 2D Taylor-Green vortex at time t on the
 * tensor grid x(1:nx) x y(1:ny) x nz planes, computed on the GPU:
 *   u(i,j,:) =  cos(x_i) sin(y_j) e,   v(i,j,:) = -sin(x_i) cos(y_j) e,
 *   p(i,j,:) = -(cos(2 x_i) + cos(2 y_j)) e^2 / 4,   e = exp(-2 nu t).
 * u, v, p are host arrays (nx, ny, nz) in Fortran order; any may be NULL (the
 * reference's absent optional arguments).  w is accepted and, as in the
 * reference, left untouched.  The drivers call it once per staggered field
 * with that field's coordinates (xu, yu for u; xv, yv for v; xp, yp for p). */
int ns_tgv(const double* x, int nx, const double* y, int ny, int nz, double t, double nu, double* u, double* v,
           double* w, double* p);

/* ------------------------------------------------------------------------
 * Routine tier: one reference routine per call, host arrays in and out,
 * using the handle's configuration for shapes, bc codes and spacings.
 * ------------------------------------------------------------------------ */

/* cal_conv (NS_functions.f90:53-158): conv_? in the reference's shapes
 * ((nx or nx-1), ny, nz) etc. per bc. */
int ns_cal_conv(ns_handle* h, const double* u, const double* v, const double* w,
                double* conv_x, double* conv_y, double* conv_z);

/* cal_diff (NS_functions.f90:161-210): Laplacian, same shapes as cal_conv. */
int ns_cal_diff(ns_handle* h, const double* u, const double* v, const double* w,
                double* diff_x, double* diff_y, double* diff_z);

/* Pressure Poisson solve: rhs (nx, ny, nz), already BC-modified as by
 * pr_bc_staggered_modify_rhs, -> dp (nx+2, ny+2, nz+2) with ghosts filled by
 * pr_bc_staggered using the set-0 faces.  FFT for all-periodic pbc
 * (big_periodic_3D.f90:526-543), DCT/DST otherwise (NS_functions.f90:1505-1630). */
int ns_poisson(ns_handle* h, const double* rhs, double* dp);

/* The three AB2-CN ADI sweeps on u*, v*, w* in place, with the set-1..3 faces
 * (big_periodic_3D.f90:425-489; re_simulation_sub_tstep_interBC_combine.f90:656-701). */
int ns_adi(ns_handle* h, double* u_star, double* v_star, double* w_star);
/* vel_bc_staggered (NS_functions.f90:213-310) on host u*, v*, w* in place:
 * the ghost and face values of the session's bc codes and its face set 0
 * (ns_set_faces).  The session's state is untouched. */
int ns_vel_bc(ns_handle* h, double* u_star, double* v_star, double* w_star);
/* Gauge and correction (big_periodic_3D.f90:562-567): with cfg.gauge,
 * dp -= dp(1,1,1); then u = u* - dt diff(dp)/dx (likewise v, w over the full
 * padded arrays) and p = dp_flag p + dp.  dp and p are p-shaped; p is read
 * (with dp_flag = 1) and written.  The session's state is untouched. */
int ns_correct(ns_handle* h, const double* u_star, const double* v_star, const double* w_star, const double* dp,
               double* u, double* v, double* w, double* p);

/* The periodic FFT pressure Poisson solve of ns_poisson without any device
 * allocation.  No counterpart in the reference: it serves callers that must
 * not allocate device memory (hosts whose device memory is owned by another
 * allocator or reserved up front, real-time loops that cannot take an
 * allocation's device synchronisation).
 *   rhs_dev: device array (nx, ny, nz), Fortran order, 16-byte aligned,
 *            already BC-modified (periodic: none);
 *   dp_dev : device array (nx+2, ny+2, nz+2), Fortran order, 8-byte aligned;
 *            the interior is the solution (zero mean) and the ghosts are
 *            the periodic copies;
 *   stream : cudaStream_t the work is enqueued on (NULL: legacy stream).
 * All scratch (half spectrum, twiddles, 1/lambda; 4 MiB) is one static
 * device array held by every device that loads the library.  Grids are
 * limited to powers of two in [16, 64] per axis (NS_ERR_SHAPE otherwise).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), keeps it for the life of the process, and should
 * come before any stream capture; a device reset after it is not supported.
 * A CUDA error already pending on the calling thread is left in place and
 * the call returns NS_ERR_CUDA without launching.  Calls share the array:
 * calls that overlap on the GPU race. */
int ns_poisson_fft_noalloc(const double* rhs_dev, double* dp_dev, int nx, int ny, int nz, double lx, double ly,
                           double lz, void* stream);

/* ------------------------------------------------------------------------
 * Tracing (the per-phase SYSTEM_CLOCK prints of big_periodic_3D.f90:328-569).
 * ------------------------------------------------------------------------ */
typedef struct ns_kernel_time {
  char name[32];        /* kernel (phase) name: predict, adi_x, fft_z_solve, ... */
  double ms;            /* summed device time between CUDA events              */
  long long launches;   /* marks recorded under this name                      */
} ns_kernel_time;

/* Run nsteps steps with a CUDA event after every kernel and return the
 * per-kernel device time (eager launches, not the captured graph). */
int ns_profile(ns_handle* h, int nsteps, ns_kernel_time* out, int max_out, int* n_out);

/* Number of kernels this handle has launched (graph replays included). */
int ns_launch_count(const ns_handle* h, long long* launches);

/* Version string of the library build. */
const char* ns_version(void);

/* Self-test of failure detection: the predictor's TMA tile loader waits on
 * each ring slot's mbarrier with a bounded wait (NS_ERR_TIMEOUT through
 * ns_get_diag when it gives up).  This call runs that same wait code on a
 * barrier armed for bytes that no copy delivers, with a limit of limit_ms
 * (0 < limit_ms <= 1000), and returns what the wait reported: NS_ERR_TIMEOUT
 * is the expected answer (NS_OK would mean a wait that cannot end did);
 * *waited_ms (may be NULL) receives the time the wait took.  Nothing is in
 * flight when it gives up, and the device stays usable. */
int ns_selftest_wait_timeout(double limit_ms, double* waited_ms);

/* ------------------------------------------------------------------------
 * Batched tier: re-simulation of many sub-blocks of a parent run at once.
 *
 * Each subdomain is the reference's re-simulated sub-block
 * (re_simulation_sub_tstep_interBC_combine.f90:415-811): wall velocity BCs
 * from the parent's u* (using_Ustar), pressure BCs from the parent's dp,
 * dp_flag = 1, the DCT pressure solve with the mean of the parent's dp, and
 * sub_tstep sub-steps over the first parent interval with the AB2 history
 * saved after the first sub-step and restored after the last (:443-454,
 * :602-612).  Boundary values are taken from snapshots of the parent
 * (big_periodic_3D.f90:664-712) and interpolated in time as MATLAB's
 * interp1(..., 'spline') over a window of 6 snapshots
 * (sub_tstep_BC_combined_interpolation.m:53-64).  All subdomains advance
 * together: every stage of the step is one persistent kernel over a work
 * queue of (subdomain, tile) items.
 * ------------------------------------------------------------------------ */
typedef struct ns_batch ns_batch;

/* One sub-block: origin in the parent (1-based, idx_xu = x0 + (0..nx) etc.,
 * big_periodic_3D.f90:20-25), cells, sub-steps in the first interval. */
typedef struct ns_subdomain {
  int x0, y0, z0;
  int nx, ny, nz;       /* nx even; ny <= 128; nz <= 256                       */
  int sub_tstep;        /* >= 1 (re_simulation_sub_tstep_interBC_combine.f90:104) */
  int reserved;
} ns_subdomain;

typedef struct ns_batch_config {
  int scheme;           /* NS_EULER, NS_AB2 or NS_AB2_CN (sub_tstep > 1 needs
                           NS_AB2; NS_AB2_CN needs sub_tstep = 1, as the
                           reference, :356-359, and the u* faces of every ADI
                           sweep: a parent created with keep_sweeps = 1)      */
  int bc;               /* velocity bc of every subdomain face: 2 or 4           */
  int pbc;              /* pressure bc: 2, 3 or 4                                */
  int restart;          /* 1: AB2 from the first step with the parent's history  */
  int n_slots;          /* parent snapshots kept on the device                   */
  int mode;             /* 0: batched launches; 1: one launch per subdomain and
                           stage (the per-subdomain loop, for comparison)        */
  int use_graph;        /* 1: capture each stage sequence in a CUDA graph        */
  double nu, dt0;       /* viscosity and the parent time step                    */
  double dx, dy, dz;    /* grid spacing (the parent's)                           */
  int grid[16];         /* persistent CTAs per stage kernel (0: one wave);
                           set by ns_batch_autotune                              */
  int using_ustar;      /* 1: velocity faces from the parent's u* (the default,
                           re_simulation_sub_tstep_interBC_combine.f90:105);
                           0: from the parent's u, plus dt0 * grad(p_previous)
                           when dp_flag = 0 (get_velpr_bc, NS_functions.f90:
                           434-444); needs sub_tstep = 1 (:360-363)           */
  int dp_flag;          /* 1: incremental pressure (the default, :104): the
                           predictor subtracts dt grad p, p += dp, pressure
                           faces and mean from the parent's dp;
                           0: p = dp, pressure faces and mean from the
                           parent's p (dp_sub = p_sub, :506-508)              */
  int reserved[6];
} ns_batch_config;

void ns_batch_config_default(ns_batch_config* c);
int ns_batch_create(const ns_batch_config* cfg, const ns_subdomain* subs, int n, ns_batch** out);
int ns_batch_destroy(ns_batch* b);
const char* ns_batch_last_error(const ns_batch* b);
/* cudaStream_t to enqueue on (NULL: the batch's own stream). */
int ns_batch_set_stream(ns_batch* b, void* stream);

/* Initial states: every subdomain's u, v, w, p and AB2 history from the
 * parent session's device state (re_simulation_sub_tstep_interBC_combine.f90:421-433). */
int ns_batch_init_from_parent(ns_batch* b, const ns_handle* parent);
/* Host state of subdomain i (reference shapes of the subdomain; history may be NULL). */
int ns_batch_set_state(ns_batch* b, int i, const double* u, const double* v, const double* w, const double* p,
                       const double* hx, const double* hy, const double* hz);
int ns_batch_get_state(ns_batch* b, int i, double* u, double* v, double* w, double* p, double* hx, double* hy,
                       double* hz);

/* Snapshot slot `slot` at parent time t: the 24 face arrays of every
 * subdomain (get_velpr_bc, NS_functions.f90:414-510, and get_pr_bc :514-562,
 * on the parent's sub-block, u_sub = u(idx_xu, idx_yu, idx_zu),
 * big_periodic_3D.f90:20-25) and the mean of the pressure source over each
 * subdomain's interior (the mean_dp of the DCT solve,
 * re_simulation_sub_tstep_interBC_combine.f90:766-768).  The sources follow
 * the batch's using_ustar / dp_flag:
 *   velocity: the parent's last u* (using_ustar = 1) or its current u
 *             (using_ustar = 0; with dp_flag = 0 plus dt0 * diff(p_prev) / h,
 *             p_prev = the parent's p at the previous ns_batch_capture of
 *             this batch, or its current p at the first one);
 *   pressure: the parent's last dp, gauge-shifted as the step shifts it
 *             (dp_flag = 1), or its current p (dp_flag = 0).
 * The arithmetic is the reference's, operation for operation, so the faces
 * equal get_velpr_bc of the same parent arrays bit for bit. */
int ns_batch_capture(ns_batch* b, const ns_handle* parent, int slot, double t);
/* The same snapshot from host data for subdomain i: faces in get_velpr_bc
 * order (ns_set_faces), NULL entries zero. */
int ns_batch_set_snapshot(ns_batch* b, int slot, double t, int i, const double* const faces[24], double mean_dp);
/* Read back snapshot slot `slot` of subdomain i (the inverse of
 * ns_batch_set_snapshot): the 24 faces in get_velpr_bc order and shapes
 * (NULL entries skipped) and the mean (may be NULL).  These are the
 * boundary arrays the reference's parent run writes to its sub-block record
 * files (big_periodic_3D.f90:664-712). */
int ns_batch_get_snapshot(ns_batch* b, int slot, int i, double* const faces[24], double* mean_dp);
/* AB2-CN batches: the 18 per-sweep faces of snapshot slot `slot` of
 * subdomain i, which the sub-block's x, y and z sweeps take as their BC rows
 * (vel_bc_staggered_CN2, NS_functions.f90:313-410).  Order and shapes are the
 * reference's records of big_periodic_3D.f90:433-489: bx_u_1s, bx_u_nxs,
 * bx_v_1s, bx_v_nxs, bx_w_1s, bx_w_nxs, by_u_1s, ..., by_w_nys, bz_u_1s, ...,
 * bz_w_nzs, each shaped as the get_velpr_bc face of the same name.
 * ns_batch_capture fills them from the parent; _set (after the slot's
 * ns_batch_set_snapshot; NULL entries zero) and _get move them to and from
 * host arrays. */
int ns_batch_set_sweep_faces(ns_batch* b, int slot, int i, const double* const faces[18]);
int ns_batch_get_sweep_faces(ns_batch* b, int slot, int i, double* const faces[18]);

/* Advance every subdomain over one parent interval [t0, t0 + dt0]: the
 * first call takes sub_tstep sub-steps, later calls one step. */
int ns_batch_advance(ns_batch* b, double t0);
/* max|div u| over the interior of subdomain i (big_periodic_3D.f90:576-579). */
int ns_batch_max_div(ns_batch* b, int i, double* max_div);
int ns_batch_launch_count(const ns_batch* b, long long* launches);
/* Time every stage kernel over a few persistent grid sizes and keep the
 * fastest in the batch's configuration (runs steps: call on a scratch state). */
int ns_batch_autotune(ns_batch* b, int reps);
/* Device time of every stage kernel of one regular step (mean over reps
 * launches, on a copy of the state), in the stage order interp, predict,
 * vel_bc x/y/z, x forward, y forward, z solve, y inverse, x inverse,
 * pr_bc x/y/z, correct, hist: ms_per_stage[16] (the last two unused).  With
 * AB2-CN the vel_bc x/y/z entries are the x, y, z ADI sweeps. */
int ns_batch_profile(ns_batch* b, int reps, double* ms_per_stage);
int ns_batch_get_config(const ns_batch* b, ns_batch_config* out);

/* Weights of MATLAB interp1(knots, y, t, 'spline') (the not-a-knot cubic
 * spline) on the window of 6 knots around t that
 * sub_tstep_BC_combined_interpolation.m:59 takes: first = index of the
 * window's first knot (knots ascending), value = sum_q w[q] y[first + q]. */
int ns_spline_weights(const double* knots, int n_knots, double t, int* first, double* w);

/* ------------------------------------------------------------------------
 * Re-simulation error metrics and the err_file writer
 * (re_simulation_sub_tstep_interBC_combine.f90:813-834, :913-931).
 *
 * out[0..3]  = rms(u_ref), rms(v_ref), rms(w_ref), rms(p_ref)   (rms_vel(1..4))
 * out[4..7]  = maxval(|x - x_ref|) / rms(x_ref) for u, v, w, p  (err_vel(1..4))
 * out[8..10] = mean(|x - x_ref|) / rms(x_ref) for u, v, w       (err_vel(5..7))
 * out[11]    = maxval(|oz - oz_ref|) / rms(oz_ref),              (err_vel(8))
 *              oz = diff(v,1,1)/dx - diff(u,1,2)/dy on (nx+1, ny+1, nz+2)
 * over the full padded arrays, mean = sum/size, rms = sqrt(sum(a*a)/size)
 * (other_utility.f90:110-129); reduced on the device.
 * ------------------------------------------------------------------------ */

/* The session's current u, v, w, p against host reference arrays of the
 * same shapes (the parent's sub-block u_sub, v_sub, w_sub, p_sub at the
 * same time step).  Uses the step's scratch fields: call between steps. */
int ns_error_metrics(ns_handle* h, const double* u_ref, const double* v_ref, const double* w_ref, const double* p_ref,
                     double* out);

/* Every subdomain of a batch against the parent session's current state
 * over its index maps (u_sub = u(idx_xu, idx_yu, idx_zu),
 * big_periodic_3D.f90:20-25,665-669): out[12 * i + q]. */
int ns_batch_error_metrics(ns_batch* b, const ns_handle* parent, double* out);

/* Write err_vel (kind 0: time_step + 8 columns, rows of err_vel(1..8)) or
 * rms_vel (kind 1: time_step + 4 columns) in the reference's CSV format:
 * the header line, then "j,<ES12.5E2>,..." for row j = 0 .. nrows-1.
 * Host-only; needs no GPU. */
int ns_write_err_csv(const char* path, int kind, int nrows, const double* rows);

/* Energy spectrum and turbulence statistics of the session's current
 * velocity (MATLAB_post_processing/PowerSpec.m, SpecProp.m, KolmoScale.m as
 * Post_processing_main.m:29-41 chains them), computed on the device from
 * the cell-centred velocity with the Poisson solve's FFT passes.  Cubic,
 * triply periodic boxes only (NS_ERR_SHAPE / NS_ERR_UNSUPPORTED_BC).
 *   k[N-1], E[N-1], count[N-1]: shell N = 1 .. nx/2 (k = N 2 pi / lx), the
 *       spectrum of PowerSpec and the number of modes in the shell;
 *   props[0..9]: dissipation, kin_Sp, kin_Ph, kin_E, up (SpecProp), eta,
 *       u_eta, tau (KolmoScale), lambda = sqrt(15 nu up^2 / eps),
 *       Re_lambda = up lambda / nu.
 * Uses the step's scratch fields: call between steps. */
int ns_spectrum(ns_handle* h, double* k, double* E, long long* count, double* props);

/* ------------------------------------------------------------------------
 * Adjoint tier: the discrete adjoint of the periodic step.
 *
 * The reference has no adjoint; this is the transpose of the tangent-linear
 * model of the step above (big_periodic_3D.f90:326-567) on a triply
 * periodic box with dp_flag = 0, for NS_AB2_CN, NS_AB2 and NS_EULER:
 * projection (symmetric), the CN-ADI sweeps with the transposed line
 * systems in the order z, y, x, and the convection linearised about the
 * stored forward velocity.  The control is the set of independent periodic
 * values of u, v, w: every entry that is a periodic copy (u(nx+1,:,:),
 * the ghost rows of the cell axes) is an image of another entry.
 * ------------------------------------------------------------------------ */

/* Run nsteps steps from the current state (as ns_step), keeping the state
 * at steps 0, K, 2K, ... (K = ckpt_every) on the device.  The state after
 * the call is the state after nsteps steps.  Device memory: 6 fields per
 * checkpoint plus 3 per step of a segment of K steps. */
int ns_adj_forward(ns_handle* h, int nsteps, int ckpt_every);

/* Gradient of a function J of the final velocity with respect to the
 * initial one, given dJ/du(T), dJ/dv(T), dJ/dw(T) (host, reference shapes;
 * an entry that is a periodic copy adds into the value it copies).  Each
 * segment of K steps is recomputed from its checkpoint and then stepped
 * back.  grad_u/v/w (host, reference shapes) receive dJ/du0 etc. on the
 * independent entries and 0 on the periodic copies; grad_hx/hy/hz (may be
 * NULL) receive dJ/d(rhs_?_previous) of the initial history (0 after an
 * Euler start).  The session state is restored to the state after the
 * forward run.  NS_ERR_UNSUPPORTED_BC unless bc = pbc = 1 on every axis
 * and dp_flag = 0. */
int ns_adj_backward(ns_handle* h, const double* dJ_du, const double* dJ_dv, const double* dJ_dw, double* grad_u,
                    double* grad_v, double* grad_w, double* grad_hx, double* grad_hy, double* grad_hz);

/* ------------------------------------------------------------------------
 * HDF5 files of the reference, without libhdf5 (host-only; need no GPU)
 *
 * The reference's snapshots, restarts and sub-block records go through the
 * HDF5 Fortran API (big_periodic_3D.f90:593-726).  These calls read and write
 * the same files: version 0 superblock, version 1 object headers, symbol-table
 * groups, contiguous little-endian double datasets, and one-value int32 /
 * double / fixed-string attributes.  Dims are given in Fortran order and data
 * in Fortran memory order, as in the Fortran API (the file's dataspace holds
 * the dims reversed).  Raw data is written when a dataset is written; every
 * ns_h5_flush / ns_h5_close leaves a complete file.  Files outside the subset
 * (chunked or compressed datasets, the newer object headers) give NS_ERR_IO.
 * ------------------------------------------------------------------------ */
typedef struct ns_h5 ns_h5;

/* h5fcreate_f (H5F_ACC_EXCL_F unless overwrite; big_periodic_3D.f90:593,605,630). */
int ns_h5_create(const char* path, int overwrite, ns_h5** f);
/* h5fopen_f, H5F_ACC_RDONLY_F (writable = 0; :296, :309) or H5F_ACC_RDWR_F
 * (writable = 1; :655-662): an existing file's groups, datasets and
 * attributes are kept, new ones are added. */
int ns_h5_open(const char* path, int writable, ns_h5** f);
/* Write the metadata so that the file on disk is complete (the reference closes and
 * reopens its record files for this, :652-662). */
int ns_h5_flush(ns_h5* f);
/* h5fclose_f: flush and close; f is freed whatever the status. */
int ns_h5_close(ns_h5* f);
/* Why the last call on f failed; with f = NULL, why the last ns_h5_create,
 * ns_h5_open or ns_h5_close of this thread failed. */
const char* ns_h5_last_error(const ns_h5* f);

/* h5gcreate_f (:672, :716): group path "t_1.0000" or "a/b" (the parent must exist). */
int ns_h5_group(ns_h5* f, const char* path);
/* h5ltset_attribute_int_f / _double_f with one value, h5ltset_attribute_string_f
 * (:594-601): on the object at obj ("/" is the root); an attribute of the same
 * name is replaced. */
int ns_h5_attr_int(ns_h5* f, const char* obj, const char* name, int value);
int ns_h5_attr_double(ns_h5* f, const char* obj, const char* name, double value);
int ns_h5_attr_string(ns_h5* f, const char* obj, const char* name, const char* value);
/* h5ltmake_dataset_double_f (:644-650, :674-709): a new dataset at path. */
int ns_h5_write_double(ns_h5* f, const char* path, int rank, const long long* dims, const double* data);

/* h5ltget_dataset_info_f: rank and dims (Fortran order, up to 32). */
int ns_h5_dims(ns_h5* f, const char* path, int* rank, long long* dims);
/* h5ltread_dataset_double_f (:298-301, :311-317): the whole dataset into out;
 * NS_ERR_SHAPE unless its dims are the buffer's dims.  Integer and 4-byte
 * float datasets are converted. */
int ns_h5_read_double(ns_h5* f, const char* path, int rank, const long long* dims, double* out);
/* One attribute value (the first element). */
int ns_h5_get_attr_int(ns_h5* f, const char* obj, const char* name, long long* value);
int ns_h5_get_attr_double(ns_h5* f, const char* obj, const char* name, double* value);
int ns_h5_get_attr_string(ns_h5* f, const char* obj, const char* name, char* buf, int buflen);
/* The members of a group, sorted, one per line, groups with a trailing '/';
 * *needed = bytes including the final NUL (buf may be NULL to ask for it). */
int ns_h5_members(ns_h5* f, const char* group, char* buf, long long buflen, long long* needed);

/* The session's state as a reference snapshot (:630-651): root attributes nx
 * (ny, nz too for a non-cubic box), dt, nu, time_scheme, time_step, time, and
 * datasets u, v, w, p, rhs_x_previous, rhs_y_previous, rhs_z_previous. */
int ns_h5_write_state(ns_handle* h, const char* path, double time, int time_step, int overwrite);
/* Restart from such a file (:309-324): u, v, w, p and, when the file has
 * them, the three histories (then the next step is AB2 or AB2-CN; without
 * them, as in the init file of :296-301, the Euler start).  time and
 * time_step (may be NULL) receive the root attributes (0 if absent). */
int ns_h5_read_state(ns_handle* h, const char* path, double* time, int* time_step);

#ifdef __cplusplus
}
#endif
#endif /* NS_GPU_H */
