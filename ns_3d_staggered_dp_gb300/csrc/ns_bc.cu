// Ghost/face fills.  Each fill runs one pass per axis in the reference's
// order (x, then y, then z), each pass over the full extent of the two other
// axes including their ghosts, so edge and corner values come out as in
// vel_bc_staggered (NS_functions.f90:213-310) and pr_bc_staggered
// (NS_functions.f90:1403-1464).
#include <algorithm>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

namespace {

struct AxisGeo {
  long long base, st;  // slot 0 of the line, stride along the axis
  int n;               // cells along the axis
  int plane;           // index into the face planes
  bool ok;
};

template <int AXIS>
__device__ __forceinline__ AxisGeo axis_geo(const Layout& L, int t) {
  const int n1 = (AXIS == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (AXIS == 2) ? L.ny + 2 : L.nz + 2;
  AxisGeo g;
  g.ok = t < n1 * n2;
  const int s1 = t % n1, s2 = t / n1;
  g.plane = t;
  if (AXIS == 0) { g.base = L.at(0, s1, s2); g.st = 1; g.n = L.nx; }
  else if (AXIS == 1) { g.base = L.at(s1, 0, s2); g.st = L.sy; g.n = L.ny; }
  else { g.base = L.at(s1, s2, 0); g.st = L.sz; g.n = L.nz; }
  return g;
}

__device__ __forceinline__ double facev(const double* f, int i) { return f ? f[i] : 0.0; }

// One field along one axis.  normal: the field is staggered along this axis
// (face slots 1..n+1); otherwise cell-centred (ghost slots 0 and n+1).
__device__ __forceinline__ void vel_fill(double* x, long long st, int n, int bc, bool normal, const double* flo,
                                         const double* fhi, int pl) {
  double* hi = x + (long long)(n + 1) * st;
  if (bc == 1) {
    if (normal) {
      *hi = x[st];                      // u(nx+1) = u(1)
      x[0] = x[(long long)n * st];      // extra slot: face 0 = face n
    } else {
      x[0] = x[(long long)n * st];      // v(1) = v(nx+1)
      *hi = x[st];                      // v(nx+2) = v(2)
    }
  } else if (bc == 2) {
    if (normal) {
      x[st] = facev(flo, pl);
      *hi = facev(fhi, pl);
    } else {
      x[0] = fma(2.0, facev(flo, pl), -x[st]);
      *hi = fma(2.0, facev(fhi, pl), -x[(long long)n * st]);
    }
  } else if (bc == 4) {
    if (normal) {
      x[st] = facev(flo, pl);
      *hi = facev(fhi, pl);
    } else {
      x[0] = facev(flo, pl);
      *hi = facev(fhi, pl);
    }
  }
}

template <int AXIS>
__device__ __forceinline__ void vel_bc_body(const Layout& L, double* us, double* vs, double* ws, const FacePlanes& F,
                                            int bc, int t) {
  const AxisGeo g = axis_geo<AXIS>(L, t);
  if (!g.ok) return;
  vel_fill(us + g.base, g.st, g.n, bc, AXIS == 0, F.f[0][0], F.f[0][1], g.plane);
  vel_fill(vs + g.base, g.st, g.n, bc, AXIS == 1, F.f[1][0], F.f[1][1], g.plane);
  vel_fill(ws + g.base, g.st, g.n, bc, AXIS == 2, F.f[2][0], F.f[2][1], g.plane);
}

template <int AXIS>
__global__ void vel_bc_kernel(Layout L, double* us, double* vs, double* ws, FacePlanes F, int bc) {
  vel_bc_body<AXIS>(L, us, vs, ws, F, bc, blockIdx.x * blockDim.x + threadIdx.x);
}

template <int AXIS>
__device__ __forceinline__ void pr_bc_body(const Layout& L, double* dp, const FacePlanes& F, int pbc, double h, int t) {
  const AxisGeo g = axis_geo<AXIS>(L, t);
  if (!g.ok) return;
  double* x = dp + g.base;
  const long long st = g.st;
  const int n = g.n;
  double* hi = x + (long long)(n + 1) * st;
  const double* flo = F.f[3][0];
  const double* fhi = F.f[3][1];
  if (pbc == 1) {
    x[0] = x[(long long)n * st];
    *hi = x[st];
  } else if (pbc == 2) {
    x[0] = fma(2.0, facev(flo, g.plane), -x[st]);
    *hi = fma(2.0, facev(fhi, g.plane), -x[(long long)n * st]);
  } else if (pbc == 3) {
    x[0] = fma(-h, facev(flo, g.plane), x[st]);
    *hi = fma(h, facev(fhi, g.plane), x[(long long)n * st]);
  } else if (pbc == 4) {
    x[0] = facev(flo, g.plane);
    *hi = facev(fhi, g.plane);
  }
}

// Lines t in [t0, t1) of the pass along AXIS.
template <int AXIS>
__global__ void pr_bc_kernel(Layout L, double* dp, FacePlanes F, int pbc, double h, int t0, int t1) {
  const int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t < t1) pr_bc_body<AXIS>(L, dp, F, pbc, h, t);
}

// Batched fill pass along AXIS: velocity (PR false) or pressure ghosts, one
// 256-element chunk of a face plane per work item.
template <int AXIS, bool PR>
__global__ void __launch_bounds__(256) bc_batch_kernel(const BatchBcArgs* __restrict__ tab,
                                                       const BatchItem* __restrict__ items, int n_items) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const BatchBcArgs& a = tab[w.sub];
    const int t = w.bx * 256 + threadIdx.x;
    if (PR) pr_bc_body<AXIS>(a.L, a.dp, a.F.ax[AXIS], a.pbc[AXIS], a.h[AXIS], t);
    else if (a.bc[AXIS] != 3) vel_bc_body<AXIS>(a.L, a.us, a.vs, a.ws, a.F.ax[AXIS], a.bc[AXIS], t);
  }
}


// Extra face slot 0 of a periodic axis (face 0 = face n) for the face field of that axis.
__global__ void extra_slot_kernel(Layout L, double* f, int axis) {
  const int n1 = (axis == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (axis == 2) ? L.ny + 2 : L.nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  const int s1 = t % n1, s2 = t / n1;
  if (axis == 0) f[L.at(0, s1, s2)] = f[L.at(L.nx, s1, s2)];
  else if (axis == 1) f[L.at(s1, 0, s2)] = f[L.at(s1, L.ny, s2)];
  else f[L.at(s1, s2, 0)] = f[L.at(s1, s2, L.nz)];
}

}  // namespace

int plane_count(const Layout& L, int axis) {
  const int n1 = (axis == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (axis == 2) ? L.ny + 2 : L.nz + 2;
  return n1 * n2;
}

cudaError_t launch_bc_batch(int axis, bool pr, const BatchBcArgs* tab, const BatchItem* items, int n_items, int grid,
                            cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  grid = std::min(grid > 0 ? grid : 4 * 152, n_items);
#define NS_BC_CASE(A, P) \
  if (axis == A && pr == P) bc_batch_kernel<A, P><<<grid, 256, 0, st>>>(tab, items, n_items);
  NS_BC_CASE(0, false) NS_BC_CASE(1, false) NS_BC_CASE(2, false) NS_BC_CASE(0, true) NS_BC_CASE(1, true)
  NS_BC_CASE(2, true)
#undef NS_BC_CASE
  return cudaGetLastError();
}

cudaError_t launch_extra_slots(const Layout& L, double* u, double* v, double* w, const int bc[3], cudaStream_t st) {
  double* f[3] = {u, v, w};
  for (int a = 0; a < 3; ++a) {
    if (bc[a] != 1) continue;
    const int n = plane_count(L, a);
    extra_slot_kernel<<<(n + 255) / 256, 256, 0, st>>>(L, f[a], a);
  }
  return cudaGetLastError();
}

cudaError_t launch_vel_bc(const Layout& L, double* us, double* vs, double* ws, const FaceSet& F, const int bc[3],
                          cudaStream_t st) {
  for (int a = 0; a < 3; ++a) {
    if (bc[a] == 3) continue;  // Neumann velocity: no fill (NS_functions.f90:247)
    const int n = plane_count(L, a);
    dim3 grid((n + 255) / 256);
    if (a == 0) vel_bc_kernel<0><<<grid, 256, 0, st>>>(L, us, vs, ws, F.ax[0], bc[0]);
    if (a == 1) vel_bc_kernel<1><<<grid, 256, 0, st>>>(L, us, vs, ws, F.ax[1], bc[1]);
    if (a == 2) vel_bc_kernel<2><<<grid, 256, 0, st>>>(L, us, vs, ws, F.ax[2], bc[2]);
  }
  return cudaGetLastError();
}

cudaError_t launch_pr_bc(const Layout& L, double* dp, const FaceSet& F, const int pbc[3], double dx, double dy,
                         double dz, cudaStream_t st) {
  const double h[3] = {dx, dy, dz};
  for (int a = 0; a < 3; ++a) {
    const int n = plane_count(L, a);
    dim3 grid((n + 255) / 256);
    if (a == 0) pr_bc_kernel<0><<<grid, 256, 0, st>>>(L, dp, F.ax[0], pbc[0], h[0], 0, n);
    if (a == 1) pr_bc_kernel<1><<<grid, 256, 0, st>>>(L, dp, F.ax[1], pbc[1], h[1], 0, n);
    if (a == 2) pr_bc_kernel<2><<<grid, 256, 0, st>>>(L, dp, F.ax[2], pbc[2], h[2], 0, n);
  }
  return cudaGetLastError();
}

cudaError_t launch_pr_bc_planes(const Layout& L, double* dp, const FaceSet& F, const int pbc[3], double dx,
                                double dy, int k0, int k1, cudaStream_t st) {
  if (k0 < 0 || k1 > L.nz + 2 || k0 > k1) return cudaErrorInvalidValue;
  if (k0 == k1) return cudaSuccess;
  // a line of the x pass is (j, k) with t = j + (ny+2) k, of the y pass (i, k) with t = i + (nx+2) k
  const int px = L.ny + 2, py = L.nx + 2;
  pr_bc_kernel<0><<<(px * (k1 - k0) + 255) / 256, 256, 0, st>>>(L, dp, F.ax[0], pbc[0], dx, px * k0, px * k1);
  pr_bc_kernel<1><<<(py * (k1 - k0) + 255) / 256, 256, 0, st>>>(L, dp, F.ax[1], pbc[1], dy, py * k0, py * k1);
  return cudaGetLastError();
}

cudaError_t launch_pr_bc_z(const Layout& L, double* dp, const FaceSet& F, int pbc_z, double dz, cudaStream_t st) {
  const int n = plane_count(L, 2);
  pr_bc_kernel<2><<<(n + 255) / 256, 256, 0, st>>>(L, dp, F.ax[2], pbc_z, dz, 0, n);
  return cudaGetLastError();
}

}  // namespace ns
