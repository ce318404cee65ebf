// Crank-Nicolson ADI line solves (big_periodic_3D.f90:425-489 with getrs on
// mat_CN; re_simulation_sub_tstep_interBC_combine.f90:656-701 with dttrsb on
// mat_CN_tridiagonal).  One thread solves one line of one field.
//
// All lines of a sweep share one matrix, so its LU factors are precomputed
// on the host (ns_api.cu) and read as broadcast loads.  Per element the
// solve is one FMA forward and one multiply + one FMA backward.
//
// Walls (bc 2, 4): the full line including the BC rows is solved; the BC
// rows' right-hand side is the sweep's face value (vel_bc_staggered_CN2,
// NS_functions.f90:313-410).
// Periodic (bc 1): the ghost rows of mat_CN only tie the ghosts to interior
// values, so the solve is reduced to the n interior unknowns, a tridiagonal
// system plus corner entries.  It is solved by Sherman-Morrison,
// x = y - (s0*y[0] + s1*y[n-1]) * z, with z = T^-1 u precomputed.  z decays
// geometrically away from the ends, so the correction is applied only where
// |z| > 1e-18 max|z| (zA, zB); the skipped terms are below double rounding.
// The periodic copies (slot 0 <- slot n, slot n+1 <- slot 1) are then written,
// which is what the ghost rows of mat_CN produce.
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

template <int AXIS>
__global__ void __launch_bounds__(128) adi_kernel(AdiArgs a) {
  const int fld = blockIdx.y;
  const LineSys S = a.sys[fld];
  const Layout L = a.L;
  const int n1 = (AXIS == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (AXIS == 2) ? L.ny + 2 : L.nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  const int s1 = t % n1, s2 = t / n1;
  // Lines outside the field's own extent in the two other axes carry no data.
  if (s1 < a.ext_lo[fld][0] || s1 > a.ext_hi[fld][0] || s2 < a.ext_lo[fld][1] || s2 > a.ext_hi[fld][1]) return;
  long long base, st;
  if (AXIS == 0) {
    base = L.at(0, s1, s2); st = 1;
  } else if (AXIS == 1) {
    base = L.at(s1, 0, s2); st = L.sy;
  } else {
    base = L.at(s1, s2, 0); st = L.sz;
  }
  double* __restrict__ x = a.f[fld] + base;
  const double* __restrict__ lf = S.l;
  const double* __restrict__ di = S.dinv;
  const double* __restrict__ cu = S.cu;
  const int lo = S.lo, m = S.hi - S.lo + 1;
  double* __restrict__ xl = x + (long long)lo * st;

  // Forward elimination, y'[i] = r[i] - l[i] y'[i-1], stored in place.
  double r0;
  if (S.periodic) {
    r0 = xl[0];
  } else {
    r0 = a.face_lo[fld] ? __ldg(a.face_lo[fld] + t) : 0.0;
  }
  double yp = r0;
  xl[0] = yp;
  for (int i = 1; i < m - 1; ++i) {
    const double r = xl[(long long)i * st];
    yp = fma(-__ldg(lf + i), yp, r);
    xl[(long long)i * st] = yp;
  }
  {
    const int i = m - 1;
    double r;
    if (S.periodic) {
      r = xl[(long long)i * st];
    } else {
      r = a.face_hi[fld] ? __ldg(a.face_hi[fld] + t) : 0.0;
    }
    yp = fma(-__ldg(lf + i), yp, r);
  }
  // Back substitution, x[i] = y'[i]/d[i] - (c[i]/d[i]) x[i+1].
  double xn = yp * __ldg(di + (m - 1));
  const double xlast = xn;
  xl[(long long)(m - 1) * st] = xn;
  for (int i = m - 2; i >= 0; --i) {
    const double y = xl[(long long)i * st];
    xn = fma(-__ldg(cu + i), xn, y * __ldg(di + i));
    xl[(long long)i * st] = xn;
  }
  if (S.periodic) {
    const double g = fma(S.s0, xn, S.s1 * xlast);
    const int zA = S.zA, zB = S.zB;
    for (int i = 0; i < zA; ++i) {
      const long long o = (long long)i * st;
      xl[o] = fma(-g, __ldg(S.z + i), xl[o]);
    }
    for (int i = (zB > zA ? zB : zA); i < m; ++i) {
      const long long o = (long long)i * st;
      xl[o] = fma(-g, __ldg(S.z + i), xl[o]);
    }
    // slots 1..n hold the solution; slot 0 <- slot n, slot n+1 <- slot 1
    x[0] = x[(long long)S.n * st];
    x[(long long)(S.n + 1) * st] = x[st];
  }
}

cudaError_t launch_adi(int axis, const AdiArgs& a, cudaStream_t st) {
  const int n1 = (axis == 0) ? a.L.ny + 2 : a.L.nx + 2;
  const int n2 = (axis == 2) ? a.L.ny + 2 : a.L.nz + 2;
  const int lines = n1 * n2;
  dim3 block(128);
  dim3 grid((lines + 127) / 128, 3);
  if (axis == 0) adi_kernel<0><<<grid, block, 0, st>>>(a);
  else if (axis == 1) adi_kernel<1><<<grid, block, 0, st>>>(a);
  else adi_kernel<2><<<grid, block, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace ns
