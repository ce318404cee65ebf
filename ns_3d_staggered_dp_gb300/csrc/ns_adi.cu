// Crank-Nicolson ADI line solves (big_periodic_3D.f90:425-489 with getrs on
// mat_CN; re_simulation_sub_tstep_interBC_combine.f90:656-701 with dttrsb on
// mat_CN_tridiagonal).
//
// All lines of a sweep share one matrix, so its LU factors (no pivoting) are
// precomputed on the host (ns_api.cu) and read as broadcast loads.  Per
// unknown the solve is one FMA forward and one multiply + one FMA backward.
// One thread solves one line; the sweep reads the line from one buffer and
// writes it to another (fixed ping-pong roles, see ns_api.cu).
//
// y and z sweeps: lanes over consecutive x, so every access of the forward
// and backward walks is coalesced.
// x sweep: the lines are contiguous, so a warp owns 32 lines and walks them
// in 32 x 32 blocks staged through shared memory (padded stride 33): every
// global access is a coalesced 256-byte row segment, each thread runs its
// recurrence from shared memory.
//
// Walls (bc 2, 4): the full line including the BC rows is solved; the BC
// rows' right-hand side is the sweep's face value (vel_bc_staggered_CN2,
// NS_functions.f90:313-410).
// Periodic (bc 1): the ghost rows of mat_CN only tie the ghosts to interior
// values, so the solve is reduced to the n interior unknowns, a tridiagonal
// system T plus corner entries, solved by Sherman-Morrison,
// x = y - (s0*y[0] + s1*y[n-1]) * z, with z = T^-1 u precomputed; z decays
// geometrically away from the ends, so the correction is applied only where
// |z| > 1e-18 max|z| (zA, zB).  The periodic copies (slot 0 <- slot n,
// slot n+1 <- slot 1) are then written, which is what the ghost rows of
// mat_CN produce.
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

namespace {

template <int AXIS>
__device__ __forceinline__ void line_of(const Layout& L, int s1, int s2, long long& base, long long& st) {
  if (AXIS == 0) { base = L.at(0, s1, s2); st = 1; }
  else if (AXIS == 1) { base = L.at(s1, 0, s2); st = L.sy; }
  else { base = L.at(s1, s2, 0); st = L.sz; }
}

__device__ __forceinline__ int axis_n(const Layout& L, int axis) { return axis == 0 ? L.nx : (axis == 1 ? L.ny : L.nz); }

// Periodic correction on the end regions and the slot copies, or the carried
// slots of a wall line; x points at slot 0 of the destination line.
__device__ __forceinline__ void finish_line(const LineSys& S, const double* __restrict__ src, double* __restrict__ x,
                                            long long st, int nax, double x_first, double x_last) {
  const int m = S.hi - S.lo + 1;
  double* xl = x + (long long)S.lo * st;
  if (S.periodic) {
    const double g = fma(S.s0, x_first, S.s1 * x_last);
    for (int e = 0; e < S.zA; ++e) xl[(long long)e * st] = fma(-g, __ldg(S.z + e), xl[(long long)e * st]);
    for (int e = (S.zB > S.zA ? S.zB : S.zA); e < m; ++e)
      xl[(long long)e * st] = fma(-g, __ldg(S.z + e), xl[(long long)e * st]);
    x[0] = xl[(long long)(m - 1) * st];         // slot 0 <- slot n
    x[(long long)(nax + 1) * st] = xl[0];       // slot n+1 <- slot 1
  } else {
    for (int s = 0; s < S.lo; ++s) x[(long long)s * st] = src[(long long)s * st];
    for (int s = S.hi + 1; s <= nax + 1; ++s) x[(long long)s * st] = src[(long long)s * st];
  }
}

}  // namespace

// One thread per line, lanes over consecutive x (y and z sweeps).
template <int AXIS>
__global__ void __launch_bounds__(128) adi_seq_kernel(AdiArgs a) {
  const int fld = blockIdx.z;
  const LineSys& S = a.sys[fld];
  const Layout L = a.L;
  const int n1 = (AXIS == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (AXIS == 2) ? L.ny + 2 : L.nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  long long base, st;
  line_of<AXIS>(L, t % n1, t / n1, base, st);
  const double* __restrict__ src = a.src[fld] + base;
  double* __restrict__ dst = a.dst[fld] + base;
  const double* lf = S.l + S.pad;
  const double* di = S.dinv + S.pad;
  const double* cu = S.cu + S.pad;
  const int m = S.hi - S.lo + 1;
  const double* sl = src + (long long)S.lo * st;
  double* xl = dst + (long long)S.lo * st;
  double yp;
  if (S.periodic) yp = sl[0];
  else yp = a.face_lo[fld] ? __ldg(a.face_lo[fld] + t) : 0.0;
  xl[0] = yp;
  for (int e = 1; e < m - 1; ++e) {
    yp = fma(-__ldg(lf + e), yp, sl[(long long)e * st]);
    xl[(long long)e * st] = yp;
  }
  {
    const int e = m - 1;
    const double r = S.periodic ? sl[(long long)e * st] : (a.face_hi[fld] ? __ldg(a.face_hi[fld] + t) : 0.0);
    yp = fma(-__ldg(lf + e), yp, r);
  }
  double xn = yp * __ldg(di + (m - 1));
  const double x_last = xn;
  xl[(long long)(m - 1) * st] = xn;
  for (int e = m - 2; e >= 0; --e) {
    xn = fma(-__ldg(cu + e), xn, xl[(long long)e * st] * __ldg(di + e));
    xl[(long long)e * st] = xn;
  }
  finish_line(S, src, dst, st, axis_n(L, AXIS), xn, x_last);
}

// x sweep: a warp owns 32 contiguous lines (consecutive y slots at one z
// slot) and walks them in blocks of 32 unknowns through shared memory.
namespace {
constexpr int XW = 4;           // warps per CTA
constexpr int XB = 32;          // unknowns per block
constexpr int XS = 33;          // padded stride
}  // namespace

__global__ void __launch_bounds__(32 * XW) adi_x_kernel(AdiArgs a) {
  __shared__ double sh[XW][XB * XS];
  const int fld = blockIdx.z;
  const LineSys& S = a.sys[fld];
  const Layout L = a.L;
  const int n1 = L.ny + 2, n2 = L.nz + 2;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int j0 = (blockIdx.x * XW + warp) * 32;
  const int k = blockIdx.y;
  if (j0 >= n1) return;
  const int nl = min(32, n1 - j0);
  double* sb = sh[warp];
  const double* lf = S.l + S.pad;
  const double* di = S.dinv + S.pad;
  const double* cu = S.cu + S.pad;
  const int m = S.hi - S.lo + 1;
  const int nb = (m + XB - 1) / XB;
  const double* src = a.src[fld] + L.at(S.lo, j0, k);  // unknown 0 of line j0
  double* dst = a.dst[fld] + L.at(S.lo, j0, k);
  const long long sy = L.sy;
  const int plane = (j0 + lane) + n1 * k;
  const bool act = lane < nl;
  double face_lo = 0.0, face_hi = 0.0;
  if (!S.periodic && act) {
    if (a.face_lo[fld]) face_lo = __ldg(a.face_lo[fld] + plane);
    if (a.face_hi[fld]) face_hi = __ldg(a.face_hi[fld] + plane);
  }
  // forward elimination, block by block; y' goes to dst
  double yp = 0.0;
  for (int b = 0; b < nb; ++b) {
    const int e0 = b * XB;
    const int ne = min(XB, m - e0);
    if (lane < ne)
      for (int l = 0; l < nl; ++l) sb[lane * XS + l] = __ldg(src + l * sy + e0 + lane);
    __syncwarp();
    if (act) {
      for (int q = 0; q < ne; ++q) {
        const int e = e0 + q;
        double r = sb[q * XS + lane];
        if (!S.periodic) {
          if (e == 0) r = face_lo;
          if (e == m - 1) r = face_hi;
        }
        yp = fma(-__ldg(lf + e), yp, r);
        sb[q * XS + lane] = yp;
      }
    }
    __syncwarp();
    if (lane < ne)
      for (int l = 0; l < nl; ++l) dst[l * sy + e0 + lane] = sb[lane * XS + l];
    __syncwarp();
  }
  // back substitution, blocks in reverse
  double xn = 0.0, x_last = 0.0;
  for (int b = nb - 1; b >= 0; --b) {
    const int e0 = b * XB;
    const int ne = min(XB, m - e0);
    if (lane < ne)
      for (int l = 0; l < nl; ++l) sb[lane * XS + l] = dst[l * sy + e0 + lane];
    __syncwarp();
    if (act) {
      for (int q = ne - 1; q >= 0; --q) {
        const int e = e0 + q;
        xn = (e == m - 1) ? sb[q * XS + lane] * __ldg(di + e)
                          : fma(-__ldg(cu + e), xn, sb[q * XS + lane] * __ldg(di + e));
        if (e == m - 1) x_last = xn;
        sb[q * XS + lane] = xn;
      }
    }
    __syncwarp();
    if (lane < ne)
      for (int l = 0; l < nl; ++l) dst[l * sy + e0 + lane] = sb[lane * XS + l];
    __syncwarp();
  }
  if (act) {
    const long long base = L.at(0, j0 + lane, k);
    finish_line(S, a.src[fld] + base, a.dst[fld] + base, 1, L.nx, xn, x_last);
  }
}

cudaError_t launch_adi(int axis, const AdiArgs& a, cudaStream_t st) {
  if (axis == 0) {
    const int n1 = a.L.ny + 2, n2 = a.L.nz + 2;
    dim3 grid((n1 + 32 * XW - 1) / (32 * XW), n2, 3);
    adi_x_kernel<<<grid, 32 * XW, 0, st>>>(a);
    return cudaGetLastError();
  }
  const int n1 = a.L.nx + 2;
  const int n2 = (axis == 2) ? a.L.ny + 2 : a.L.nz + 2;
  dim3 grid((n1 * n2 + 127) / 128, 1, 3);
  if (axis == 1) adi_seq_kernel<1><<<grid, 128, 0, st>>>(a);
  else adi_seq_kernel<2><<<grid, 128, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace ns
