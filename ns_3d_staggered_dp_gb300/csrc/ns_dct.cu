// Wall-bounded pressure Poisson solve: the per-axis trigonometric transforms
// of DCT_poisson_solver (NS_functions.f90:1505-1630) and their mix with the
// periodic FFT axes.
//
// A non-periodic axis of N cells is transformed with an exact N x N matrix
// pair (forward F, inverse G = F^-1), built on the host from the MKL
// trigonometric-transform definitions the reference uses:
//   pbc 3 (Neumann on the wall)    : F = DCT-II  (MKL backward staggered cosine)
//   pbc 2 (Dirichlet on the wall)  : flip the sign of every other input,
//                                    DCT-II, reverse the output (= DST-II)
//   pbc 4 (Dirichlet on the ghost) : F = DST-I of N points
// and applied to a line held in shared memory (2N FMAs per complex output).
// Any N works (the subdomain edges 24 and 48 included).
//
// Data flow: with x periodic the x pass is the r2c FFT of ns_fft.cu and the
// y/z passes act on the complex half spectrum (real and imaginary parts
// transform alike).  With every axis non-periodic the x pass applies F_x to
// the real divergence line and packs modes (2q, 2q+1) into one complex value,
// so the y/z passes again act on complex lines; the solve scales the real and
// imaginary parts by their own eigenvalues (double2 table).
// The divergence kernels add the pressure-BC terms of
// pr_bc_staggered_modify_rhs (NS_functions.f90:1345-1400) on the first and
// last cells of every non-periodic axis.
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

namespace {

// Divergence of u*, v*, w* over dt at cell (i, j, k), plus the pressure-BC
// terms of the boundary cells; a given right-hand side is taken as it is
// (already BC-modified).
__device__ __forceinline__ double rhs_cell(const DivArgs& d, const SpecPlan& S, const FOne& c, int i, int j, int k) {
  const Layout& L = d.L;
  const long long g = L.at(i, j, k);
  if (d.rhs) return d.rhs[g];
  double r = fmul(c, fsub(c, d.us[g + 1], d.us[g]), d.cdx);
  r = fma(fsub(c, d.vs[g + L.sy], d.vs[g]), d.cdy, r);
  r = fma(fsub(c, d.ws[g + L.sz], d.ws[g]), d.cdz, r);
  return r + S.bc_term(i, j, k);
}

}  // namespace

// x pass for a non-periodic x axis: real line -> F_x -> packed modes.
// One warp per line (j, k); lane q computes the modes 2q' and 2q'+1.
__global__ void __launch_bounds__(128) dense_x_fwd_kernel(SpecPlan S, DivArgs d, double2* __restrict__ spec) {
  extern __shared__ __align__(16) double xs[];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int line = blockIdx.x * 4 + warp;
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const bool valid = line < ny * nz;
  const int j = valid ? 1 + line % ny : 1, k = valid ? 1 + line / ny : 1;
  double* r = xs + warp * nx;
  const FOne c{d.one, d.mzero};
  if (valid)
    for (int i = lane; i < nx; i += 32) r[i] = rhs_cell(d, S, c, i + 1, j, k);
  __syncwarp();
  if (!valid) return;
  const double* __restrict__ FT = S.fwd[0];  // F^T: FT[n * N + kk] = F[kk][n]
  double2* out = spec + (long long)S.nxs * ((j - 1) + (long long)ny * (k - 1));
  for (int q = lane; q < nx / 2; q += 32) {
    double a = 0.0, b = 0.0;
    for (int n = 0; n < nx; ++n) {
      const double2 f = *reinterpret_cast<const double2*>(FT + (long long)n * nx + 2 * q);
      a = fma(f.x, r[n], a);
      b = fma(f.y, r[n], b);
    }
    out[q] = make_double2(a, b);
  }
}

// x inverse for a non-periodic x axis: packed modes -> G_x -> dp slots 1..nx.
__global__ void __launch_bounds__(128) dense_x_inv_kernel(SpecPlan S, const double2* __restrict__ spec, double* dp,
                                                          Layout L) {
  extern __shared__ __align__(16) double xs[];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int line = blockIdx.x * 4 + warp;
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const bool valid = line < ny * nz;
  const int j = valid ? 1 + line % ny : 1, k = valid ? 1 + line / ny : 1;
  double* X = xs + warp * nx;
  const double2* in = spec + (long long)S.nxs * ((j - 1) + (long long)ny * (k - 1));
  if (valid)
    for (int q = lane; q < nx / 2; q += 32) {
      const double2 v = in[q];
      X[2 * q] = v.x;
      X[2 * q + 1] = v.y;
    }
  __syncwarp();
  if (!valid) return;
  const double* __restrict__ GT = S.inv[0];  // G^T: GT[kk * N + n] = G[n][kk] (x = G X)
  double* o = dp + L.at(1, j, k);
  for (int n = lane; n < nx; n += 32) {
    double a = 0.0;
    for (int kk = 0; kk < nx; ++kk) a = fma(__ldg(GT + (long long)kk * nx + n), X[kk], a);
    o[n] = a;
  }
}

// Dense transform of complex lines along y (AXIS 1) or z (AXIS 2), lanes over
// consecutive spectrum columns (coalesced).  With SOLVE (z only): forward,
// scale by the eigenvalue table, inverse, all on chip.
template <int AXIS, bool FWD, bool SOLVE>
__global__ void __launch_bounds__(128) dense_yz_kernel(SpecPlan S, double2* __restrict__ spec) {
  extern __shared__ __align__(16) double2 ls[];
  constexpr int LPC = 16, T = 8;  // 16 lines (columns) x 8 threads per line
  const int l = threadIdx.x % LPC, t = threadIdx.x / LPC;
  const int N = (AXIS == 1) ? S.ny : S.nz;
  const int col = blockIdx.x * LPC + l;
  const bool valid = col < S.nxs;
  const int o = blockIdx.y;  // the other index (z for y-lines, y for z-lines)
  const long long st = (AXIS == 1) ? (long long)S.nxs : (long long)S.nxs * S.ny;
  const long long base = (AXIS == 1) ? col + (long long)S.nxs * S.ny * o : col + (long long)S.nxs * o;
  double2* line = ls + l;  // element n at line[n * LPC]
  double2* g = spec + base;
  if (valid)
    for (int n = t; n < N; n += T) line[n * LPC] = g[(long long)n * st];
  __syncthreads();
  const double* __restrict__ M = (SOLVE || FWD) ? S.fwd[AXIS] : S.inv[AXIS];
  // outputs k = t + T*q
  double2 acc[16];
  const int nq = (N + T - 1) / T;
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_double2(0.0, 0.0);
  for (int n = 0; n < N; ++n) {
    const double2 v = line[n * LPC];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      if (q < nq) {
        const int kk = t + T * q;
        if (kk < N) {
          const double m = __ldg(M + (long long)kk * N + n);
          acc[q].x = fma(m, v.x, acc[q].x);
          acc[q].y = fma(m, v.y, acc[q].y);
        }
      }
    }
  }
  if (SOLVE) {
    // scale by 1/lambda per (real, imaginary) part; the singular mode takes the mean value
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int kk = t + T * q;
      if (q < nq && kk < N && valid) {
        const long long gi = base + (long long)kk * st;
        const double2 s = __ldg(S.inv_lam2 + gi);
        acc[q].x *= s.x;
        acc[q].y *= s.y;
        if (S.has_mean && gi == 0) acc[q].x = S.mean_val;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int kk = t + T * q;
      if (q < nq && kk < N) line[kk * LPC] = acc[q];
    }
    __syncthreads();
    const double* __restrict__ Gm = S.inv[AXIS];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = make_double2(0.0, 0.0);
    for (int n = 0; n < N; ++n) {
      const double2 v = line[n * LPC];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        if (q < nq) {
          const int kk = t + T * q;
          if (kk < N) {
            const double m = __ldg(Gm + (long long)kk * N + n);
            acc[q].x = fma(m, v.x, acc[q].x);
            acc[q].y = fma(m, v.y, acc[q].y);
          }
        }
      }
    }
  }
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int kk = t + T * q;
    if (q < nq && kk < N) g[(long long)kk * st] = acc[q];
  }
}

cudaError_t launch_dense_x(bool fwd, const SpecPlan& S, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                           cudaStream_t st) {
  const int lines = S.ny * S.nz;
  const size_t sm = (size_t)4 * S.nx * sizeof(double);
  if (fwd) dense_x_fwd_kernel<<<(lines + 3) / 4, 128, sm, st>>>(S, d, spec);
  else dense_x_inv_kernel<<<(lines + 3) / 4, 128, sm, st>>>(S, spec, dp, L);
  return cudaGetLastError();
}

cudaError_t launch_dense_yz(int axis, int mode, const SpecPlan& S, double2* spec, cudaStream_t st) {
  const int N = axis == 1 ? S.ny : S.nz;
  if (N > 128) return cudaErrorInvalidValue;
  const size_t sm = (size_t)N * 16 * sizeof(double2);
  dim3 grid((S.nxs + 15) / 16, axis == 1 ? S.nz : S.ny);
  if (axis == 1 && mode == 0) dense_yz_kernel<1, true, false><<<grid, 128, sm, st>>>(S, spec);
  else if (axis == 1 && mode == 1) dense_yz_kernel<1, false, false><<<grid, 128, sm, st>>>(S, spec);
  else if (axis == 2 && mode == 2) dense_yz_kernel<2, true, true><<<grid, 128, sm, st>>>(S, spec);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace ns
