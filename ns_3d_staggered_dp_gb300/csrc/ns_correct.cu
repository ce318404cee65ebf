// Projection correction (big_periodic_3D.f90:562-567;
// re_simulation_sub_tstep_interBC_combine.f90:793-802):
//   dp = dp - dp(1,1,1)   (gauge, periodic driver only)
//   u = -dt*diff(dp,1,1)/dx + u*,  v = ..., w = ...,  p = dp_flag*p + dp
// computed over each field's full padded extent, ghosts included, exactly as
// the reference's whole-array expressions.  The gauge constant cancels in
// the differences, so it is applied to p only.  The extra face slot 0 of a
// periodic axis is produced from the same inputs as face n (its periodic
// image), so both hold the same bits.
//
// Also the max|div u| diagnostic (big_periodic_3D.f90:576-579) as an
// integer atomicMax on the bit patterns of |div| (order-preserving for
// non-negative doubles; a NaN sorts above every finite value).
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

// Slot (i, j, k) of the padded box.
__device__ __forceinline__ void correct_body(const CorrectArgs& a, int i, int j, int k) {
  const Layout L = a.L;
  const FOne c{a.one, a.mzero};
  const long long g = L.at(i, j, k);
  const double* __restrict__ dp = a.dp;
  const double dpc = dp[g];
  // u: face slots 1..nx+1 along x (slot 0 = image of slot nx when periodic)
  {
    int ii = i;
    if (ii == 0 && a.per[0]) ii = L.nx;
    if (ii >= 1) {
      const long long gg = L.at(ii, j, k);
      a.u[g] = fma(a.gx, fsub(c, dp[gg], dp[gg - 1]), a.us[gg]);
    }
  }
  {
    int jj = j;
    if (jj == 0 && a.per[1]) jj = L.ny;
    if (jj >= 1) {
      const long long gg = L.at(i, jj, k);
      a.v[g] = fma(a.gy, fsub(c, dp[gg], dp[gg - L.sy]), a.vs[gg]);
    }
  }
  {
    int kk = k;
    if (kk == 0 && a.per[2]) kk = L.nz;
    if (kk >= 1) {
      const long long gg = L.at(i, j, kk);
      a.w[g] = fma(a.gz, fsub(c, dp[gg], dp[gg - L.sz]), a.ws[gg]);
    }
  }
  {
    double d = dpc;
    if (a.gauge) d = fsub(c, d, dp[L.at(0, 0, 0)]);
    a.p[g] = a.dp_flag ? fadd(c, a.p[g], d) : d;
  }
}

// Flat slot index t of the padded box (x fastest).  A subdomain box holds
// fewer than 2^31 slots, so the split takes two 32-bit divisions (a 64-bit
// division by a runtime value is a long software sequence per slot).
__device__ __forceinline__ void correct_body(const CorrectArgs& a, unsigned t) {
  const Layout L = a.L;
  const unsigned nx2 = (unsigned)L.nx + 2u, ny2 = (unsigned)L.ny + 2u, nz2 = (unsigned)L.nz + 2u;
  if (t >= nx2 * ny2 * nz2) return;
  const unsigned r = t / nx2, k = r / ny2;
  correct_body(a, (int)(t - r * nx2), (int)(r - k * ny2), (int)k);
}

// Plane k0 + blockIdx.y; the x blocks cover its (nx+2)(ny+2) slots, which a
// 32-bit division splits into (i, j).
__global__ void __launch_bounds__(256) correct_kernel(CorrectArgs a, int k0) {
  const unsigned nx2 = (unsigned)a.L.nx + 2u;
  const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nx2 * ((unsigned)a.L.ny + 2u)) return;
  const unsigned j = q / nx2;
  correct_body(a, (int)(q - j * nx2), (int)j, k0 + (int)blockIdx.y);
}

// Batched: one 256-element chunk of a subdomain box per work item.
__global__ void __launch_bounds__(256) correct_batch_kernel(const CorrectArgs* __restrict__ tab,
                                                            const BatchItem* __restrict__ items, int n_items) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    correct_body(tab[w.sub], (unsigned)w.bx * 256u + threadIdx.x);
  }
}

cudaError_t launch_correct_batch(const CorrectArgs* tab, const BatchItem* items, int n_items, int grid,
                                 cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  grid = grid > 0 ? grid : 8 * 152;
  if (grid > n_items) grid = n_items;
  correct_batch_kernel<<<grid, 256, 0, st>>>(tab, items, n_items);
  return cudaGetLastError();
}

cudaError_t launch_correct(const CorrectArgs& a, cudaStream_t st) { return launch_correct_planes(a, 0, a.L.nz + 2, st); }

cudaError_t launch_correct_planes(const CorrectArgs& a, int k0, int k1, cudaStream_t st) {
  if (k0 < 0 || k1 > a.L.nz + 2 || k0 > k1) return cudaErrorInvalidValue;
  if (k0 == k1) return cudaSuccess;
  const long long plane = (long long)(a.L.nx + 2) * (a.L.ny + 2);
  const dim3 grid((unsigned)((plane + 255) / 256), (unsigned)(k1 - k0));
  correct_kernel<<<grid, 256, 0, st>>>(a, k0);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) diag_kernel(Layout L, const double* __restrict__ u, const double* __restrict__ v,
                                                   const double* __restrict__ w, double idx, double idy, double idz,
                                                   unsigned long long* out) {
  const long long tot = (long long)L.nx * L.ny * L.nz;
  unsigned long long best = 0ull;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.nx);
    const int j = 1 + (int)((t / L.nx) % L.ny);
    const int k = 1 + (int)(t / ((long long)L.nx * L.ny));
    const long long g = L.at(i, j, k);
    const double d = (u[g + 1] - u[g]) * idx + (v[g + L.sy] - v[g]) * idy + (w[g + L.sz] - w[g]) * idz;
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(d));
    best = b > best ? b : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, best, o);
    best = x > best ? x : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

cudaError_t launch_diag(const Layout& L, const double* u, const double* v, const double* w, double idx, double idy,
                        double idz, unsigned long long* out_bits, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out_bits, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  diag_kernel<<<152 * 4, 256, 0, st>>>(L, u, v, w, idx, idy, idz, out_bits);
  return cudaGetLastError();
}

}  // namespace ns
