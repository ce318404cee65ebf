// Energy spectrum and turbulence statistics of the current velocity, on the
// device: MATLAB_post_processing/PowerSpec.m (and PowerSpec3D.m), SpecProp.m
// and KolmoScale.m as Post_processing_main.m:30-41 chains them.
//
//   u_p = cell average of u (and v_p, w_p), n^3 cells
//   muu = |fftn(u_p)|^2 / n^6 (likewise v, w), wavenumber magnitude
//   r = sqrt(kx^2 + ky^2 + kz^2) with the FFT bins (0..n/2, -n/2+1..-1)
//   shell N = 1..n/2 (in units of dk = 2 pi / L): r <= 1.5 for N = 1,
//   N - 1/2 < r <= N + 1/2 for 1 < N < n/2, n/2 - 1/2 < r <= n/2 for the last
//   E(N) = sum over the shell of (muu + mvv + mww) * 2 pi k^2 / (count dk^3)
//   dissipation = sum 2 nu k^2 E dk, kin_Sp = sum E dk,
//   kin_Ph = sum (u^2 + v^2 + w^2) / (2 n^3), kin_E = sum (muu + mvv + mww) / 2,
//   up = sqrt(sum(u^2 + v^2 + w^2) / (3 n^3)), eta = (nu^3/eps)^(1/4),
//   u_eta = (nu eps)^(1/4), tau = (nu/eps)^(1/2),
//   lambda = sqrt(15 nu up^2 / eps), Re_lambda = up lambda / nu.
// Because r^2 is an integer and the shell edges sit at N^2 +- N + 1/4, the
// shells are decided exactly with integers: N^2 - N + 1 <= r^2 <= N^2 + N
// (r^2 <= 2 for the first, (n/2)^2 - n/2 + 1 <= r^2 <= (n/2)^2 for the last).
//
// The transforms are the Poisson solve's forward FFT passes (half spectrum,
// x fastest); a half-spectrum bin with 0 < kx < n/2 stands for two modes.
#include <cmath>
#include <string>
#include <vector>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"
#include "ns_session.cuh"

namespace ns {
namespace {

constexpr int kSpecThreads = 256;
constexpr int kSpecBlocks = 152 * 4;

// Cell average of a face field along its own axis, into cell slots 1..n.
__global__ void __launch_bounds__(256) cell_center_kernel(Layout L, const double* __restrict__ f,
                                                          double* __restrict__ out, int axis) {
  const long long n = (long long)L.nx * L.ny * L.nz;
  const long long off = axis == 0 ? 1 : (axis == 1 ? L.sy : L.sz);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.nx);
    const long long r = t / L.nx;
    const int j = 1 + (int)(r % L.ny);
    const int k = 1 + (int)(r / L.ny);
    const long long g = L.at(i, j, k);
    out[g] = (f[g] + f[g + off]) * 0.5;
  }
}

// Block partial sums of c0^2 + c1^2 + c2^2 over the cells.
__global__ void __launch_bounds__(kSpecThreads) energy_kernel(Layout L, const double* __restrict__ c0,
                                                              const double* __restrict__ c1,
                                                              const double* __restrict__ c2, double* partial) {
  const long long n = (long long)L.nx * L.ny * L.nz;
  double s = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.nx);
    const long long r = t / L.nx;
    const int j = 1 + (int)(r % L.ny);
    const int k = 1 + (int)(r / L.ny);
    const long long g = L.at(i, j, k);
    s = fma(c0[g], c0[g], s);
    s = fma(c1[g], c1[g], s);
    s = fma(c2[g], c2[g], s);
  }
  __shared__ double red[kSpecThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < kSpecThreads / 32; ++w) a += red[w];
    partial[blockIdx.x] = a;
  }
}

// Shell of r2 (1..kend), 0 for none.
__device__ __forceinline__ int shell_of(long long r2, int kend) {
  if (r2 <= 2) return 1;
  int N = (int)llrint(sqrt((double)r2));
  while ((long long)N * N + N < r2) ++N;
  while ((long long)N * N - N + 1 > r2) --N;
  if (N > kend) return 0;
  if (N == kend && r2 > (long long)kend * kend) return 0;
  return N;
}

// Shell sums of mult * |spec|^2 (bin 0: every mode) and, when counting, the
// number of full-spectrum modes per shell; per-block partials.
__global__ void __launch_bounds__(kSpecThreads) shell_kernel(const double2* __restrict__ spec, int nx, int ny, int nz,
                                                             int kend, double* __restrict__ part,
                                                             unsigned long long* __restrict__ cpart, int count) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* bins = reinterpret_cast<double*>(smem_raw);
  unsigned int* cnt = reinterpret_cast<unsigned int*>(bins + (kend + 1));
  for (int b = threadIdx.x; b <= kend; b += blockDim.x) { bins[b] = 0.0; cnt[b] = 0u; }
  __syncthreads();
  const int nxh = nx / 2 + 1;
  const long long tot = (long long)nxh * ny * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(t % nxh);
    const long long r = t / nxh;
    const int jy = (int)(r % ny);
    const int jz = (int)(r / ny);
    const long long ry = jy <= ny / 2 ? jy : jy - ny;
    const long long rz = jz <= nz / 2 ? jz : jz - nz;
    const long long r2 = (long long)kx * kx + ry * ry + rz * rz;
    const int mult = (kx == 0 || 2 * kx == nx) ? 1 : 2;
    const double2 v = spec[t];
    const double e = mult * fma(v.x, v.x, v.y * v.y);
    atomicAdd(&bins[0], e);
    const int N = shell_of(r2, kend);
    if (N > 0) {
      atomicAdd(&bins[N], e);
      if (count) atomicAdd(&cnt[N], (unsigned)mult);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b <= kend; b += blockDim.x) {
    part[(long long)blockIdx.x * (kend + 1) + b] = bins[b];
    if (count) cpart[(long long)blockIdx.x * (kend + 1) + b] = cnt[b];
  }
}

}  // namespace
}  // namespace ns

using namespace ns;

extern "C" {

int ns_spectrum(ns_handle* h, double* k_out, double* E_out, long long* count_out, double* props) {
  if (!h) return NS_ERR_ARG;
  if (!k_out || !E_out || !count_out || !props) return api_fail(h, NS_ERR_ARG, "spectrum: all outputs are required");
  const ns_config& c = h->cfg;
  if (c.nx != c.ny || c.nx != c.nz || c.lx != c.ly || c.lx != c.lz)
    return api_fail(h, NS_ERR_SHAPE, "spectrum: a cubic box (nx = ny = nz, lx = ly = lz)");
  for (int a = 0; a < 3; ++a)
    if (c.pbc[a] != 1) return api_fail(h, NS_ERR_UNSUPPORTED_BC, "spectrum: the triply periodic box only");
  const int n = c.nx, kend = n / 2;
  const Layout& L = h->L;
  cudaStream_t st = h->stream;
  double* cc[3] = {h->us, h->vs, h->ws};  // cell-centred u, v, w (scratch between steps)
  const double* f[3] = {h->u, h->v, h->w};
  auto fail_cuda = [&](cudaError_t e) { return api_fail(h, NS_ERR_CUDA, std::string("spectrum: ") + cudaGetErrorString(e)); };
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 3; ++q) {
    cell_center_kernel<<<152 * 8, 256, 0, st>>>(L, f[q], cc[q], q);
    api_mark(h, "spec_center", 1);
  }
  double* part = nullptr;
  unsigned long long* cpart = nullptr;
  double* epart = nullptr;
  const size_t nb = (size_t)kSpecBlocks * (kend + 1);
  if ((e = cudaMallocAsync(&part, 3 * nb * sizeof(double), st)) != cudaSuccess) return fail_cuda(e);
  if ((e = cudaMallocAsync(&cpart, nb * sizeof(unsigned long long), st)) != cudaSuccess) return fail_cuda(e);
  if ((e = cudaMallocAsync(&epart, kSpecBlocks * sizeof(double), st)) != cudaSuccess) return fail_cuda(e);
  energy_kernel<<<kSpecBlocks, kSpecThreads, 0, st>>>(L, cc[0], cc[1], cc[2], epart);
  api_mark(h, "spec_energy", 1);
  const size_t smem = (kend + 1) * (sizeof(double) + sizeof(unsigned int));
  for (int q = 0; q < 3 && e == cudaSuccess; ++q) {
    DivArgs d{};
    d.L = L;
    d.rhs = cc[q];
    d.one = 1.0; d.mzero = -0.0;
    if ((e = launch_fft_forward3(h->plan, d, h->spec, st, api_marker(h))) != cudaSuccess) break;
    shell_kernel<<<kSpecBlocks, kSpecThreads, smem, st>>>(h->spec, n, n, n, kend, part + q * nb, cpart, q == 0);
    api_mark(h, "spec_shells", 1);
    e = cudaGetLastError();
  }
  std::vector<double> hp(3 * nb), he(kSpecBlocks);
  std::vector<unsigned long long> hc(nb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, 3 * nb * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cpart, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(he.data(), epart, kSpecBlocks * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(part, st);
  cudaFreeAsync(cpart, st);
  cudaFreeAsync(epart, st);
  if (e != cudaSuccess) return fail_cuda(e);
  // the x split leaves every bin times 2: |DFT|^2 = |spec|^2 / 4; muu divides by n^6
  const double ncell = (double)n * n * n;
  const double norm = 0.25 / (ncell * ncell);
  std::vector<double> shell(kend + 1, 0.0);
  std::vector<long long> cnt(kend + 1, 0);
  for (int q = 0; q < 3; ++q)
    for (int b = 0; b < kSpecBlocks; ++b)
      for (int N = 0; N <= kend; ++N) shell[N] += hp[q * nb + (size_t)b * (kend + 1) + N];
  for (int b = 0; b < kSpecBlocks; ++b)
    for (int N = 0; N <= kend; ++N) cnt[N] += (long long)hc[(size_t)b * (kend + 1) + N];
  double esum = 0.0;
  for (int b = 0; b < kSpecBlocks; ++b) esum += he[b];
  const double pi = 3.1415926535897932;
  const double dk = 2.0 * pi / c.lx;
  double kin_sp = 0.0, diss = 0.0;
  for (int N = 1; N <= kend; ++N) {
    const double kk = N * dk;
    const double spec_n = shell[N] * norm;
    const double En = cnt[N] > 0 ? spec_n * 2.0 * pi * kk * kk / ((double)cnt[N] * dk * dk * dk) : 0.0;
    k_out[N - 1] = kk;
    E_out[N - 1] = En;
    count_out[N - 1] = cnt[N];
    kin_sp += En * dk;
    diss += 2.0 * c.nu * kk * kk * En * dk;
  }
  const double nu = c.nu;
  const double up = std::sqrt(esum / (3.0 * ncell));
  props[0] = diss;
  props[1] = kin_sp;
  props[2] = 0.5 * esum / ncell;         // kin_Ph
  props[3] = 0.5 * shell[0] * norm;       // kin_E
  props[4] = up;
  props[5] = std::pow(nu * nu * nu / diss, 0.25);  // eta
  props[6] = std::pow(nu * diss, 0.25);            // u_eta
  props[7] = std::sqrt(nu / diss);                 // tau
  props[8] = std::sqrt(15.0 * nu * up * up / diss);  // lambda (Taylor microscale)
  props[9] = up * props[8] / nu;                   // Re_lambda
  return NS_OK;
}

}  // extern "C"
