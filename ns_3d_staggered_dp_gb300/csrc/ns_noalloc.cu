// ns_poisson_fft_noalloc: the periodic FFT pressure Poisson solve with all of
// its scratch (half spectrum, twiddle tables, inverse eigenvalues) in one
// file-scope device array, for callers that must not allocate device memory.
//
// Who cannot allocate: solvers embedded in a host application whose device
// memory is wholly owned by another allocator (a framework's caching pool,
// or an arena the host reserved up front so that nothing else may take
// device memory), and real-time loops that cannot take the implicit device
// synchronisation and latency of an allocation.
//
// Limits and rules:
//  - The scratch is kNoAllocScratchDoubles doubles (4 MiB) in every device
//    that loads the library, held until the process exits (the driver places
//    it when it loads the library's module, which with lazy module loading is
//    the module's first use); grids up to
//    64 x 64 x 64 (powers of two, each in [16, 64]) fit.  Larger grids are
//    rejected with NS_ERR_SHAPE.
//  - The device address of the array is looked up with cudaGetSymbolAddress
//    on the first call on each device (with that device current) and kept
//    for the life of the process.  Make that first call before any stream
//    capture.  A device reset (cudaDeviceReset) after it is not supported:
//    the module is reloaded and the kept address is stale.
//  - A CUDA error already pending on the calling thread is left in place:
//    the call then returns NS_ERR_CUDA without launching anything.
//  - All calls share the array and it keeps the last call's contents; the
//    tables are rebuilt by every call and the spectrum is fully overwritten,
//    so nothing has to start at zero.  Calls that overlap on the GPU (two
//    streams, or two host threads) race on the array.
//  - Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {
bool fft_size_supported(int nx, int ny, int nz);
}

using namespace ns;

namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 19;  // 4 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Twiddles W_N^m = exp(-2 pi i m/N) of the four transforms and the inverse
// eigenvalues 1/(2 N lambda) (lambda as big_periodic_3D.f90:242-255; mean mode 0).
__global__ void noalloc_tables(double2* tw, int M, int nx, int ny, int nz, double* inv_lam, double dx, double dy,
                               double dz) {
  const int nxh = M + 1;
  const int ntw = M + (M / 2 + 1) + ny + nz;
  const long long nl = (long long)nxh * ny * nz;
  const double scale = 1.0 / (2.0 * (double)nx * (double)ny * (double)nz);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntw + nl;
       t += (long long)gridDim.x * blockDim.x) {
    if (t < ntw) {
      int m = (int)t, N;
      if (m < M) { N = M; }
      else if ((m -= M) < M / 2 + 1) { N = nx; }
      else if ((m -= M / 2 + 1) < ny) { N = ny; }
      else { m -= ny; N = nz; }
      double s, c;
      sincospi(2.0 * (double)m / (double)N, &s, &c);
      tw[t] = make_double2(c, -s);
    } else {
      const long long q = t - ntw;
      const int i = (int)(q % nxh), j = (int)((q / nxh) % ny), k = (int)(q / ((long long)nxh * ny));
      const double pi = 3.1415926535897932;
      const double sx = sin(pi * i / nx) / dx, sy = sin(pi * j / ny) / dy, sz = sin(pi * k / nz) / dz;
      const double lam = -4.0 * ((sx * sx + sy * sy) + sz * sz);
      inv_lam[q] = (i == 0 && j == 0 && k == 0) ? 0.0 : scale / lam;
    }
  }
}

bool pow2_in(int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

}  // namespace

extern "C" int ns_poisson_fft_noalloc(const double* rhs_dev, double* dp_dev, int nx, int ny, int nz, double lx,
                                      double ly, double lz, void* stream) {
  if (!rhs_dev || !dp_dev || !(lx > 0) || !(ly > 0) || !(lz > 0) || ((uintptr_t)rhs_dev & 15) ||
      ((uintptr_t)dp_dev & 7)) {
    std::fprintf(stderr, "ns_poisson_fft_noalloc: null or misaligned pointer, or non-positive length\n");
    return NS_ERR_ARG;
  }
  if (!pow2_in(nx, 16, 64) || !pow2_in(ny, 16, 64) || !pow2_in(nz, 16, 64)) {
    std::fprintf(stderr,
                 "ns_poisson_fft_noalloc: grid %d x %d x %d exceeds the static scratch "
                 "(powers of two in [16, 64] per axis, at most 64^3)\n", nx, ny, nz);
    return NS_ERR_SHAPE;
  }
  const int M = nx / 2, nxh = M + 1;
  const size_t n_spec = (size_t)nxh * ny * nz * 2;          // doubles of the half spectrum
  const size_t n_lam = (size_t)nxh * ny * nz;
  const size_t n_tw = (size_t)(M + M / 2 + 1 + ny + nz) * 2;
  if (n_spec + n_lam + n_tw > kNoAllocScratchDoubles) return NS_ERR_SHAPE;

  // An error left by the caller's earlier work is not ours to consume: report it, launch nothing.
  if (cudaPeekAtLastError() != cudaSuccess) {
    std::fprintf(stderr, "ns_poisson_fft_noalloc: a CUDA error is already pending: %s\n",
                 cudaGetErrorString(cudaPeekAtLastError()));
    return NS_ERR_CUDA;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NS_ERR_CUDA;
  double* base;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        std::fprintf(stderr, "ns_poisson_fft_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
        return NS_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<double*>(p);
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2* spec = reinterpret_cast<double2*>(base);  // 256-byte aligned
  double* inv_lam = base + n_spec;
  double2* tw = reinterpret_cast<double2*>(base + n_spec + n_lam + ((n_spec + n_lam) & 1));
  const double dx = lx / nx, dy = ly / ny, dz = lz / nz;

  noalloc_tables<<<152, 256, 0, st>>>(tw, M, nx, ny, nz, inv_lam, dx, dy, dz);
  if (cudaGetLastError() != cudaSuccess) return NS_ERR_CUDA;

  FftPlan P{};
  P.nx = nx; P.ny = ny; P.nz = nz; P.nxh = nxh; P.nxs = nxh;
  P.tw_x = tw;
  P.tw_xr = tw + M;
  P.tw_y = tw + M + (M / 2 + 1);
  P.tw_z = tw + M + (M / 2 + 1) + ny;
  P.inv_lam = inv_lam;
  P.dp_unaligned = 1;  // dp is the caller's (nx+2)^3 array: pairs (2m+1, 2m+2) are not 16-byte aligned

  // rhs (nx, ny, nz), Fortran order: cell slot (s, j, k) at (s-1) + nx (j-1) + nx ny (k-1)
  Layout Lr{};
  Lr.nx = nx; Lr.ny = ny; Lr.nz = nz;
  Lr.px = nx; Lr.sy = nx; Lr.sz = (long long)nx * ny;
  Lr.off = -1 - (long long)nx - (long long)nx * ny;
  // dp (nx+2, ny+2, nz+2), Fortran order: slot (i, j, k) at i + (nx+2) j + (nx+2)(ny+2) k
  Layout Ld{};
  Ld.nx = nx; Ld.ny = ny; Ld.nz = nz;
  Ld.px = nx + 2; Ld.sy = nx + 2; Ld.sz = (long long)(nx + 2) * (ny + 2);
  Ld.off = 0;

  DivArgs d{};
  d.L = Lr;
  d.rhs = rhs_dev;
  d.one = 1.0;
  d.mzero = -0.0;
  if (launch_fft_poisson(P, d, spec, dp_dev, Ld, st, Marker{}) != cudaSuccess) return NS_ERR_CUDA;
  const int pbc[3] = {1, 1, 1};
  if (launch_pr_bc(Ld, dp_dev, FaceSet{}, pbc, dx, dy, dz, st) != cudaSuccess) return NS_ERR_CUDA;
  return NS_OK;
}
