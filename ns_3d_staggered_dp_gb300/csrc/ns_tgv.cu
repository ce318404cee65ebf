// TGV (NS_functions.f90:18-50): the 2D Taylor-Green vortex on a tensor grid,
// the initial condition of the reference's test drivers.
//
//   u(i,j,:) =  cos(x_i) sin(y_j) e
//   v(i,j,:) = -sin(x_i) cos(y_j) e
//   p(i,j,:) = -0.25 (cos(2 x_i) + cos(2 y_j)) e e,     e = exp(-2 nu t)
//
// Every product is rounded in the reference's order (no contraction into an
// FMA), so the fields differ from a host evaluation only through the sine and
// cosine values.  The reference never writes w; neither does this routine.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/ns_gpu.h"

namespace {

// One thread per (i, j) column writes all nz planes of that column.
__global__ void tgv_kernel(const double* __restrict__ x, int nx, const double* __restrict__ y, int ny, int nz,
                           double e, double* __restrict__ u, double* __restrict__ v, double* __restrict__ p) {
  const long long plane = (long long)nx * ny;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < plane;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx), j = (int)(q / nx);
    const double xi = x[i], yj = y[j];
    double uu = 0.0, vv = 0.0, pp = 0.0;
    if (u) uu = __dmul_rn(__dmul_rn(cos(xi), sin(yj)), e);
    if (v) vv = __dmul_rn(__dmul_rn(-sin(xi), cos(yj)), e);
    if (p) pp = __dmul_rn(__dmul_rn(__dmul_rn(-0.25, __dadd_rn(cos(2.0 * xi), cos(2.0 * yj))), e), e);
    for (int k = 0; k < nz; ++k) {
      const long long g = q + plane * k;
      if (u) u[g] = uu;
      if (v) v[g] = vv;
      if (p) p[g] = pp;
    }
  }
}

}  // namespace

extern "C" int ns_tgv(const double* x, int nx, const double* y, int ny, int nz, double t, double nu, double* u,
                      double* v, double* w, double* p) {
  (void)w;  // the reference accepts w and leaves it as it is
  if (!x || !y || nx < 1 || ny < 1 || nz < 1) return NS_ERR_ARG;
  if (!u && !v && !p) return NS_OK;
  const size_t n = (size_t)nx * ny * nz;
  const double e = std::exp(-2.0 * nu * t);
  cudaStream_t st = nullptr;
  double* buf = nullptr;
  int status = NS_OK;
  const int nout = (u ? 1 : 0) + (v ? 1 : 0) + (p ? 1 : 0);
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NS_ERR_CUDA;
  if (cudaMallocAsync(&buf, (nx + ny + nout * n) * sizeof(double), st) != cudaSuccess) {
    cudaStreamDestroy(st);
    return NS_ERR_NOMEM;
  }
  double* dx = buf;
  double* dy = buf + nx;
  double* out = dy + ny;
  double* du = u ? out : nullptr;
  double* dv = v ? out + (u ? n : 0) : nullptr;
  double* dp = p ? out + (size_t)(nout - 1) * n : nullptr;
  cudaError_t err = cudaMemcpyAsync(dx, x, nx * sizeof(double), cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess) err = cudaMemcpyAsync(dy, y, ny * sizeof(double), cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess) {
    const long long plane = (long long)nx * ny;
    const int grid = (int)std::min<long long>((plane + 255) / 256, 152LL * 8);
    tgv_kernel<<<grid, 256, 0, st>>>(dx, nx, dy, ny, nz, e, du, dv, dp);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess && u) err = cudaMemcpyAsync(u, du, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess && v) err = cudaMemcpyAsync(v, dv, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess && p) err = cudaMemcpyAsync(p, dp, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(buf, st);
  if (cudaStreamSynchronize(st) != cudaSuccess || err != cudaSuccess) status = NS_ERR_CUDA;
  cudaStreamDestroy(st);
  return status;
}
