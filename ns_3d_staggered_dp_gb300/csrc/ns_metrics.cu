// Re-simulation error metrics on the device and the err_file writer
// (re_simulation_sub_tstep_interBC_combine.f90:813-834 and :913-931).
//
// After each re-simulated step the reference compares the sub-block's
// u, v, w, p with the parent's data over the same index maps (u_sub =
// u(idx_xu, idx_yu, idx_zu), big_periodic_3D.f90:665-669), over the full
// padded arrays:
//   rms_vel(1..4) = rms(u_sub), rms(v_sub), rms(w_sub), rms(p_sub)
//   err_vel(1..4) = maxval(|x - x_sub|) / rms(x_sub)        (u, v, w, p)
//   err_vel(5..7) = mean(|x - x_sub|) / rms(x_sub)          (u, v, w)
//   err_vel(8)    = maxval(|oz - oz_sub|) / rms(oz_sub),
//                   oz = diff(v,1,1)/dx - diff(u,1,2)/dy on (nx+1, ny+1, nz+2)
// with mean(a) = sum(a)/size(a) and rms(a) = sqrt(sum(a*a)/size(a))
// (other_utility.f90:110-129).
//
// A sub-block slot s maps to the parent slot s + (x0-1, y0-1, z0-1) for every
// field (the index maps are x0 + 0..n along every axis, and a slot is the
// reference index on a face axis, the index minus one on a cell axis).  One
// kernel reduces the five quantities of every box: CTAs (chunk, quantity,
// box) write partial sums and maxima, which the host combines in a fixed
// order, so the result does not depend on scheduling.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"
#include "ns_session.cuh"

namespace ns {

namespace {

constexpr int kMetricThreads = 256;

// Reference extent of quantity q (0..3 u, v, w, p; 4 the vorticity) along each axis, and the slot of index 0.
__device__ __forceinline__ void q_extent(const Layout& L, int q, int& ex, int& ey, int& ez, int& sx, int& sy, int& sz) {
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  if (q == 4) {  // oz on (nx+1, ny+1, nz+2): slots x 1..nx+1, y 1..ny+1, z 0..nz+1
    ex = nx + 1; ey = ny + 1; ez = nz + 2; sx = 1; sy = 1; sz = 0;
    return;
  }
  ex = (q == 0) ? nx + 1 : nx + 2;
  ey = (q == 1) ? ny + 1 : ny + 2;
  ez = (q == 2) ? nz + 1 : nz + 2;
  sx = (q == 0) ? 1 : 0;
  sy = (q == 1) ? 1 : 0;
  sz = (q == 2) ? 1 : 0;
}

__global__ void __launch_bounds__(kMetricThreads) metrics_kernel(const MetricBox* __restrict__ boxes,
                                                                  double* __restrict__ partial) {
  const int chunk = blockIdx.x, nchunk = gridDim.x, q = blockIdx.y, box = blockIdx.z;
  const MetricBox& B = boxes[box];
  int ex, ey, ez, sx, sy, sz;
  q_extent(B.La, q, ex, ey, ez, sx, sy, sz);
  const long long n = (long long)ex * ey * ez;
  double s2 = 0.0, s1 = 0.0, mx = 0.0;
  for (long long t = (long long)chunk * blockDim.x + threadIdx.x; t < n; t += (long long)nchunk * blockDim.x) {
    const int i = (int)(t % ex);
    const long long r = t / ex;
    const int j = (int)(r % ey);
    const int k = (int)(r / ey);
    const long long ga = B.La.at(sx + i, sy + j, sz + k);
    const long long gb = B.Lb.at(sx + i + B.ox, sy + j + B.oy, sz + k + B.oz);
    double x, y;
    if (q < 4) {
      x = B.a[q][ga];
      y = B.b[q][gb];
    } else {
      x = (B.a[1][ga] - B.a[1][ga - 1]) * B.idx - (B.a[0][ga] - B.a[0][ga - B.La.sy]) * B.idy;
      y = (B.b[1][gb] - B.b[1][gb - 1]) * B.idx - (B.b[0][gb] - B.b[0][gb - B.Lb.sy]) * B.idy;
    }
    const double d = fabs(x - y);
    s2 = fma(y, y, s2);
    s1 += d;
    mx = fmax(mx, d);
  }
  __shared__ double r2[kMetricThreads / 32], r1[kMetricThreads / 32], rm[kMetricThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) { r2[w] = s2; r1[w] = s1; rm[w] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a2 = 0.0, a1 = 0.0, am = 0.0;
    for (int v = 0; v < kMetricThreads / 32; ++v) { a2 += r2[v]; a1 += r1[v]; am = fmax(am, rm[v]); }
    double* o = partial + 3 * ((long long)(box * 5 + q) * nchunk + chunk);
    o[0] = a2; o[1] = a1; o[2] = am;
  }
}

}  // namespace

cudaError_t launch_metrics(const MetricBox* dev_boxes, const std::vector<MetricBox>& host_boxes, double* out,
                           cudaStream_t st) {
  const int nbox = (int)host_boxes.size();
  if (nbox == 0) return cudaSuccess;
  long long biggest = 0;
  for (const MetricBox& B : host_boxes)
    biggest = std::max<long long>(biggest, (long long)(B.La.nx + 2) * (B.La.ny + 2) * (B.La.nz + 2));
  const int nchunk = (int)std::min<long long>(64, std::max<long long>(1, biggest / (kMetricThreads * 64)));
  const size_t np = (size_t)nbox * 5 * nchunk * 3;
  double* partial = nullptr;
  cudaError_t e = cudaMallocAsync(&partial, np * sizeof(double), st);
  if (e != cudaSuccess) return e;
  metrics_kernel<<<dim3(nchunk, 5, nbox), kMetricThreads, 0, st>>>(dev_boxes, partial);
  e = cudaGetLastError();
  std::vector<double> hp(np);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), partial, np * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(partial, st);
  if (e != cudaSuccess) return e;
  for (int bx = 0; bx < nbox; ++bx) {
    const Layout& L = host_boxes[bx].La;
    double s2[5], s1[5], mx[5], cnt[5];
    for (int q = 0; q < 5; ++q) {
      s2[q] = s1[q] = mx[q] = 0.0;
      for (int c = 0; c < nchunk; ++c) {
        const double* p = hp.data() + 3 * ((size_t)(bx * 5 + q) * nchunk + c);
        s2[q] += p[0];
        s1[q] += p[1];
        mx[q] = std::fmax(mx[q], p[2]);
      }
      const int ex = q == 4 ? L.nx + 1 : (q == 0 ? L.nx + 1 : L.nx + 2);
      const int ey = q == 4 ? L.ny + 1 : (q == 1 ? L.ny + 1 : L.ny + 2);
      const int ez = q == 4 ? L.nz + 2 : (q == 2 ? L.nz + 1 : L.nz + 2);
      cnt[q] = (double)ex * ey * ez;
    }
    double* o = out + 12 * (size_t)bx;
    double rms[5];
    for (int q = 0; q < 5; ++q) rms[q] = std::sqrt(s2[q] / cnt[q]);
    for (int q = 0; q < 4; ++q) o[q] = rms[q];
    for (int q = 0; q < 4; ++q) o[4 + q] = mx[q] / rms[q];
    for (int q = 0; q < 3; ++q) o[8 + q] = (s1[q] / cnt[q]) / rms[q];
    o[11] = mx[4] / rms[4];
  }
  return cudaSuccess;
}

}  // namespace ns

using namespace ns;

extern "C" {

int ns_error_metrics(ns_handle* h, const double* u_ref, const double* v_ref, const double* w_ref, const double* p_ref,
                     double* out) {
  if (!h) return NS_ERR_ARG;
  if (!u_ref || !v_ref || !w_ref || !p_ref || !out) return api_fail(h, NS_ERR_ARG, "metrics: all arrays are required");
  // the reference fields go to the step's scratch fields (free between steps)
  double* scratch[4] = {h->us, h->vs, h->ws, h->dp};
  const double* refs[4] = {u_ref, v_ref, w_ref, p_ref};
  for (int f = 0; f < 4; ++f) {
    const cudaError_t e = api_h2d_field(h, scratch[f], refs[f], f);
    if (e != cudaSuccess) return api_fail(h, NS_ERR_CUDA, std::string("metrics upload: ") + cudaGetErrorString(e));
  }
  MetricBox B{};
  B.La = h->L; B.Lb = h->L;
  const double* st[4] = {h->u, h->v, h->w, h->p};
  for (int f = 0; f < 4; ++f) { B.a[f] = st[f]; B.b[f] = scratch[f]; }
  B.ox = B.oy = B.oz = 0;
  B.idx = 1.0 / h->dx; B.idy = 1.0 / h->dy;
  MetricBox* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(MetricBox), h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, &B, sizeof(MetricBox), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_metrics(d, std::vector<MetricBox>{B}, out, h->stream);
  if (d) cudaFreeAsync(d, h->stream);
  api_mark(h, "metrics", 1);
  if (e != cudaSuccess) return api_fail(h, NS_ERR_CUDA, std::string("metrics: ") + cudaGetErrorString(e));
  return NS_OK;
}

int ns_write_err_csv(const char* path, int kind, int nrows, const double* rows) {
  if (!path || (kind != 0 && kind != 1) || nrows < 0 || (nrows > 0 && !rows)) return NS_ERR_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return NS_ERR_ARG;
  const int ncol = kind == 0 ? 8 : 4;
  if (kind == 0)
    std::fputs("time_step, rel_err_u, rel_err_v, rel_err_w, rel_err_p, rel_err_u_m, rel_err_v_m, rel_err_w_m, "
               "rel_err_p_m\n", f);
  else
    std::fputs("time_step, rms_u, rms_v, rms_w, rms_p\n", f);
  for (int j = 0; j < nrows; ++j) {
    std::fprintf(f, "%d", j);
    for (int c = 0; c < ncol; ++c) std::fprintf(f, ",%12.5E", rows[(size_t)j * ncol + c]);
    std::fputc('\n', f);
  }
  const int bad = std::ferror(f);
  std::fclose(f);
  return bad ? NS_ERR_ARG : NS_OK;
}

}  // extern "C"
