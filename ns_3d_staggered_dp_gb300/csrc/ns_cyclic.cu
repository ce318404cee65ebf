// The z stage of the all-periodic Poisson solve as cyclic tridiagonal line
// solves (big_periodic_3D.f90:526-548 solves the whole problem with a 3D r2c
// FFT; this stage replaces its z FFT, 1/lambda and z IFFT).
//
// After the x and y transforms every spectrum line along z, mode (kx, ky), is
// the periodic system
//   p[j-1] - c p[j] + p[j+1] = rs R[j],  c = 2 - h_z^2 (lambda_x + lambda_y),
// indices mod nz, rs = h_z^2 * scale * nz (the z FFT pair it replaces was
// unnormalised), whose exact solution the z FFT, the divide by the 3D
// eigenvalue and the z IFFT give.  Here it is solved directly:
// Sherman-Morrison on T = the system without its corners and with
// T[0][0] = -2c, T[n-1][n-1] = -c - 1/c (gamma = c), u = (c, 0, .., 0, 1),
// v = (1, 0, .., 0, 1/c):
//   y = T^-1 rs R,  q = T^-1 u,  x = y - (y[0] + y[n-1]/c) / (1 + q[0] + q[n-1]/c) q.
// T's Thomas multipliers m, q, and w = rs T^-1 e0 (so y[0] = w . R, summed in
// the forward walk, which gives the correction before the backward walk)
// depend on the mode only and are tabulated once per plan, laid out like the
// spectrum.  Per complex unknown that is 10 FP64 operations against about 47
// for the FFT pair.
//
// The mode (0, 0) is singular (c = 2): the FFT solve drops its mean
// (lambda(0) = +Inf), i.e. gives the zero-mean solution of the system with
// the right-hand side's mean removed.  Here, by linearity, through the same
// walk with its own tables: p[0] pinned to zero and the Dirichlet system on
// p[1..n-1] solved (m[0] = 0), the right-hand side's mean taken out through
// alpha q with q = D^-1 1, and the mean of the result (a fixed functional of
// the data, V . R) subtracted as the line is written.
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

namespace {

constexpr int CYC_T = 128;  // lines per CTA

// One thread per mode t = kx + nxh*ky; tables at t + j*S (S = nxh*ny).
// V: the singular line's mean functional (n entries).
__global__ void __launch_bounds__(CYC_T) cyc_table_kernel(FftPlan P, double* __restrict__ M, double* __restrict__ W,
                                                          double* __restrict__ Q, double2* __restrict__ CS,
                                                          double* __restrict__ V) {
  const int S = P.nxh * P.ny;
  const int t = blockIdx.x * CYC_T + threadIdx.x;
  if (t >= S) return;
  const int n = P.nz;
  const int kx = t % P.nxh, ky = t / P.nxh;
  if (t == 0) {
    // The singular line as the general walk: the Dirichlet system on p[1..n-1]
    // (p[0] pinned: m[0] = 0, diagonal -2), q = e = D^-1 1 (e[0] = 0), w = rs/n
    // (so y0 = rs mean(R) and alpha q removes the right-hand side's mean), and
    // V with V . R = mean of the result, subtracted as the line is written.
    double m = 0.0;
    M[0] = 0.0;
    for (int j = 1; j < n; ++j) {
      m = 1.0 / (-2.0 - m);
      M[(long long)j * S] = m;
    }
    double de = 0.0;
    Q[0] = 0.0;
    for (int j = 1; j < n; ++j) {
      de = (1.0 - de) * M[(long long)j * S];
      Q[(long long)j * S] = de;
    }
    double xe = de, E = de;
    for (int j = n - 2; j >= 1; --j) {
      xe = Q[(long long)j * S] - M[(long long)j * S] * xe;
      Q[(long long)j * S] = xe;
      E += xe;
    }
    for (int j = 0; j < n; ++j) {
      W[(long long)j * S] = P.cyc_rs / n;
      V[j] = P.cyc_rs / n * (Q[(long long)j * S] - E / n);
    }
    CS[0] = make_double2(0.0, 1.0);
    return;
  }
  const double c = 2.0 - P.cyc_h2 * (P.eig_x[kx] + P.eig_o[ky]);
  const double ic = 1.0 / c;
  // multipliers of T: m_j = 1 / (T_jj - m_{j-1})
  double m = 0.0;
  for (int j = 0; j < n; ++j) {
    const double tj = j == 0 ? -2.0 * c : (j == n - 1 ? -c - ic : -c);
    m = 1.0 / (tj - m);
    M[(long long)j * S + t] = m;
  }
  // q = T^-1 u and w = T^-1 e0 (forward into the tables, then backward in place)
  double dq = 0.0, dw = 0.0;
  for (int j = 0; j < n; ++j) {
    const double mj = M[(long long)j * S + t];
    const double uj = j == 0 ? c : (j == n - 1 ? 1.0 : 0.0);
    const double ej = j == 0 ? 1.0 : 0.0;
    dq = (uj - dq) * mj;
    dw = (ej - dw) * mj;
    Q[(long long)j * S + t] = dq;
    W[(long long)j * S + t] = dw;
  }
  double xq = dq, xw = dw;
  for (int j = n - 2; j >= 0; --j) {
    const double mj = M[(long long)j * S + t];
    xq = Q[(long long)j * S + t] - mj * xq;
    xw = W[(long long)j * S + t] - mj * xw;
    Q[(long long)j * S + t] = xq;
    W[(long long)j * S + t] = xw;
  }
  for (int j = 0; j < n; ++j) W[(long long)j * S + t] *= P.cyc_rs;
  const double q0 = Q[t], qn = Q[(long long)(n - 1) * S + t];
  CS[t] = make_double2(ic, 1.0 / (1.0 + q0 + qn * ic));
}

// One thread per z line (mode t): forward walk (Thomas with T's multipliers,
// y[0] = w . R alongside), the Sherman-Morrison coefficient, backward walk
// writing x = y - alpha q.
// SING: the singular line (t = 0), which ends by removing the mean of its
// result; the other lines skip that subtraction.
template <bool SING>
__device__ __forceinline__ void cyc_walk(const FftPlan& P, double2* __restrict__ spec, int t) {
  const int S = P.nxh * P.ny;
  const int n = P.nz;
  const double rs = P.cyc_rs;
  const double* __restrict__ M = P.cyc_m + t;
  double2* g = spec + t;
  // the singular line (t = 0) runs the same walk on its own tables and ends
  // by removing the mean of its result, beta = V . R (load-only pre-pass)
  double2 beta = make_double2(0.0, 0.0);
  if (SING) {
#pragma unroll 8
    for (int j = 0; j < n; ++j) {
      const double2 r = g[(long long)j * S];
      const double v = __ldg(P.cyc_v + j);
      beta.x = fma(v, r.x, beta.x);
      beta.y = fma(v, r.y, beta.y);
    }
  }
  const double* __restrict__ W = P.cyc_w + t;
  const double* __restrict__ Q = P.cyc_q + t;
  // The next PD unknowns of the line (and their table entries) are loaded
  // into registers before the current PD are processed: the loads would
  // otherwise wait behind the stores to the same line.
  constexpr int PD = 8;
  double2 rb[PD], rn[PD];
  double mb[PD], mn[PD], wb[PD], wn[PD];
#pragma unroll
  for (int q = 0; q < PD; ++q) {
    const bool in = q < n;
    rb[q] = in ? g[(long long)q * S] : make_double2(0.0, 0.0);
    mb[q] = in ? __ldg(M + (long long)q * S) : 0.0;
    wb[q] = in ? __ldg(W + (long long)q * S) : 0.0;
  }
  double2 d = make_double2(0.0, 0.0), y0 = make_double2(0.0, 0.0);
  for (int j0 = 0; j0 < n; j0 += PD) {
#pragma unroll
    for (int q = 0; q < PD; ++q) {
      const int j = j0 + PD + q;
      const bool in = j < n;
      rn[q] = in ? g[(long long)j * S] : make_double2(0.0, 0.0);
      mn[q] = in ? __ldg(M + (long long)j * S) : 0.0;
      wn[q] = in ? __ldg(W + (long long)j * S) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < PD; ++q) {
      const int j = j0 + q;
      if (j < n) {
        d.x = fma(rb[q].x, rs, -d.x) * mb[q];
        d.y = fma(rb[q].y, rs, -d.y) * mb[q];
        y0.x = fma(wb[q], rb[q].x, y0.x);
        y0.y = fma(wb[q], rb[q].y, y0.y);
        g[(long long)j * S] = d;
      }
    }
#pragma unroll
    for (int q = 0; q < PD; ++q) { rb[q] = rn[q]; mb[q] = mn[q]; wb[q] = wn[q]; }
  }
  const double2 cs = __ldg(P.cyc_s + t);  // (1/c, 1/(1 + q[0] + q[n-1]/c))
  const double ax = fma(d.x, cs.x, y0.x) * cs.y, ay = fma(d.y, cs.x, y0.y) * cs.y;
  // backward walk from j = n-1 (where y = d), PD unknowns ahead (all of them
  // written by this thread's forward walk, read back in program order)
  double2 p = d;
  double qb[PD], qn[PD];
#pragma unroll
  for (int q = 0; q < PD; ++q) {
    const int j = n - 2 - q;
    const bool in = j >= 0;
    rb[q] = in ? g[(long long)j * S] : make_double2(0.0, 0.0);
    mb[q] = in ? __ldg(M + (long long)j * S) : 0.0;
    qb[q] = in ? __ldg(Q + (long long)j * S) : 0.0;
  }
  {
    const double q = __ldg(Q + (long long)(n - 1) * S);
    double2 x = make_double2(fma(-ax, q, p.x), fma(-ay, q, p.y));
    if (SING) { x.x -= beta.x; x.y -= beta.y; }
    g[(long long)(n - 1) * S] = x;
  }
  for (int j0 = n - 2; j0 >= 0; j0 -= PD) {
#pragma unroll
    for (int q = 0; q < PD; ++q) {
      const int j = j0 - PD - q;
      const bool in = j >= 0;
      rn[q] = in ? g[(long long)j * S] : make_double2(0.0, 0.0);
      mn[q] = in ? __ldg(M + (long long)j * S) : 0.0;
      qn[q] = in ? __ldg(Q + (long long)j * S) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < PD; ++q) {
      const int j = j0 - q;
      if (j >= 0) {
        p.x = fma(-mb[q], p.x, rb[q].x);
        p.y = fma(-mb[q], p.y, rb[q].y);
        double2 x = make_double2(fma(-ax, qb[q], p.x), fma(-ay, qb[q], p.y));
        if (SING) { x.x -= beta.x; x.y -= beta.y; }
        g[(long long)j * S] = x;
      }
    }
#pragma unroll
    for (int q = 0; q < PD; ++q) { rb[q] = rn[q]; mb[q] = mn[q]; qb[q] = qn[q]; }
  }
}

// Threads 0..S-2 take the lines 1..S-1; the singular line 0 goes to the
// first thread of a warp of its own (a warp running both walks would take as
// long as the two together).
__host__ __device__ __forceinline__ int cyc_sing_thread(int S) { return (S - 1 + 31) / 32 * 32; }

__global__ void __launch_bounds__(CYC_T) cyc_solve_kernel(FftPlan P, double2* __restrict__ spec) {
  const int S = P.nxh * P.ny;
  const int g = blockIdx.x * CYC_T + threadIdx.x;
  if (g < S - 1) cyc_walk<false>(P, spec, g + 1);
  else if (g == cyc_sing_thread(S)) cyc_walk<true>(P, spec, 0);
}

}  // namespace

size_t cyc_table_doubles(const FftPlan& P) {
  const size_t S = (size_t)P.nxh * P.ny;
  return 3 * S * P.nz + 2 * S + P.nz;
}

cudaError_t launch_cyc_table(FftPlan& P, double* buf, cudaStream_t st) {
  const size_t S = (size_t)P.nxh * P.ny, V = S * P.nz;
  double* M = buf;
  double* W = buf + V;
  double* Q = buf + 2 * V;
  double2* CS = reinterpret_cast<double2*>(buf + 3 * V);
  double* mv = buf + 3 * V + 2 * S;
  cyc_table_kernel<<<(unsigned)((S + CYC_T - 1) / CYC_T), CYC_T, 0, st>>>(P, M, W, Q, CS, mv);
  P.cyc_m = M;
  P.cyc_w = W;
  P.cyc_q = Q;
  P.cyc_s = CS;
  P.cyc_v = mv;
  return cudaGetLastError();
}

cudaError_t launch_cyc_z_solve(const FftPlan& P, double2* spec, cudaStream_t st) {
  const int threads = cyc_sing_thread(P.nxh * P.ny) + 1;
  cyc_solve_kernel<<<(unsigned)((threads + CYC_T - 1) / CYC_T), CYC_T, 0, st>>>(P, spec);
  return cudaGetLastError();
}

}  // namespace ns
