// Periodic pressure Poisson solve by FFT (big_periodic_3D.f90:215-256 plan and
// eigenvalues, :498-548 solve): RHS = div(u*)/dt, r2c 3D DFT, divide by
// lambda = -4 sum sin^2(pi k/n)/h^2 (lambda(0,0,0) = +Inf, so the mean mode is
// zeroed), c2r with 1/(nx ny nz), dp interior.
//
// Five kernels, each streaming lines through shared memory:
//   x-forward : divergence of u*, v*, w* fused with the r2c transform of each
//               x-line (an nx/2-point complex FFT of the packed even/odd
//               samples and the split into nx/2+1 bins)
//   y-forward : complex FFT along y
//   z-solve   : complex FFT along z, multiply by 1/(lambda * scale), inverse
//               FFT along z, all on the line held on chip
//   y-inverse, x-inverse (c2r, writes dp slots 1..nx)
// A line of N = R1*R2 points is transformed in two register passes
// ("four-step"): R1 threads each do an R2-point DFT, a twiddle multiply and a
// shared-memory transpose, then R1-point DFTs.  Register DFTs are radix-2
// decimation-in-time with every butterfly in Linzer-Feig FMA form (6 FMAs
// for a general twiddle, 4 for the trivial ones).  The spectrum is
// (nx/2+1, ny, nz) complex with x fastest, as the reference's DFTI
// descriptor (cstrides, :217-221).  The overall scale of the forward split,
// the inverse split and the 1/N of the backward transform are folded into
// the inverse-eigenvalue table.
#include "ns_fft_core.cuh"
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {
namespace {

// Line geometry of a y/z-pass block over the outer indices [o0, o1) (kz for
// a y pass, ky for a z pass).  Blocks with blockIdx.x < nxh/LPC own LPC
// consecutive kx at one outer index; the last column of blocks owns the
// Nyquist plane kx = nx/2, with lanes over LPC consecutive outer indices.
struct LineGeo {
  long long base;
  bool valid;
};
__host__ __device__ __forceinline__ int yz_nblk(int nxh, int LPC) { return (nxh - 1 + LPC - 1) / LPC; }
__device__ __forceinline__ LineGeo yz_line(int axis, int nxh, int ny, int l, int LPC, int o0, int o1) {
  const int M = nxh - 1;
  const int nblk = yz_nblk(nxh, LPC);
  LineGeo G;
  int kx, o;
  if ((int)blockIdx.x < nblk) {
    kx = blockIdx.x * LPC + l;
    o = o0 + blockIdx.y;
    G.valid = kx < M;
    if (!G.valid) kx = 0;
  } else {
    kx = M;
    o = o0 + blockIdx.y * LPC + l;
    G.valid = o < o1;
    if (!G.valid) o = o0;
  }
  if (axis == 1) G.base = kx + (long long)nxh * ny * o;  // line along y at (kx, kz = o)
  else G.base = kx + (long long)nxh * o;                 // line along z at (kx, ky = o)
  return G;
}

// Complex FFT along y (AXIS 1) or z (AXIS 2), forward (DIR -1) or inverse.
template <int AXIS, int N, int DIR>
__global__ void __launch_bounds__(lpc<N>() * Split<N>::R1) fft_yz_kernel(FftPlan P, double2* __restrict__ spec, FOne c,
                                                                          int o0, int o1) {
  using F = YZ<N>;
  constexpr int LPC = F::LPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* sb = reinterpret_cast<double2*>(smem_raw);
  const int l = threadIdx.x, t = threadIdx.y;
  const LineGeo G = yz_line(AXIS, P.nxh, P.ny, l, LPC, o0, o1);
  if ((int)blockIdx.x == yz_nblk(P.nxh, LPC) && (int)(blockIdx.y * LPC) >= o1 - o0) return;  // whole block idle
  double2* g = spec + G.base;
  const long long st = AXIS == 1 ? (long long)P.nxh : (long long)P.nxh * P.ny;
  const double2* tw = AXIS == 1 ? P.tw_y : P.tw_z;
  if (DIR < 0) {
    if (G.valid) F::fwdA(g, st, sb, tw, l, t, c);
    __syncthreads();
    double2 xk[F::KQ][F::R1];
    F::fwdB(xk, sb, l, t, c);
    if (G.valid) {
#pragma unroll
      for (int q = 0; q < F::KQ; ++q)
#pragma unroll
        for (int k1 = 0; k1 < F::R1; ++k1) g[(long long)(t + F::T * q + F::R2 * k1) * st] = xk[q][k1];
    }
  } else {
    double2 xk[F::KQ][F::R1];
#pragma unroll
    for (int q = 0; q < F::KQ; ++q)
#pragma unroll
      for (int k1 = 0; k1 < F::R1; ++k1)
        xk[q][k1] = G.valid ? g[(long long)(t + F::T * q + F::R2 * k1) * st] : make_double2(0.0, 0.0);
    F::invA(xk, sb, tw, l, t, c);
    __syncthreads();
    if (G.valid) F::invB(g, st, sb, l, t, c);
  }
}

// The session's FFT-based y transform of a packed-x box (dct_y_body).
template <int N, bool FWD, int PB>
__global__ void __launch_bounds__(lpc<N>() * Split<N>::R1) dct_y_kernel(FftPlan P, double2* __restrict__ spec, FOne c) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  dct_y_body<N, FWD, PB>(P, spec, reinterpret_cast<double2*>(smem_raw), blockIdx.x, threadIdx.x, threadIdx.y, c);
}

template <int N>
__global__ void __launch_bounds__(lpc<N>() * Split<N>::R1) fft_z_solve_kernel(FftPlan P, double2* __restrict__ spec, FOne c) {
  using F = YZ<N>;
  constexpr int LPC = F::LPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* sb = reinterpret_cast<double2*>(smem_raw);
  const int l = threadIdx.x, t = threadIdx.y;
  if ((int)blockIdx.x == yz_nblk(P.nxh, LPC) && blockIdx.y * LPC >= (unsigned)P.ny) return;
  const LineGeo G = yz_line(2, P.nxh, P.ny, l, LPC, 0, P.ny);
  double2* g = spec + G.base;
  const double* lam = P.inv_lam + G.base;
  const long long st = (long long)P.nxh * P.ny;
  if (G.valid) F::fwdA(g, st, sb, P.tw_z, l, t, c);
  __syncthreads();
  double2 xk[F::KQ][F::R1];
  F::fwdB(xk, sb, l, t, c);
#pragma unroll
  for (int q = 0; q < F::KQ; ++q)
#pragma unroll
    for (int k1 = 0; k1 < F::R1; ++k1) {
      const int kz = t + F::T * q + F::R2 * k1;
      const double s = G.valid ? __ldg(lam + (long long)kz * st) : 0.0;
      xk[q][k1].x = fmul(c, xk[q][k1].x, s);
      xk[q][k1].y = fmul(c, xk[q][k1].y, s);
      // singular mode of a Neumann/periodic mix: fixed mean (NS_functions.f90:1576-1577)
      if (P.has_mean && G.valid && G.base == 0 && kz == 0) xk[q][k1] = make_double2(P.mean_val, 0.0);
    }
  __syncthreads();
  F::invA(xk, sb, P.tw_z, l, t, c);
  __syncthreads();
  if (G.valid) F::invB(g, st, sb, l, t, c);
}

// ---------------------------------------------------------------------------
// x passes: T threads per line are consecutive lanes (lines are contiguous).
// Shared buffer per line: R1 rows of (R2 + 1) entries, then the packed
// M-point spectrum for the real/complex split.
// ---------------------------------------------------------------------------
template <int M>
struct XP {
  static constexpr int R1 = Split<M>::R1, R2 = Split<M>::R2, T = R1, KQ = R2 / T;
  static constexpr int LINES = 256 / T;          // lines per CTA
  static constexpr int ROW = R2 + 1;             // padded row (bank spread)
  static constexpr int LS = (R1 * ROW > M + 2) ? R1 * ROW : M + 2;  // transpose area, reused by the split
  __device__ static __forceinline__ int sidx(int r, int q) { return r * ROW + q; }
};

template <int M, bool FROM_RHS, bool HAS_BC>
__global__ void __launch_bounds__(256) fft_x_fwd_kernel(FftPlan P, DivArgs d, double2* __restrict__ spec) {
  using X = XP<M>;
  constexpr int R1 = X::R1, R2 = X::R2, T = X::T, KQ = X::KQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const FOne c{d.one, d.mzero};
  const int t = threadIdx.x, l = threadIdx.y;
  const int line = blockIdx.x * X::LINES + l;
  const Layout L = d.L;
  const int ny = L.ny, nz = L.nz;
  const bool valid = line < ny * nz;
  const int j = valid ? 1 + line % ny : 1;
  const int k = valid ? 1 + line / ny : 1;
  double2* sb = reinterpret_cast<double2*>(smem_raw) + (long long)l * X::LS;
  double2* zb = sb;  // the split area reuses the transpose area after a barrier
  const FOne& cc = c;
  // Step A: packed input z[m] = r[2m] + i r[2m+1], m = n1 + R1 n2, n1 = t.
  {
    double2 x[R2];
    const double* us = d.us + L.at(0, j, k);
    const double* vs0 = d.vs + L.at(0, j, k);
    const double* vs1 = d.vs + L.at(0, j + 1, k);
    const double* ws0 = d.ws + L.at(0, j, k);
    const double* ws1 = d.ws + L.at(0, j, k + 1);
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      const int m = t + R1 * n2;
      const int s = 2 * m + 1;  // cell slots s, s+1
      if (FROM_RHS) {  // a given Poisson right-hand side in the cell slots
        x[n2] = *reinterpret_cast<const double2*>(d.rhs + L.at(s, j, k));
        continue;
      }
      const double2 ua = *reinterpret_cast<const double2*>(us + s);
      const double ub = us[s + 2];
      const double2 va = *reinterpret_cast<const double2*>(vs0 + s);
      const double2 vb = *reinterpret_cast<const double2*>(vs1 + s);
      const double2 wa = *reinterpret_cast<const double2*>(ws0 + s);
      const double2 wb = *reinterpret_cast<const double2*>(ws1 + s);
      double r0 = fmul(cc, fsub(cc, ua.y, ua.x), d.cdx);
      r0 = fma(fsub(cc, vb.x, va.x), d.cdy, r0);
      r0 = fma(fsub(cc, wb.x, wa.x), d.cdz, r0);
      double r1 = fmul(cc, fsub(cc, ub, ua.y), d.cdx);
      r1 = fma(fsub(cc, vb.y, va.y), d.cdy, r1);
      r1 = fma(fsub(cc, wb.y, wa.y), d.cdz, r1);
      if (HAS_BC) {  // pr_bc_staggered_modify_rhs on the wall cells of y and z
        r0 += P.bc_term(s, j, k);
        r1 += P.bc_term(s + 1, j, k);
      }
      x[n2] = make_double2(r0, r1);
    }
    dft<R2, -1>(x, cc);
    sb[X::sidx(t, 0)] = x[0];
#pragma unroll
    for (int k2 = 1; k2 < R2; ++k2) sb[X::sidx(t, k2)] = cmul(cc, x[k2], __ldg(P.tw_x + ((t * k2) % M)));
  }
  __syncthreads();
  // Step B: Z[k2 + R2 k1] to the split area.
  {
    double2 x[KQ][R1];
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) x[q][n1] = sb[X::sidx(n1, t + T * q)];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int k2 = t + T * q;
      dft<R1, -1>(x[q], cc);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) zb[k2 + R2 * k1] = x[q][k1];
    }
  }
  __syncthreads();
  // Split: X[k] = E - F, X[M-k] = conj(E + F), E = Z[k] + conj(Z[M-k]),
  // F = i W^k (Z[k] - conj(Z[M-k])), W = exp(-2 pi i / nx)   (all times 2).
  if (valid) {
    double2* out = spec + (long long)P.nxh * ((j - 1) + (long long)P.ny * (k - 1));
    for (int kk = t; kk <= M / 2; kk += T) {
      const double2 zk = zb[kk];
      const double2 zm = zb[(M - kk) % M];
      const double2 E = make_double2(fadd(cc, zk.x, zm.x), fsub(cc, zk.y, zm.y));
      const double2 O = make_double2(fsub(cc, zk.x, zm.x), fadd(cc, zk.y, zm.y));
      const double2 w = __ldg(P.tw_xr + kk);
      // F = i * W * O
      const double2 WO = cmul(cc, O, w);
      const double2 Fv = make_double2(-WO.y, WO.x);
      out[kk] = make_double2(fsub(cc, E.x, Fv.x), fsub(cc, E.y, Fv.y));
      if (kk == 0) out[M] = make_double2(fadd(cc, E.x, Fv.x), 0.0);
      else if (kk != M / 2) out[M - kk] = make_double2(fadd(cc, E.x, Fv.x), -fadd(cc, E.y, Fv.y));
    }
  }
}

template <int M, bool ALIGNED>
__global__ void __launch_bounds__(256) fft_x_inv_kernel(FftPlan P, const double2* __restrict__ spec, double* dp,
                                                        Layout L, FOne c, int line0, int line1) {
  using X = XP<M>;
  constexpr int R1 = X::R1, R2 = X::R2, T = X::T, KQ = X::KQ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = threadIdx.x, l = threadIdx.y;
  const int line = line0 + blockIdx.x * X::LINES + l;
  const int ny = L.ny;
  const bool valid = line < line1;
  const int j = valid ? 1 + line % ny : 1;
  const int k = valid ? 1 + line / ny : 1;
  double2* sb = reinterpret_cast<double2*>(smem_raw) + (long long)l * X::LS;
  double2* zb = sb;  // the unsplit area is reused by the transpose after a barrier
  const double2* in = spec + (long long)P.nxh * ((j - 1) + (long long)P.ny * (k - 1));
  // Unsplit: Z[k] = E + F, Z[M-k] = conj(E - F), E = X[k] + conj(X[M-k]),
  // F = i conj(W^k) (X[k] - conj(X[M-k]))   (all times 2).
  if (valid) {
    for (int kk = t; kk <= M / 2; kk += T) {
      double2 xk = in[kk];
      double2 xm = in[M - kk];
      if (kk == 0) { xk.y = 0.0; xm.y = 0.0; }
      const double2 E = make_double2(fadd(c, xk.x, xm.x), fsub(c, xk.y, xm.y));
      const double2 D = make_double2(fsub(c, xk.x, xm.x), fadd(c, xk.y, xm.y));
      const double2 w = __ldg(P.tw_xr + kk);
      const double2 WD = cmulc(c, D, w);
      const double2 Fv = make_double2(-WD.y, WD.x);
      zb[kk] = make_double2(fadd(c, E.x, Fv.x), fadd(c, E.y, Fv.y));
      if (kk != 0 && kk != M / 2) zb[M - kk] = make_double2(fsub(c, E.x, Fv.x), -fsub(c, E.y, Fv.y));
    }
  }
  __syncthreads();
  // Inverse step A: k2 = t + T q, R1-point inverse DFT over k1, twiddle.
  {
    double2 x[KQ][R1];
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) x[q][k1] = zb[t + T * q + R2 * k1];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int k2 = t + T * q;
      dft<R1, 1>(x[q], c);
      sb[X::sidx(0, k2)] = x[q][0];
#pragma unroll
      for (int a = 1; a < R1; ++a) sb[X::sidx(a, k2)] = cmulc(c, x[q][a], __ldg(P.tw_x + ((a * k2) % M)));
    }
  }
  __syncthreads();
  // Inverse step B: alpha = t, R2-point inverse DFT over k2, z[alpha + R1 beta].
  {
    double2 x[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) x[k2] = sb[X::sidx(t, k2)];
    dft<R2, 1>(x, c);
    if (valid) {
      double* o = dp + L.at(0, j, k);
#pragma unroll
      for (int b = 0; b < R2; ++b) {
        const int m = t + R1 * b;
        if (ALIGNED) {
          *reinterpret_cast<double2*>(o + 2 * m + 1) = x[b];
        } else {
          o[2 * m + 1] = x[b].x;
          o[2 * m + 2] = x[b].y;
        }
      }
    }
  }
}

template <int M>
size_t xp_smem() { return (size_t)XP<M>::LINES * XP<M>::LS * sizeof(double2); }
template <int N>
size_t yz_smem() { return (size_t)N * lpc<N>() * sizeof(double2); }

template <int N, bool FWD, int PB>
cudaError_t launch_dct_y_n(const FftPlan& P, double2* spec, cudaStream_t st) {
  const size_t sm = yz_smem<N>();
  auto kern = dct_y_kernel<N, FWD, PB>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  constexpr int LPC = lpc<N>();
  const int grid = (P.nxs * P.nz + LPC - 1) / LPC;
  kern<<<grid, dim3(LPC, Split<N>::R1), sm, st>>>(P, spec, FOne{1.0, -0.0});
  return cudaGetLastError();
}


template <int M>
cudaError_t launch_x_fwd(const FftPlan& P, const DivArgs& d, double2* spec, cudaStream_t st) {
  const size_t sm = xp_smem<M>();
  auto kern = d.rhs ? fft_x_fwd_kernel<M, true, false>
                    : (P.any_bc_term() ? fft_x_fwd_kernel<M, false, true> : fft_x_fwd_kernel<M, false, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int lines = d.L.ny * d.L.nz;
  dim3 block(XP<M>::T, XP<M>::LINES);
  kern<<<(lines + XP<M>::LINES - 1) / XP<M>::LINES, block, sm, st>>>(P, d, spec);
  return cudaGetLastError();
}
// x lines of the cell planes k in [k0, k1) (slots 1..nz).
template <int M>
cudaError_t launch_x_inv(const FftPlan& P, const double2* spec, double* dp, const Layout& L, FOne c, cudaStream_t st,
                         int k0, int k1) {
  const size_t sm = xp_smem<M>();
  auto kern = P.dp_unaligned ? fft_x_inv_kernel<M, false> : fft_x_inv_kernel<M, true>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int line0 = L.ny * (k0 - 1), line1 = L.ny * (k1 - 1);
  dim3 block(XP<M>::T, XP<M>::LINES);
  kern<<<(line1 - line0 + XP<M>::LINES - 1) / XP<M>::LINES, block, sm, st>>>(P, spec, dp, L, c, line0, line1);
  return cudaGetLastError();
}
// Lines of the outer indices [o0, o1) (o1 < 0: all of them).
template <int AXIS, int N, int DIR>
cudaError_t launch_yz(const FftPlan& P, double2* spec, FOne c, cudaStream_t st, int o0 = 0, int o1 = -1) {
  const size_t sm = yz_smem<N>();
  auto kern = fft_yz_kernel<AXIS, N, DIR>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  if (o1 < 0) o1 = AXIS == 1 ? P.nz : P.ny;
  constexpr int LPC = lpc<N>();
  dim3 grid(yz_nblk(P.nxh, LPC) + 1, o1 - o0);
  dim3 block(LPC, Split<N>::R1);
  kern<<<grid, block, sm, st>>>(P, spec, c, o0, o1);
  return cudaGetLastError();
}
template <int N>
cudaError_t launch_z(const FftPlan& P, double2* spec, FOne c, cudaStream_t st) {
  const size_t sm = yz_smem<N>();
  cudaError_t e = cudaFuncSetAttribute(fft_z_solve_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  constexpr int LPC = lpc<N>();
  dim3 grid(yz_nblk(P.nxh, LPC) + 1, P.ny);
  dim3 block(LPC, Split<N>::R1);
  fft_z_solve_kernel<N><<<grid, block, sm, st>>>(P, spec, c);
  return cudaGetLastError();
}

#define NS_SIZE_SWITCH(n, CALL) \
  switch (n) {                  \
    case 16: CALL(16); break;   \
    case 32: CALL(32); break;   \
    case 64: CALL(64); break;   \
    case 128: CALL(128); break; \
    case 256: CALL(256); break; \
    case 512: CALL(512); break; \
    default: return cudaErrorInvalidValue; \
  }

// The lengths of the FFT-based DCT passes: 24 and 48 (one 12-point stage)
// and the powers of two from 32 to 512.
#define NS_DCT_SIZE_SWITCH(n, CALL) \
  switch (n) {                      \
    case 24: CALL(24); break;       \
    case 32: CALL(32); break;       \
    case 48: CALL(48); break;       \
    case 64: CALL(64); break;       \
    case 128: CALL(128); break;     \
    case 256: CALL(256); break;     \
    case 512: CALL(512); break;     \
    default: return cudaErrorInvalidValue; \
  }

}  // namespace

cudaError_t launch_dct_y(bool fwd, const FftPlan& P, double2* spec, cudaStream_t st) {
  if (P.dct_y != 2 && P.dct_y != 3) return cudaErrorInvalidValue;
#define DCT_Y(n)                                                                                  \
  e = fwd ? (P.dct_y == 2 ? launch_dct_y_n<(n), true, 2>(P, spec, st) : launch_dct_y_n<(n), true, 3>(P, spec, st))  \
          : (P.dct_y == 2 ? launch_dct_y_n<(n), false, 2>(P, spec, st) : launch_dct_y_n<(n), false, 3>(P, spec, st));
  cudaError_t e = cudaSuccess;
  NS_DCT_SIZE_SWITCH(P.ny, DCT_Y)
#undef DCT_Y
  return e;
}

// The divergence (plus the pressure-BC terms) of the rows, or the given
// right-hand side d.rhs, one thread per point, into out[N row + i]: a
// streaming pass at full occupancy, so the transform reads whole rows
// instead of six shifted velocity loads.
template <int N>
__global__ void __launch_bounds__(256) dct_x_div_kernel(FftPlan P, DivArgs d, double* __restrict__ out, FOne c) {
  const long long idx = blockIdx.x * 256LL + threadIdx.x;
  if (idx >= (long long)N * P.ny * P.nz) return;
  const int i = (int)(idx % N), row = (int)(idx / N);
  const int j = 1 + row % P.ny, k = 1 + row / P.ny;
  const Layout& L = d.L;
  const long long g = L.at(i + 1, j, k);
  if (d.rhs) {  // a given right-hand side, already BC-modified
    out[idx] = d.rhs[g];
    return;
  }
  double v = fmul(c, fsub(c, d.us[g + 1], d.us[g]), d.cdx);
  v = fma(fsub(c, d.vs[g + L.sy], d.vs[g]), d.cdy, v);
  v = fma(fsub(c, d.ws[g + L.sz], d.ws[g]), d.cdz, v);
  out[idx] = v + 0.0;  // the boundary cells' terms follow in dct_x_bc_kernel
}

// The pressure-BC terms of the boundary cells (pr_bc_staggered_modify_rhs,
// NS_functions.f90:1345-1400) added to the divergence rows: a pass over the
// boundary cells only, so that the divergence kernel's warps do not branch
// at every row's ends.
__global__ void __launch_bounds__(256) dct_x_bc_kernel(FftPlan P, double* __restrict__ out) {
  const long long q = blockIdx.x * 256LL + threadIdx.x;
  if (q >= P.bc_cells()) return;
  int i, j, k;
  P.bc_cell(q, i, j, k);
  const long long e = (long long)P.nx * ((j - 1) + (long long)P.ny * (k - 1)) + (i - 1);
  out[e] = out[e] + P.bc_term_edge(i, j, k);
}

// The session's FFT-based x transforms (dct_x_fwd_body in place on the
// divergence rows, dct_x_inv_body).
template <int N, int PB>
__global__ void __launch_bounds__(lpc<N>() * Split<N>::R1) dct_x_fwd_kernel(FftPlan P, double2* spec, FOne c) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  dct_x_fwd_body<N, PB, false>(P, nullptr, spec, reinterpret_cast<double2*>(smem_raw), blockIdx.x, threadIdx.x,
                               threadIdx.y, c);
}

template <int N, int PB>
__global__ void __launch_bounds__(lpc<N>() * Split<N>::R1) dct_x_inv_kernel(FftPlan P, const double2* __restrict__ spec,
                                                                            double* dp, Layout L, FOne c) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  dct_x_inv_body<N, PB>(P, spec, dp, L, reinterpret_cast<double2*>(smem_raw), blockIdx.x, threadIdx.x, threadIdx.y, c);
}

template <int N, int PB>
cudaError_t launch_dct_x_n(bool fwd, const FftPlan& P, const DivArgs* d, double2* spec, const double2* cspec,
                           double* dp, const Layout& L, cudaStream_t st, const Marker* mk) {
  constexpr int LPC = lpc<N>();
  const size_t sm = yz_smem<N>() + (size_t)LPC * (N + 1) * sizeof(double2);
  const int grid = (P.ny * P.nz + 2 * LPC - 1) / (2 * LPC);
  const FOne c{1.0, -0.0};
  cudaError_t e;
  if (fwd) {
    const long long pts = (long long)N * P.ny * P.nz;
    dct_x_div_kernel<N><<<(unsigned)((pts + 255) / 256), 256, 0, st>>>(P, *d, reinterpret_cast<double*>(spec), c);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (!d->rhs && P.any_bc_term()) {
      dct_x_bc_kernel<<<(unsigned)((P.bc_cells() + 255) / 256), 256, 0, st>>>(P, reinterpret_cast<double*>(spec));
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (mk) (*mk)("dct_x_div");
    e = cudaFuncSetAttribute(dct_x_fwd_kernel<N, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dct_x_fwd_kernel<N, PB><<<grid, dim3(LPC, Split<N>::R1), sm, st>>>(P, spec, c);
  } else {
    e = cudaFuncSetAttribute(dct_x_inv_kernel<N, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dct_x_inv_kernel<N, PB><<<grid, dim3(LPC, Split<N>::R1), sm, st>>>(P, cspec, dp, L, c);
  }
  return cudaGetLastError();
}

cudaError_t launch_dct_x_fwd(const FftPlan& P, const DivArgs& d, double2* spec, cudaStream_t st, const Marker& mk) {
  if (P.dct_x != 2 && P.dct_x != 3) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
#define DCT_XF(n)                                                                                   \
  e = P.dct_x == 2 ? launch_dct_x_n<(n), 2>(true, P, &d, spec, nullptr, nullptr, d.L, st, &mk)      \
                   : launch_dct_x_n<(n), 3>(true, P, &d, spec, nullptr, nullptr, d.L, st, &mk);
  NS_DCT_SIZE_SWITCH(P.nx, DCT_XF)
#undef DCT_XF
  return e;
}

cudaError_t launch_dct_x_inv(const FftPlan& P, const double2* spec, double* dp, const Layout& L, cudaStream_t st) {
  if (P.dct_x != 2 && P.dct_x != 3) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
#define DCT_XI(n)                                                                                   \
  e = P.dct_x == 2 ? launch_dct_x_n<(n), 2>(false, P, nullptr, nullptr, spec, dp, L, st, nullptr)   \
                   : launch_dct_x_n<(n), 3>(false, P, nullptr, nullptr, spec, dp, L, st, nullptr);
  NS_DCT_SIZE_SWITCH(P.nx, DCT_XI)
#undef DCT_XI
  return e;
}

bool fft_size_supported(int nx, int ny, int nz) {
  auto ok = [](int n) { return n == 16 || n == 32 || n == 64 || n == 128 || n == 256 || n == 512; };
  return ok(nx) && ok(ny) && ok(nz);
}

// Forward 3D transform of a cell field (d.rhs, cell slots) of an all-periodic
// plan into spec: r2c along x (the split leaves every bin times 2), then
// complex FFTs along y and z.
cudaError_t launch_fft_forward3(const FftPlan& P, const DivArgs& d, double2* spec, cudaStream_t st,
                                const Marker& mk) {
  if (P.kind[0] != 0 || P.kind[1] != 0 || P.kind[2] != 0 || !d.rhs) return cudaErrorInvalidValue;
  const FOne c{d.one, d.mzero};
  cudaError_t e = cudaSuccess;
#define X_FWD(n) e = launch_x_fwd<(n) / 2>(P, d, spec, st)
  NS_SIZE_SWITCH(P.nx, X_FWD)
#undef X_FWD
  if (e != cudaSuccess) return e;
  mk("fft_x_fwd");
#define Y_FWD(n) e = launch_yz<1, (n), -1>(P, spec, c, st)
  NS_SIZE_SWITCH(P.ny, Y_FWD)
#undef Y_FWD
  if (e != cudaSuccess) return e;
  mk("fft_y_fwd");
#define Z_FWD(n) e = launch_yz<2, (n), -1>(P, spec, c, st)
  NS_SIZE_SWITCH(P.nz, Z_FWD)
#undef Z_FWD
  if (e != cudaSuccess) return e;
  mk("fft_z_fwd");
  return e;
}

// Divergence, forward transforms and the line solve: everything up to the
// inverse passes.
cudaError_t launch_poisson_fwd(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk) {
  const FOne c{d.one, d.mzero};
  cudaError_t e = cudaSuccess;
  // x forward: r2c FFT (periodic) or the dense transform with packed modes
  if (P.kind[0] == 0) {
#define X_FWD(n) e = launch_x_fwd<(n) / 2>(P, d, spec, st)
    NS_SIZE_SWITCH(P.nx, X_FWD)
#undef X_FWD
    if (e != cudaSuccess) return e;
    mk("fft_x_fwd");
  } else if (P.dct_x) {
    if ((e = launch_dct_x_fwd(P, d, spec, st, mk)) != cudaSuccess) return e;
    mk("dct_x_fwd");
  } else {
    if ((e = launch_dense_x(true, P, d, spec, dp, L, st)) != cudaSuccess) return e;
    mk("dense_x_fwd");
  }
  // The middle axis m is transformed, the solve axis s is solved per line:
  // (m, s) = (y, z) unless y is the wall axis of a z-periodic box.
  const int m = P.kind[1] == 2 ? 2 : 1;
  const int nm = m == 1 ? P.ny : P.nz;
  if (P.kind[m] == 0) {
    if (m == 1) {
#define Y_FWD(n) e = launch_yz<1, (n), -1>(P, spec, c, st)
      NS_SIZE_SWITCH(nm, Y_FWD)
#undef Y_FWD
    } else {
#define Z_FWD(n) e = launch_yz<2, (n), -1>(P, spec, c, st)
      NS_SIZE_SWITCH(nm, Z_FWD)
#undef Z_FWD
    }
    if (e != cudaSuccess) return e;
    mk(m == 1 ? "fft_y_fwd" : "fft_z_fwd");
  } else if (m == 1 && P.dct_y) {
    if ((e = launch_dct_y(true, P, spec, st)) != cudaSuccess) return e;
    mk("dct_y_fwd");
  } else {
    if ((e = launch_dense_yz(m, true, P, spec, st)) != cudaSuccess) return e;
    mk(m == 1 ? "dense_y_fwd" : "dense_z_fwd");
  }
  if (P.kind[2] == 0 && P.kind[1] != 2 && P.zcyc) {
    if ((e = launch_cyc_z_solve(P, spec, st)) != cudaSuccess) return e;
    mk("cyc_z_solve");
  } else if (P.kind[2] == 0 && P.kind[1] != 2) {
#define Z_SOL(n) e = launch_z<(n)>(P, spec, c, st)
    NS_SIZE_SWITCH(P.nz, Z_SOL)
#undef Z_SOL
    if (e != cudaSuccess) return e;
    mk("fft_z_solve");
  } else {
    if ((e = launch_tri_solve(3 - m, P, spec, st)) != cudaSuccess) return e;
    mk(m == 1 ? "tri_z_solve" : "tri_y_solve");
  }
  return e;
}

bool poisson_inv_by_planes(const FftPlan& P) { return P.kind[0] == 0 && P.kind[1] == 0; }
bool poisson_inv_x_by_planes(const FftPlan& P) { return P.kind[0] == 0; }

// The inverse pass of the middle axis (y, or z when y is the wall axis of a
// z-periodic box).  With poisson_inv_by_planes(P) it works plane by plane
// in z and [k0, k1) (cell slots 1..nz) selects planes; otherwise the range
// must be all of [1, nz + 1).
cudaError_t launch_poisson_inv_mid(const FftPlan& P, const DivArgs& d, double2* spec, const Layout& L,
                                   cudaStream_t st, const Marker& mk, int k0, int k1) {
  const FOne c{d.one, d.mzero};
  cudaError_t e = cudaSuccess;
  if (k0 < 1 || k1 > L.nz + 1 || k0 > k1) return cudaErrorInvalidValue;
  if (k0 == k1) return cudaSuccess;
  if ((k0 != 1 || k1 != L.nz + 1) && !poisson_inv_by_planes(P)) return cudaErrorInvalidValue;
  const int m = P.kind[1] == 2 ? 2 : 1;
  const int nm = m == 1 ? P.ny : P.nz;
  if (P.kind[m] == 0) {
    if (m == 1) {
#define Y_INV(n) e = launch_yz<1, (n), 1>(P, spec, c, st, k0 - 1, k1 - 1)
      NS_SIZE_SWITCH(nm, Y_INV)
#undef Y_INV
    } else {
#define Z_INV(n) e = launch_yz<2, (n), 1>(P, spec, c, st)
      NS_SIZE_SWITCH(nm, Z_INV)
#undef Z_INV
    }
    if (e != cudaSuccess) return e;
    mk(m == 1 ? "fft_y_inv" : "fft_z_inv");
  } else if (m == 1 && P.dct_y) {
    if ((e = launch_dct_y(false, P, spec, st)) != cudaSuccess) return e;
    mk("dct_y_inv");
  } else {
    if ((e = launch_dense_yz(m, false, P, spec, st)) != cudaSuccess) return e;
    mk(m == 1 ? "dense_y_inv" : "dense_z_inv");
  }
  return e;
}

// The x inverse pass into dp.  With poisson_inv_x_by_planes(P) (an x FFT)
// it works plane by plane in z; the dense x transform takes the whole box.
cudaError_t launch_poisson_inv_x(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                                 cudaStream_t st, const Marker& mk, int k0, int k1) {
  const FOne c{d.one, d.mzero};
  cudaError_t e = cudaSuccess;
  if (k0 < 1 || k1 > L.nz + 1 || k0 > k1) return cudaErrorInvalidValue;
  if (k0 == k1) return cudaSuccess;
  if ((k0 != 1 || k1 != L.nz + 1) && !poisson_inv_x_by_planes(P)) return cudaErrorInvalidValue;
  if (P.kind[0] == 0) {
#define X_INV(n) e = launch_x_inv<(n) / 2>(P, spec, dp, L, c, st, k0, k1)
    NS_SIZE_SWITCH(P.nx, X_INV)
#undef X_INV
    if (e != cudaSuccess) return e;
    mk("fft_x_inv");
  } else if (P.dct_x) {
    if ((e = launch_dct_x_inv(P, spec, dp, L, st)) != cudaSuccess) return e;
    mk("dct_x_inv");
  } else {
    if ((e = launch_dense_x(false, P, d, spec, dp, L, st)) != cudaSuccess) return e;
    mk("dense_x_inv");
  }
  return e;
}

// Both inverse passes into dp for the cell slots [k0, k1) (see the two
// functions above for which ranges each plan takes).
cudaError_t launch_poisson_inv(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk, int k0, int k1) {
  cudaError_t e = launch_poisson_inv_mid(P, d, spec, L, st, mk, k0, k1);
  if (e != cudaSuccess) return e;
  return launch_poisson_inv_x(P, d, spec, dp, L, st, mk, k0, k1);
}

cudaError_t launch_fft_poisson(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk) {
  cudaError_t e = launch_poisson_fwd(P, d, spec, dp, L, st, mk);
  if (e != cudaSuccess) return e;
  return launch_poisson_inv(P, d, spec, dp, L, st, mk, 1, L.nz + 1);
}

}  // namespace ns
