// Register DFTs, the four-step line engine and the FFT-based (Makhoul)
// DCT-II/III line bodies, shared by the session passes (ns_fft.cu) and the
// batched spectral passes (ns_dct.cu).  Everything here is a template or an
// inline device function with internal linkage in each translation unit.
#pragma once

#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {
namespace {

// ---------------------------------------------------------------------------
// Register DFTs
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }
__host__ __device__ constexpr int brevc(int i, int bits) {
  return bits == 0 ? 0 : (((i & 1) << (bits - 1)) | brevc(i >> 1, bits - 1));
}

// Linzer-Feig constants of W32^q = exp(-2 pi i q / 32), q in [0,16):
// mode 0: W = f (1 + i t);  mode 1: W = f (t + i).
__device__ __forceinline__ void lf32(int q, double& f, double& t, int& mode) {
  switch (q) {
    case 1: f = 0.9807852804032304; t = -0.19891236737965798; mode = 0; break;
    case 2: f = 0.9238795325112867; t = -0.4142135623730951; mode = 0; break;
    case 3: f = 0.8314696123025452; t = -0.6681786379192989; mode = 0; break;
    case 5: f = -0.8314696123025452; t = -0.668178637919299; mode = 1; break;
    case 6: f = -0.9238795325112867; t = -0.41421356237309515; mode = 1; break;
    case 7: f = -0.9807852804032304; t = -0.19891236737965806; mode = 1; break;
    case 9: f = -0.9807852804032304; t = 0.19891236737965792; mode = 1; break;
    case 10: f = -0.9238795325112867; t = 0.41421356237309503; mode = 1; break;
    case 11: f = -0.8314696123025455; t = 0.6681786379192984; mode = 1; break;
    case 13: f = -0.8314696123025453; t = 0.6681786379192988; mode = 0; break;
    case 14: f = -0.9238795325112867; t = 0.4142135623730952; mode = 0; break;
    case 15: f = -0.9807852804032304; t = 0.19891236737965837; mode = 0; break;
    default: f = 1.0; t = 0.0; mode = 0; break;
  }
}

constexpr double SQH = 0.70710678118654752440;  // sqrt(1/2)

// DIT butterfly a' = a + W b, b' = a - W b with W = W32^q (DIR = -1) or its
// conjugate (DIR = +1).
template <int DIR>
__device__ __forceinline__ void bfly(double2& a, double2& b, int q, const FOne& c) {
  double2 y;
  double f;
  if (q == 0) {
    const double2 a0 = a;
    a.x = fadd(c, a0.x, b.x); a.y = fadd(c, a0.y, b.y);
    b.x = fsub(c, a0.x, b.x); b.y = fsub(c, a0.y, b.y);
    return;
  }
  if (q == 8) {  // W = -i (forward) / +i (inverse)
    const double2 a0 = a, b0 = b;
    if (DIR < 0) {
      a.x = fadd(c, a0.x, b0.y); a.y = fsub(c, a0.y, b0.x);
      b.x = fsub(c, a0.x, b0.y); b.y = fadd(c, a0.y, b0.x);
    } else {
      a.x = fsub(c, a0.x, b0.y); a.y = fadd(c, a0.y, b0.x);
      b.x = fadd(c, a0.x, b0.y); b.y = fsub(c, a0.y, b0.x);
    }
    return;
  }
  if (q == 4) {  // W = sqrt(1/2)(1 -+ i)
    if (DIR < 0) { y.x = fadd(c, b.x, b.y); y.y = fsub(c, b.y, b.x); }
    else { y.x = fsub(c, b.x, b.y); y.y = fadd(c, b.y, b.x); }
    f = SQH;
  } else if (q == 12) {  // W = -sqrt(1/2)(1 +- i)
    if (DIR < 0) { y.x = fsub(c, b.x, b.y); y.y = fadd(c, b.y, b.x); }
    else { y.x = fadd(c, b.x, b.y); y.y = fsub(c, b.y, b.x); }
    f = -SQH;
  } else {
    double t;
    int mode;
    lf32(q, f, t, mode);
    if (DIR > 0) {  // conjugate root
      if (mode == 0) t = -t;
      else { f = -f; t = -t; }
    }
    if (mode == 0) { y.x = fma(-t, b.y, b.x); y.y = fma(t, b.x, b.y); }
    else { y.x = fma(t, b.x, -b.y); y.y = fma(t, b.y, b.x); }
  }
  const double2 a0 = a;
  a.x = fma(f, y.x, a0.x); a.y = fma(f, y.y, a0.y);
  b.x = fma(-f, y.x, a0.x); b.y = fma(-f, y.y, a0.y);
}

// Radix-2 in-place R-point DFT (R a power of two, R <= 32), natural order in and out.
// Every index is a template constant, so the array stays in registers.
template <int R, int I>
struct BitRev {
  static __device__ __forceinline__ void run(double2 (&x)[R]) {
    constexpr int J = brevc(I, ilog2c(R));
    if constexpr (J > I) {
      const double2 t = x[I];
      x[I] = x[J];
      x[J] = t;
    }
    BitRev<R, I + 1>::run(x);
  }
};
template <int R>
struct BitRev<R, R> {
  static __device__ __forceinline__ void run(double2 (&)[R]) {}
};
template <int R, int LEN, int S, int K, int DIR>
struct Bfly {  // butterfly K of group S of stage LEN, then the next one
  static __device__ __forceinline__ void run(double2 (&x)[R], const FOne& c) {
    bfly<DIR>(x[S + K], x[S + K + LEN / 2], K * (32 / LEN), c);
    if constexpr (K + 1 < LEN / 2) Bfly<R, LEN, S, K + 1, DIR>::run(x, c);
    else if constexpr (S + LEN < R) Bfly<R, LEN, S + LEN, 0, DIR>::run(x, c);
  }
};
template <int R, int LEN, int DIR>
struct Stage {
  static __device__ __forceinline__ void run(double2 (&x)[R], const FOne& c) {
    Bfly<R, LEN, 0, 0, DIR>::run(x, c);
    if constexpr (LEN < R) Stage<R, 2 * LEN, DIR>::run(x, c);
  }
};
template <int R, int DIR>
__device__ __forceinline__ void dft_pow2(double2 (&x)[R], const FOne& c) {
  BitRev<R, 0>::run(x);
  Stage<R, 2, DIR>::run(x, c);
}

// 3-point DFT in FMA form: with s = a1 + a2, d = a1 - a2 and t = a0 - s/2,
// X0 = a0 + s, X1 = t - i (sqrt(3)/2) d, X2 = t + i (sqrt(3)/2) d (forward;
// the inverse takes the conjugate roots).
template <int DIR>
__device__ __forceinline__ void dft3(double2& a0, double2& a1, double2& a2, const FOne& c) {
  constexpr double H3 = 0.86602540378443864676;  // sqrt(3)/2
  const double2 s = make_double2(fadd(c, a1.x, a2.x), fadd(c, a1.y, a2.y));
  const double2 d = make_double2(fsub(c, a1.x, a2.x), fsub(c, a1.y, a2.y));
  const double2 t = make_double2(fma(s.x, -0.5, a0.x), fma(s.y, -0.5, a0.y));
  a0 = make_double2(fadd(c, a0.x, s.x), fadd(c, a0.y, s.y));
  const double g = DIR < 0 ? H3 : -H3;
  a1 = make_double2(fma(g, d.y, t.x), fma(-g, d.x, t.y));
  a2 = make_double2(fma(-g, d.y, t.x), fma(g, d.x, t.y));
}

// 12-point DFT by the prime-factor (Good-Thomas) split 12 = 3 x 4, which
// needs no twiddles: 3-point DFTs over n1 of x[(4 n1 + 3 n2) mod 12] for each
// n2, then 4-point DFTs over n2, whose output k2 of row k1 is
// X[(4 k1 + 9 k2) mod 12] (9 = 3 x (3^-1 mod 4), 4 = 4 x (4^-1 mod 3)).
template <int DIR>
__device__ __forceinline__ void dft12(double2 (&x)[12], const FOne& c) {
  double2 y[4][3];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    double2 a0 = x[(3 * n2) % 12], a1 = x[(4 + 3 * n2) % 12], a2 = x[(8 + 3 * n2) % 12];
    dft3<DIR>(a0, a1, a2, c);
    y[n2][0] = a0;
    y[n2][1] = a1;
    y[n2][2] = a2;
  }
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    double2 z[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft_pow2<4, DIR>(z, c);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[(4 * k1 + 9 * k2) % 12] = z[k2];
  }
}

// In-place R-point DFT, natural order in and out: R a power of two up to 32,
// or 12.
template <int R, int DIR>
__device__ __forceinline__ void dft(double2 (&x)[R], const FOne& c) {
  if constexpr (R == 12) dft12<DIR>(x, c);
  else dft_pow2<R, DIR>(x, c);
}

__device__ __forceinline__ double2 cmul(const FOne& c, double2 a, double2 w) {
  double2 r;
  r.x = fma(a.x, w.x, -fmul(c, a.y, w.y));
  r.y = fma(a.x, w.y, fmul(c, a.y, w.x));
  return r;
}
__device__ __forceinline__ double2 cmulc(const FOne& c, double2 a, double2 w) {  // a * conj(w)
  double2 r;
  r.x = fma(a.x, w.x, fmul(c, a.y, w.y));
  r.y = fma(a.y, w.x, -fmul(c, a.x, w.y));
  return r;
}

// Four-step split N = R1 * R2 (R1 <= R2), T = R1 threads per line.
template <int N> struct Split;
template <> struct Split<8> { static constexpr int R1 = 2, R2 = 4; };
template <> struct Split<24> { static constexpr int R1 = 2, R2 = 12; };
template <> struct Split<48> { static constexpr int R1 = 4, R2 = 12; };
template <> struct Split<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Split<32> { static constexpr int R1 = 4, R2 = 8; };
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 8, R2 = 16; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };
template <> struct Split<512> { static constexpr int R1 = 16, R2 = 32; };

// ---------------------------------------------------------------------------
// Line engine: LPC lines per CTA (lanes over lines, coalesced when the lines
// are neighbouring columns), T = R1 threads per line.
// Shared buffer index for line l: (r * R2 + q) * LPC + l.
// ---------------------------------------------------------------------------
// Lines per CTA of the session kernels: 8 for the long lines (register-heavy
// 16-point DFTs), else 16.
template <int N>
constexpr int lpc() { return N >= 256 ? 8 : 16; }

template <int N, int LPC_ = lpc<N>()>
struct YZ {
  static constexpr int R1 = Split<N>::R1, R2 = Split<N>::R2, T = R1, KQ = R2 / T;
  static constexpr int LPC = LPC_;
  __device__ static __forceinline__ int sidx(int r, int q, int l) { return (r * R2 + q) * LPC + l; }

  // Forward step A: thread n1 = t loads x[n1 + R1 n2], R2-point DFT, twiddle, to smem (n1, k2).
  __device__ static __forceinline__ void fwdA(const double2* __restrict__ g, long long st, double2* sb,
                                              const double2* __restrict__ tw, int l, int t, const FOne& c) {
    double2 x[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) x[n2] = g[(long long)(t + R1 * n2) * st];
    dft<R2, -1>(x, c);
    sb[sidx(t, 0, l)] = x[0];
#pragma unroll
    for (int k2 = 1; k2 < R2; ++k2) sb[sidx(t, k2, l)] = cmul(c, x[k2], __ldg(tw + ((t * k2) % N)));
  }
  // Forward step B: for k2 = t + T*q: R1-point DFT over n1 -> X[k2 + R2 k1] in xk[q][k1].
  __device__ static __forceinline__ void fwdB(double2 (&xk)[KQ][R1], const double2* sb, int l, int t,
                                              const FOne& c) {
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int k2 = t + T * q;
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) xk[q][n1] = sb[sidx(n1, k2, l)];
      dft<R1, -1>(xk[q], c);
    }
  }
  // Inverse step A: from X[k2 + R2 k1] held in xk, R1-point inverse DFT, twiddle, to smem (k2, alpha).
  __device__ static __forceinline__ void invA(double2 (&xk)[KQ][R1], double2* sb, const double2* __restrict__ tw,
                                              int l, int t, const FOne& c) {
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int k2 = t + T * q;
      dft<R1, 1>(xk[q], c);
      sb[sidx(0, k2, l)] = xk[q][0];
#pragma unroll
      for (int a = 1; a < R1; ++a) sb[sidx(a, k2, l)] = cmulc(c, xk[q][a], __ldg(tw + ((a * k2) % N)));
    }
  }
  // Inverse step B: thread alpha = t, R2-point inverse DFT over k2, x[alpha + R1 beta] to global.
  __device__ static __forceinline__ void invB(double2* __restrict__ g, long long st, const double2* sb, int l, int t,
                                              const FOne& c) {
    double2 x[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) x[k2] = sb[sidx(t, k2, l)];
    dft<R2, 1>(x, c);
#pragma unroll
    for (int b = 0; b < R2; ++b) g[(long long)(t + R1 * b) * st] = x[b];
  }
};

// The y transform of a packed-x box (two real lines, .x and .y, per complex
// slot) through an FFT (Makhoul).  DCT-II of a real line x of N points
// (dense_pair's pbc-3 matrix F[k][s] = cos(pi k (2s+1) / (2N))) is
//   X_k = Re(exp(-i pi k / (2N)) V_k),  V = DFT_N(v),  v_m = x_{2m}, v_{N-1-m} = x_{2m+1}.
// The two real lines of a slot share one complex FFT and are separated in the
// post-twiddle: with U_k = exp(-i pi k / (2N)) V_k / 2 (and V_N = V_0),
//   X_k = (Re U_k - Im U_{N-k}) + i (Im U_k + Re U_{N-k}).
// pbc 2's matrix is the same transform of the line with its even (0-based)
// samples negated, modes reversed (k -> N-1-k).  The inverse is the exact
// inverse (DCT-III with its 1/N): V_k = exp(i pi k / (2N)) (X_k - i X_{N-k}) / N
// (X_N = 0), v = the unnormalised inverse DFT of V, x_{2m} = v_m,
// x_{2m+1} = v_{N-1-m}.  About 2.8 log2(N) / 2 + 3 FP64 instructions per real
// value against 3N/8 + 1.5 for the folded dense products.  Lines are numbered
// tl = col + nxs kz; block blk of a pass takes lines blk LPC .. blk LPC + LPC-1.
template <int N, bool FWD, int PB, int LPC_ = lpc<N>()>
__device__ __forceinline__ void dct_y_body(const FftPlan& P, double2* __restrict__ spec, double2* sb, int blk, int l,
                                           int t, const FOne& c) {
  using F = YZ<N, LPC_>;
  constexpr int LPC = F::LPC, R1 = F::R1, R2 = F::R2, T = F::T, KQ = F::KQ;
  const int tl = blk * LPC + l;
  const bool valid = tl < P.nxs * P.nz;
  const int col = valid ? tl % P.nxs : 0, o = valid ? tl / P.nxs : 0;
  const long long st = P.nxs;
  double2* g = spec + col + (long long)P.nxs * P.ny * o;
  const double2* tw = P.dct_tw;
  auto src_of = [](int n) { return n < N / 2 ? 2 * n : 2 * (N - 1 - n) + 1; };  // the sample v_n holds
  auto mode_of = [](int k) { return PB == 2 ? N - 1 - k : k; };
  auto neg = [](double2 v) { return make_double2(-v.x, -v.y); };
  if (FWD) {
    double2 x[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      const int s = src_of(t + R1 * n2);
      double2 v = valid ? g[(long long)s * st] : make_double2(0.0, 0.0);
      if (PB == 2 && (s & 1) == 0) v = neg(v);
      x[n2] = v;
    }
    dft<R2, -1>(x, c);
    sb[F::sidx(t, 0, l)] = x[0];
#pragma unroll
    for (int k2 = 1; k2 < R2; ++k2) sb[F::sidx(t, k2, l)] = cmul(c, x[k2], __ldg(tw + ((t * k2) % N)));
    __syncthreads();
    double2 xk[KQ][R1];
    F::fwdB(xk, sb, l, t, c);  // xk[q][k1] = V[k2 + R2 k1], k2 = t + T q
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) sb[(t + T * q + R2 * k1) * LPC + l] = xk[q][k1];
    __syncthreads();
    if (valid)
      for (int k = t; k <= N / 2; k += R1) {
        const double2 Uk = cmul(c, sb[k * LPC + l], __ldg(P.dct_wf + k));
        const double2 Um = cmul(c, sb[((N - k) % N) * LPC + l], __ldg(P.dct_wf + (N - k)));
        g[(long long)mode_of(k) * st] = make_double2(fsub(c, Uk.x, Um.y), fadd(c, Uk.y, Um.x));
        if (k != 0 && k != N / 2)
          g[(long long)mode_of(N - k) * st] = make_double2(fsub(c, Um.x, Uk.y), fadd(c, Um.y, Uk.x));
      }
  } else {
    double2 xk[KQ][R1];
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        const int k = t + T * q + R2 * k1;
        const double2 X = valid ? g[(long long)mode_of(k) * st] : make_double2(0.0, 0.0);
        const double2 Xm = (valid && k != 0) ? g[(long long)mode_of(N - k) * st] : make_double2(0.0, 0.0);
        const double2 d = make_double2(fadd(c, X.x, Xm.y), fsub(c, X.y, Xm.x));  // X_k - i X_{N-k}
        xk[q][k1] = cmul(c, d, __ldg(P.dct_wi + k));
      }
    F::invA(xk, sb, tw, l, t, c);
    __syncthreads();
    double2 x[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) x[k2] = sb[F::sidx(t, k2, l)];
    dft<R2, 1>(x, c);
#pragma unroll
    for (int b = 0; b < R2; ++b) {
      const int s = src_of(t + R1 * b);
      double2 v = x[b];
      if (PB == 2 && (s & 1) == 0) v = neg(v);
      if (valid) g[(long long)s * st] = v;
    }
  }
}

// The x transform of a wall x axis through the same FFT-based DCT: two real
// x lines (rows 2l and 2l+1 of a CTA's 2 LPC rows, row = (j-1) + ny (k-1))
// are the real and imaginary parts of one complex line.  Both passes stage
// the rows in shared memory as pairs, pr[l (N+1) + n] = (row 2l, row 2l+1) at
// sample or mode n (stride N+1 keeps the per-pair reads conflict-free), so
// the global side moves whole rows with coalesced accesses.  A packed
// spectrum row read as doubles is the modes in order.
// Forward: the real rows (row = (j-1) + ny (k-1), block blk takes rows
// 2 LPC blk ..) become their packed modes in spec.  DIV: the rows are the
// divergence of d (plus the pressure-BC terms, or d->rhs as it is), computed
// here with the two rows of a pair interleaved (element e: row 2 (e / 2N) +
// e % 2, point (e / 2) % N); else the rows are read from spec, in place.
template <int N, int PB, bool DIV, int LPC_ = lpc<N>()>
__device__ __forceinline__ void dct_x_fwd_body(const FftPlan& P, const DivArgs* d, double2* spec, double2* sb, int blk,
                                               int l, int t, const FOne& c) {
  using F = YZ<N, LPC_>;
  constexpr int LPC = F::LPC, R1 = F::R1, R2 = F::R2, T = F::T, KQ = F::KQ, PS = N + 1;
  double2* pr = sb + N * LPC;
  double* prd = reinterpret_cast<double*>(pr);
  const int nrows = P.ny * P.nz;
  const int row0 = blk * 2 * LPC;
  const int tid = t * LPC + l, nth = LPC * R1;
  double* out = reinterpret_cast<double*>(spec);
  if (DIV) {
    const Layout L = d->L;
    for (int e = tid; e < 2 * LPC * N; e += nth) {
      const int pair = e / (2 * N), i = (e >> 1) % N, row = row0 + 2 * pair + (e & 1);
      double v = 0.0;
      if (row < nrows) {
        const int j = 1 + row % P.ny, k = 1 + row / P.ny;
        const long long g = L.at(i + 1, j, k);
        if (d->rhs) {
          v = d->rhs[g];
        } else {
          v = fmul(c, fsub(c, d->us[g + 1], d->us[g]), d->cdx);
          v = fma(fsub(c, d->vs[g + L.sy], d->vs[g]), d->cdy, v);
          v = fma(fsub(c, d->ws[g + L.sz], d->ws[g]), d->cdz, v);
          v = v + P.bc_term(i + 1, j, k);
        }
      }
      prd[2 * PS * pair + 2 * i + (e & 1)] = v;
    }
  } else {
    for (int e = tid; e < 2 * LPC * N; e += nth) {
      const int rr = e / N, i = e % N, row = row0 + rr;
      prd[2 * PS * (rr >> 1) + 2 * i + (rr & 1)] = row < nrows ? out[(long long)N * row + i] : 0.0;
    }
  }
  __syncthreads();
  auto src_of = [](int n) { return n < N / 2 ? 2 * n : 2 * (N - 1 - n) + 1; };
  auto mode_of = [](int k) { return PB == 2 ? N - 1 - k : k; };
  const double2* tw = P.dctx_tw;
  {
    double2 x[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      const int s = src_of(t + R1 * n2);
      double2 v = pr[l * PS + s];
      if (PB == 2 && (s & 1) == 0) v = make_double2(-v.x, -v.y);
      x[n2] = v;
    }
    dft<R2, -1>(x, c);
    sb[F::sidx(t, 0, l)] = x[0];
#pragma unroll
    for (int k2 = 1; k2 < R2; ++k2) sb[F::sidx(t, k2, l)] = cmul(c, x[k2], __ldg(tw + ((t * k2) % N)));
  }
  __syncthreads();
  double2 xk[KQ][R1];
  F::fwdB(xk, sb, l, t, c);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) sb[(t + T * q + R2 * k1) * LPC + l] = xk[q][k1];
  __syncthreads();
  for (int k = t; k <= N / 2; k += R1) {
    const double2 Uk = cmul(c, sb[k * LPC + l], __ldg(P.dctx_wf + k));
    const double2 Um = cmul(c, sb[((N - k) % N) * LPC + l], __ldg(P.dctx_wf + (N - k)));
    pr[l * PS + mode_of(k)] = make_double2(fsub(c, Uk.x, Um.y), fadd(c, Uk.y, Um.x));
    if (k != 0 && k != N / 2) pr[l * PS + mode_of(N - k)] = make_double2(fsub(c, Um.x, Uk.y), fadd(c, Um.y, Uk.x));
  }
  __syncthreads();
  for (int e = tid; e < 2 * LPC * N; e += nth) {
    const int rr = e / N, i = e % N, row = row0 + rr;
    if (row < nrows) out[(long long)N * row + i] = prd[2 * PS * (rr >> 1) + 2 * i + (rr & 1)];
  }
}

// Inverse: packed modes of the rows of block blk -> dp slots 1..nx.
template <int N, int PB, int LPC_ = lpc<N>()>
__device__ __forceinline__ void dct_x_inv_body(const FftPlan& P, const double2* __restrict__ spec, double* dp,
                                               const Layout& L, double2* sb, int blk, int l, int t, const FOne& c) {
  using F = YZ<N, LPC_>;
  constexpr int LPC = F::LPC, R1 = F::R1, R2 = F::R2, T = F::T, KQ = F::KQ, PS = N + 1;
  double2* pr = sb + N * LPC;
  double* prd = reinterpret_cast<double*>(pr);
  const int nrows = P.ny * P.nz;
  const int row0 = blk * 2 * LPC;
  const int tid = t * LPC + l, nth = LPC * R1;
  const double* in = reinterpret_cast<const double*>(spec);
  for (int e = tid; e < 2 * LPC * N; e += nth) {
    const int rr = e / N, i = e % N, row = row0 + rr;
    prd[2 * PS * (rr >> 1) + 2 * i + (rr & 1)] = row < nrows ? in[(long long)N * row + i] : 0.0;
  }
  __syncthreads();
  auto src_of = [](int n) { return n < N / 2 ? 2 * n : 2 * (N - 1 - n) + 1; };
  auto mode_of = [](int k) { return PB == 2 ? N - 1 - k : k; };
  double2 xk[KQ][R1];
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      const int k = t + T * q + R2 * k1;
      const double2 X = pr[l * PS + mode_of(k)];
      const double2 Xm = k ? pr[l * PS + mode_of(N - k)] : make_double2(0.0, 0.0);
      const double2 dd = make_double2(fadd(c, X.x, Xm.y), fsub(c, X.y, Xm.x));  // X_k - i X_{N-k}
      xk[q][k1] = cmul(c, dd, __ldg(P.dctx_wi + k));
    }
  F::invA(xk, sb, P.dctx_tw, l, t, c);
  __syncthreads();
  {
    double2 x[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) x[k2] = sb[F::sidx(t, k2, l)];
    dft<R2, 1>(x, c);
#pragma unroll
    for (int b = 0; b < R2; ++b) {
      const int s = src_of(t + R1 * b);
      double2 v = x[b];
      if (PB == 2 && (s & 1) == 0) v = make_double2(-v.x, -v.y);
      pr[l * PS + s] = v;
    }
  }
  __syncthreads();
  for (int e = tid; e < 2 * LPC * N; e += nth) {
    const int rr = e / N, i = e % N, row = row0 + rr;
    if (row < nrows) dp[L.at(i + 1, 1 + row % P.ny, 1 + row / P.ny)] = prd[2 * PS * (rr >> 1) + 2 * i + (rr & 1)];
  }
}

}  // namespace
}  // namespace ns
