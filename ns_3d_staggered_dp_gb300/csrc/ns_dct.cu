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
// so the y/z passes again act on complex lines.  The wall axis that is
// transformed last is not transformed at all: its lines are solved as
// tridiagonal systems (tri_solve_kernel), which gives the same solution as
// transform, eigenvalue divide and inverse transform along that axis; with
// packed x modes the real and imaginary parts are two systems.
// The divergence kernels add the pressure-BC terms of
// pr_bc_staggered_modify_rhs (NS_functions.f90:1345-1400) on the first and
// last cells of every non-periodic axis.
#include <cmath>
#include <vector>

#include "ns_fft_core.cuh"
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
__device__ __forceinline__ void dense_x_fwd_body(const SpecPlan& S, const DivArgs& d, double2* __restrict__ spec,
                                                 double* xs, int bx) {
  // a group of G lanes per line, 128/G lines per CTA (several short lines share a warp)
  const int G = dense_x_group(S.nx);
  const int grp = threadIdx.x / G, gl = threadIdx.x % G;
  const int line = bx * (128 / G) + grp;
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const bool valid = line < ny * nz;
  const int j = valid ? 1 + line % ny : 1, k = valid ? 1 + line / ny : 1;
  double* r = xs + grp * nx;
  const FOne c{d.one, d.mzero};
  if (valid)
    for (int i = gl; i < nx; i += G) r[i] = rhs_cell(d, S, c, i + 1, j, k);
  __syncwarp();
  const double* __restrict__ FT = S.fwd[0];  // F^T: FT[n * N + kk] = F[kk][n]
  double2* out = spec + (long long)S.nxs * ((j - 1) + (long long)ny * (k - 1));
  if (S.sym[0] & 1) {
    // F[k][N-1-n] = (-1)^k F[k][n]: fold the line (s[n] = r[n] + r[N-1-n] at n,
    // d[n] = r[n] - r[N-1-n] at N-1-n); mode 2q sums F s, mode 2q+1 sums F d
    const int H = nx / 2;
    if (valid)
      for (int n = gl; n < H; n += G) {
        const double a0 = r[n], b0 = r[nx - 1 - n];
        r[n] = a0 + b0;
        r[nx - 1 - n] = a0 - b0;
      }
    __syncwarp();
    const int lv1 = (S.sym[0] >> 2) & 3;  // bit p: the modes of parity p fold once more
    if (lv1 == 1 || lv1 == 2) {
      // Second fold of one branch over its H points (sign (-1)^((k >> 1) & 1)):
      // the even branch s (at 0..H-1) into s2 at n and d2 at H-1-n, the odd
      // branch d (d[n] at N-1-n) into s2 at N-1-n and d2 at H+n, n < H/2.
      // The folded mode of a pair then sums H/2 terms, the other one sums
      // the mirrored terms n and H-1-n together.
      const int Q = H / 2;
      if (valid)
        for (int n = gl; n < Q; n += G) {
          const int ia = lv1 == 1 ? n : nx - 1 - n, ib = lv1 == 1 ? H - 1 - n : H + n;
          const double a0 = r[ia], b0 = r[ib];
          r[ia] = a0 + b0;
          r[ib] = a0 - b0;
        }
      __syncwarp();
      if (!valid) return;
      for (int q = gl; q < H; q += G) {
        const int b1 = q & 1;  // ((2q or 2q+1) >> 1) & 1
        double a = 0.0, b = 0.0;
        if (lv1 == 1) {  // mode 2q folded, mode 2q+1 on d
          for (int n = 0; n < Q; ++n) {
            const double2 f = *reinterpret_cast<const double2*>(FT + (long long)n * nx + 2 * q);
            const double fm = FT[(long long)(H - 1 - n) * nx + 2 * q + 1];
            a = fma(f.x, b1 ? r[H - 1 - n] : r[n], a);
            b = fma(f.y, r[nx - 1 - n], b);
            b = fma(fm, r[H + n], b);
          }
        } else {  // mode 2q on s, mode 2q+1 folded
          for (int n = 0; n < Q; ++n) {
            const double2 f = *reinterpret_cast<const double2*>(FT + (long long)n * nx + 2 * q);
            const double fm = FT[(long long)(H - 1 - n) * nx + 2 * q];
            a = fma(f.x, r[n], a);
            a = fma(fm, r[H - 1 - n], a);
            b = fma(f.y, b1 ? r[H + n] : r[nx - 1 - n], b);
          }
        }
        out[q] = make_double2(a, b);
      }
      return;
    }
    if (!valid) return;
    for (int q = gl; q < H; q += G) {
      double a = 0.0, b = 0.0;
      for (int n = 0; n < H; ++n) {
        const double2 f = *reinterpret_cast<const double2*>(FT + (long long)n * nx + 2 * q);
        a = fma(f.x, r[n], a);
        b = fma(f.y, r[nx - 1 - n], b);
      }
      out[q] = make_double2(a, b);
    }
    return;
  }
  if (!valid) return;
  for (int q = gl; q < nx / 2; q += G) {
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
__device__ __forceinline__ void dense_x_inv_body(const SpecPlan& S, const double2* __restrict__ spec, double* dp,
                                                 const Layout& L, double* xs, int bx) {
  const int G = dense_x_inv_group(S.sym[0], S.nx);
  const int grp = threadIdx.x / G, gl = threadIdx.x % G;
  const int line = bx * (128 / G) + grp;
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const bool valid = line < ny * nz;
  const int j = valid ? 1 + line % ny : 1, k = valid ? 1 + line / ny : 1;
  double* X = xs + grp * nx;
  const double2* in = spec + (long long)S.nxs * ((j - 1) + (long long)ny * (k - 1));
  if (valid)
    for (int q = gl; q < nx / 2; q += G) {
      const double2 v = in[q];
      X[2 * q] = v.x;
      X[2 * q + 1] = v.y;
    }
  __syncwarp();
  if (!valid) return;
  const double* __restrict__ GT = S.inv[0];  // G^T: GT[kk * N + n] = G[n][kk] (x = G X)
  double* o = dp + L.at(1, j, k);
  const int lvi = (S.sym[0] >> 4) & 3;  // bit p: the columns of parity p fold once more
  if ((S.sym[0] & 2) && (lvi == 1 || lvi == 2)) {
    // Row pairs (n, H-1-n), n < H/2: G[H-1-n][k] = (-1)^((k >> 1) & 1) G[n][k]
    // on the columns of parity pf, so their partial sums F0 (k = pf mod 4)
    // and F1 (k = pf + 2 mod 4) give both rows as F0 + F1 and F0 - F1; the
    // other parity is summed for both rows.  Then out[r] = E_r + O_r and
    // out[N-1-r] = E_r - O_r for r = n and H-1-n.
    const int H = nx / 2, Q = H / 2, pf = lvi == 1 ? 0 : 1, pu = 1 - pf;
    for (int n = gl; n < Q; n += G) {
      const int m = H - 1 - n;
      double f0 = 0.0, f1 = 0.0, un = 0.0, um = 0.0;
      for (int c = 0; c < nx; c += 4) {
        const double x0 = X[c + pf], x1 = X[c + pf + 2], y0 = X[c + pu], y1 = X[c + pu + 2];
        f0 = fma(__ldg(GT + (long long)(c + pf) * nx + n), x0, f0);
        f1 = fma(__ldg(GT + (long long)(c + pf + 2) * nx + n), x1, f1);
        un = fma(__ldg(GT + (long long)(c + pu) * nx + n), y0, un);
        un = fma(__ldg(GT + (long long)(c + pu + 2) * nx + n), y1, un);
        um = fma(__ldg(GT + (long long)(c + pu) * nx + m), y0, um);
        um = fma(__ldg(GT + (long long)(c + pu + 2) * nx + m), y1, um);
      }
      const double fn = f0 + f1, fm = f0 - f1;
      const double en = pf ? un : fn, on = pf ? fn : un;  // even and odd sums of row n
      const double em = pf ? um : fm, om = pf ? fm : um;  // and of row m
      o[n] = en + on;
      o[nx - 1 - n] = en - on;
      o[m] = em + om;
      o[nx - 1 - m] = em - om;
    }
    return;
  }
  if (S.sym[0] & 2) {
    // G[N-1-n][k] = (-1)^k G[n][k]: out[n] = E + O, out[N-1-n] = E - O
    for (int n = gl; n < nx / 2; n += G) {
      double e = 0.0, od = 0.0;
      for (int kk = 0; kk + 1 < nx; kk += 2) {
        e = fma(__ldg(GT + (long long)kk * nx + n), X[kk], e);
        od = fma(__ldg(GT + (long long)(kk + 1) * nx + n), X[kk + 1], od);
      }
      o[n] = e + od;
      o[nx - 1 - n] = e - od;
    }
    return;
  }
  for (int n = gl; n < nx; n += G) {
    double a = 0.0;
    for (int kk = 0; kk < nx; ++kk) a = fma(__ldg(GT + (long long)kk * nx + n), X[kk], a);
    o[n] = a;
  }
}

// Dense transform of complex lines along y (AXIS 1) or z (AXIS 2).  Lines are
// numbered t = col + nxs * o (o: z for y-lines, y for z-lines) and a CTA takes
// 16 consecutive ones, so narrow spectra fill it too; neighbouring lanes read
// neighbouring columns (coalesced).
template <int AXIS, bool FWD>
__device__ __forceinline__ void dense_yz_body(const SpecPlan& S, double2* __restrict__ spec, double2* ls, int bx) {
  constexpr int LPC = 16, T = 8;  // 16 lines x 8 threads per line
  const int l = threadIdx.x % LPC, t = threadIdx.x / LPC;
  const int N = (AXIS == 1) ? S.ny : S.nz;
  const int n_other = (AXIS == 1) ? S.nz : S.ny;
  const int tl = bx * LPC + l;
  const bool valid = tl < S.nxs * n_other;
  const int col = valid ? tl % S.nxs : 0;
  const int o = valid ? tl / S.nxs : 0;
  const long long st = (AXIS == 1) ? (long long)S.nxs : (long long)S.nxs * S.ny;
  const long long base = (AXIS == 1) ? col + (long long)S.nxs * S.ny * o : col + (long long)S.nxs * o;
  double2* line = ls + l;  // element n at line[n * LPC]
  double2* g = spec + base;
  if (valid)
    for (int n = t; n < N; n += T) line[n * LPC] = g[(long long)n * st];
  __syncthreads();
  const double* __restrict__ M = FWD ? S.fwd[AXIS] : S.inv[AXIS];  // row = output index
  const bool sym = (S.sym[AXIS] >> (FWD ? 0 : 1)) & 1;
  if (sym && FWD) {
    // F[k][N-1-n] = (-1)^k F[k][n]: fold the line into s[n] = x[n] + x[N-1-n]
    // (kept at n) and d[n] = x[n] - x[N-1-n] (kept at N-1-n); an even mode
    // then sums F[k][n] s[n], an odd one F[k][n] d[n], over n < N/2.
    const int H = N / 2;
    if (valid)
      for (int n = t; n < H; n += T) {
        const double2 a = line[n * LPC], b = line[(N - 1 - n) * LPC];
        line[n * LPC] = make_double2(a.x + b.x, a.y + b.y);
        line[(N - 1 - n) * LPC] = make_double2(a.x - b.x, a.y - b.y);
      }
    __syncthreads();
    const int lv1 = (S.sym[AXIS] >> 2) & 3;  // bit p: the modes of parity p fold once more
    if (lv1 == 1 || lv1 == 2) {
      // Second fold of branch p over its H points (sign (-1)^((k >> 1) & 1)):
      // the even branch s (at 0..H-1) into s2 at q and d2 at H-1-q, the odd
      // branch d (d[q] at N-1-q) into s2 at N-1-q and d2 at H+q, q < H/2.
      const int Q = H / 2, pf = lv1 == 1 ? 0 : 1;
      if (valid)
        for (int q = t; q < Q; q += T) {
          const int ia = pf ? N - 1 - q : q, ib = pf ? H + q : H - 1 - q;
          const double2 a = line[ia * LPC], b = line[ib * LPC];
          line[ia * LPC] = make_double2(a.x + b.x, a.y + b.y);
          line[ib * LPC] = make_double2(a.x - b.x, a.y - b.y);
        }
      __syncthreads();
      if (!valid) return;
      // each thread takes modes 2m + pu (H terms) and 2m + pf (H/2 terms) for
      // m = t, t + T, ..., so every thread has the same loop lengths
      const int pu = 1 - pf;
      for (int m = t; m < H; m += T) {
        {
          const int kk = 2 * m + pu;
          const double2* src = pu ? line + (long long)(N - 1) * LPC : line;
          const int step = pu ? -LPC : LPC;
          const double* __restrict__ row = M + (long long)kk * N;
          double2 acc = make_double2(0.0, 0.0);
          for (int n = 0; n < H; ++n) {
            const double2 v = src[n * step];
            const double mm = __ldg(row + n);
            acc.x = fma(mm, v.x, acc.x);
            acc.y = fma(mm, v.y, acc.y);
          }
          g[(long long)kk * st] = acc;
        }
        {
          const int kk = 2 * m + pf, b1 = m & 1;  // (kk >> 1) & 1
          const double2* src;
          int step;
          if (pf == 0) { src = b1 ? line + (long long)(H - 1) * LPC : line; step = b1 ? -LPC : LPC; }
          else { src = b1 ? line + (long long)H * LPC : line + (long long)(N - 1) * LPC; step = b1 ? LPC : -LPC; }
          const double* __restrict__ row = M + (long long)kk * N;
          double2 acc = make_double2(0.0, 0.0);
          for (int n = 0; n < Q; ++n) {
            const double2 v = src[n * step];
            const double mm = __ldg(row + n);
            acc.x = fma(mm, v.x, acc.x);
            acc.y = fma(mm, v.y, acc.y);
          }
          g[(long long)kk * st] = acc;
        }
      }
      return;
    }
    if (!valid) return;
    for (int kk = t; kk < N; kk += T) {  // kk has the parity of t
      const double2* src = (kk & 1) ? line + (long long)(N - 1) * LPC : line;
      const int step = (kk & 1) ? -LPC : LPC;
      const double* __restrict__ row = M + (long long)kk * N;
      double2 acc = make_double2(0.0, 0.0);
      for (int n = 0; n < H; ++n) {
        const double2 v = src[n * step];
        const double m = __ldg(row + n);
        acc.x = fma(m, v.x, acc.x);
        acc.y = fma(m, v.y, acc.y);
      }
      g[(long long)kk * st] = acc;
    }
    return;
  }
  const int lvi = (S.sym[AXIS] >> 4) & 3;  // bit p: the columns of parity p fold once more
  if (sym && (lvi == 1 || lvi == 2) && N % 8 == 0) {
    // Row pairs (n, H-1-n), n < H/2, from the second fold of the columns of
    // parity pf (see dense_x_inv_body).  The two threads t and t^1 of a pair
    // (lanes 16 apart) take one half of the columns each and add their sums
    // by shuffle; every lane stays in the loop for the shuffles.
    const int H = N / 2, Q = H / 2, pf = lvi == 1 ? 0 : 1, pu = 1 - pf;
    const int half = t & 1, pr = t >> 1;
    const int c0 = half ? H : 0, c1 = half ? N : H;
    for (int n = pr; n < Q; n += T / 2) {
      const int m = H - 1 - n;
      const double* __restrict__ rn = M + (long long)n * N;
      const double* __restrict__ rm = M + (long long)m * N;
      double2 f0 = make_double2(0.0, 0.0), f1 = f0, un = f0, um = f0;
      for (int c = c0; c < c1; c += 4) {
        const double2 x0 = line[(c + pf) * LPC], x1 = line[(c + pf + 2) * LPC];
        const double2 y0 = line[(c + pu) * LPC], y1 = line[(c + pu + 2) * LPC];
        const double a0 = __ldg(rn + c + pf), a1 = __ldg(rn + c + pf + 2);
        const double b0 = __ldg(rn + c + pu), b1 = __ldg(rn + c + pu + 2);
        const double e0 = __ldg(rm + c + pu), e1 = __ldg(rm + c + pu + 2);
        f0.x = fma(a0, x0.x, f0.x); f0.y = fma(a0, x0.y, f0.y);
        f1.x = fma(a1, x1.x, f1.x); f1.y = fma(a1, x1.y, f1.y);
        un.x = fma(b0, y0.x, un.x); un.y = fma(b0, y0.y, un.y);
        un.x = fma(b1, y1.x, un.x); un.y = fma(b1, y1.y, un.y);
        um.x = fma(e0, y0.x, um.x); um.y = fma(e0, y0.y, um.y);
        um.x = fma(e1, y1.x, um.x); um.y = fma(e1, y1.y, um.y);
      }
      f0.x += __shfl_xor_sync(0xffffffffu, f0.x, 16); f0.y += __shfl_xor_sync(0xffffffffu, f0.y, 16);
      f1.x += __shfl_xor_sync(0xffffffffu, f1.x, 16); f1.y += __shfl_xor_sync(0xffffffffu, f1.y, 16);
      un.x += __shfl_xor_sync(0xffffffffu, un.x, 16); un.y += __shfl_xor_sync(0xffffffffu, un.y, 16);
      um.x += __shfl_xor_sync(0xffffffffu, um.x, 16); um.y += __shfl_xor_sync(0xffffffffu, um.y, 16);
      if (valid && half == 0) {
        const double2 fn = make_double2(f0.x + f1.x, f0.y + f1.y), fm = make_double2(f0.x - f1.x, f0.y - f1.y);
        const double2 en = pf ? un : fn, on = pf ? fn : un;  // even and odd sums of row n
        const double2 em = pf ? um : fm, om = pf ? fm : um;  // and of row m
        g[(long long)n * st] = make_double2(en.x + on.x, en.y + on.y);
        g[(long long)(N - 1 - n) * st] = make_double2(en.x - on.x, en.y - on.y);
        g[(long long)m * st] = make_double2(em.x + om.x, em.y + om.y);
        g[(long long)(N - 1 - m) * st] = make_double2(em.x - om.x, em.y - om.y);
      }
    }
    return;
  }
  if (sym) {
    // G[N-1-n][k] = (-1)^k G[n][k]: even and odd partial sums of row n give
    // out[n] = E + O and out[N-1-n] = E - O
    if (!valid) return;
    const int H = N / 2;
    for (int r = t; r < H; r += T) {
      const double* __restrict__ row = M + (long long)r * N;
      double2 e = make_double2(0.0, 0.0), od = make_double2(0.0, 0.0);
      for (int c = 0; c + 1 < N; c += 2) {
        const double2 v0 = line[c * LPC], v1 = line[(c + 1) * LPC];
        const double m0 = __ldg(row + c), m1 = __ldg(row + c + 1);
        e.x = fma(m0, v0.x, e.x);
        e.y = fma(m0, v0.y, e.y);
        od.x = fma(m1, v1.x, od.x);
        od.y = fma(m1, v1.y, od.y);
      }
      g[(long long)r * st] = make_double2(e.x + od.x, e.y + od.y);
      g[(long long)(N - 1 - r) * st] = make_double2(e.x - od.x, e.y - od.y);
    }
    return;
  }
  // general N: the full matrix product, outputs k = t + T*q
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
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int kk = t + T * q;
    if (q < nq && kk < N) g[(long long)kk * st] = acc[q];
  }
}

// ---------------------------------------------------------------------------
// Tridiagonal solve along the wall axis s.  After the transforms of the other
// two axes every spectrum line along s is an independent system
//   p[j-1] - (2 - e_j - sigma h^2) p[j] + p[j+1] = h^2 scale rhs[j],
// sigma = lambda_x + lambda_other, e_j the pressure-BC change of the end rows.
// Its solution is that of the per-axis transform, eigenvalue divide and
// inverse transform of DCT_poisson_solver (NS_functions.f90:1505-1630) along s.
// The solve used for lines of 8 rows and more is the twisted factorisation
// from a table of multipliers (tri_twist_body, below); this one-thread
// Thomas solve (no pivoting: the rows are diagonally dominant) computes its
// multipliers into shared memory and serves shorter lines.  The one singular
// line (Neumann/periodic everywhere, both modes 0) drops its rhs mean, pins
// its last entry and takes the mean value (NS_functions.f90:1576-1577).
// ---------------------------------------------------------------------------
constexpr int TRI_T = 32;  // lines per CTA (one warp)

// One real component of a line, general path (the singular line).
__device__ void tri_real(double* x, long long sx, int N, double sig_h2, double elo, double ehi, double rs, double* cm,
                         bool sing, double target) {
  double mean_r = 0.0;
  if (sing) {
    for (int j = 0; j < N; ++j) mean_r += x[j * sx];
    mean_r /= N;
  }
  const int last = sing ? N - 2 : N - 1;
  double m = 0.0, d = 0.0;
  for (int j = 0; j <= last; ++j) {
    double b = -2.0 + sig_h2;
    if (j == 0) b += elo;
    if (j == N - 1) b += ehi;
    m = 1.0 / (b - m);
    d = fma(x[j * sx] - mean_r, rs, -d) * m;
    x[j * sx] = d;
    cm[j * TRI_T] = m;
  }
  double p = 0.0;
  if (sing) x[(long long)(N - 1) * sx] = 0.0;
  else p = d;
  for (int j = N - 2; j >= 0; --j) {
    p = fma(-cm[j * TRI_T], p, x[j * sx]);
    x[j * sx] = p;
  }
  if (sing) {
    double mp = 0.0;
    for (int j = 0; j < N; ++j) mp += x[j * sx];
    const double shift = target - mp / N;
    for (int j = 0; j < N; ++j) x[j * sx] += shift;
  }
}

// The singular line by a whole warp.  Its system is the Neumann one along
// the axis (end rows -x_0 + x_1, x_{N-2} - x_{N-1}; sigma = 0), whose
// solution with the rhs mean dropped and the mean set to target (the
// reference pins the last entry and shifts, NS_functions.f90:1576-1577) is
// the flux F_j = x_{j+1} - x_j = sum_{i<=j} R_i, R = rs (r - mean r), then
// x_j = sum_{i<j} F_i shifted to the target mean: two prefix sums over the
// warp, lane l holding the rows [l seg, l seg + seg), seg = ceil(N/32).  r is
// read from src (stride 1, re-read by each pass), the solution written to x
// (stride sx doubles).
__device__ __noinline__ void sing_line_warp(const double* src, double* x, long long sx, int N, double rs,
                                            double target) {
  const int lane = threadIdx.x & 31;
  const int seg = (N + 31) / 32, j0 = min(lane * seg, N), j1 = min(j0 + seg, N);
  auto warp_sum = [](double v) {
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
  };
  auto warp_excl = [&](double tot) {  // exclusive scan of the lanes' totals
    double incl = tot;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += y;
    }
    return incl - tot;
  };
  double s = 0.0;
  for (int j = j0; j < j1; ++j) s += src[j];
  const double mean_r = warp_sum(s) / N;
  s = 0.0;
  for (int j = j0; j < j1; ++j) s += (src[j] - mean_r) * rs;
  const double f0 = warp_excl(s);  // F before this lane's rows
  // x_j = x_{j0} + sum_{j0<=i<j} F_i: the lane's sum of F over its rows
  double fs = 0.0, f = f0;
  for (int j = j0; j < j1; ++j) {
    f += (src[j] - mean_r) * rs;
    fs += f;
  }
  const double xb = warp_excl(fs);  // x at this lane's first row (x_0 = 0)
  double xv = xb, ms = 0.0;
  f = f0;
  for (int j = j0; j < j1; ++j) {
    x[(long long)j * sx] = xv;
    ms += xv;
    f += (src[j] - mean_r) * rs;
    xv += f;
  }
  const double shift = target - warp_sum(ms) / N;
  __syncwarp();
  for (int j = j0; j < j1; ++j) x[(long long)j * sx] += shift;
}


template <int AXIS, bool PACKED>
__device__ __forceinline__ void tri_solve_body(const SpecPlan& S, double2* __restrict__ spec, double* cm, int bx,
                                               int by) {
  // cm: [N][TRI_T] multipliers (x2 when PACKED)
  const int l = threadIdx.x;
  const int N = AXIS == 1 ? S.ny : S.nz;
  const int n_other = AXIS == 1 ? S.nz : S.ny;
  // Columns: with a periodic x the Nyquist column is handled by the last
  // block column, lanes over the other index (no idle lanes).
  const int nreg = PACKED ? S.nxs : S.nxs - 1;
  const int nblk = (nreg + TRI_T - 1) / TRI_T;
  int col, o;
  bool valid;
  if (bx < nblk) {
    col = bx * TRI_T + l;
    o = by;
    valid = col < nreg;
  } else {
    if (by * TRI_T >= n_other) return;
    col = S.nxs - 1;
    o = by * TRI_T + l;
    valid = o < n_other;
  }
  if (!valid) return;
  const long long st = AXIS == 1 ? (long long)S.nxs : (long long)S.nxs * S.ny;
  double2* g = spec + (AXIS == 1 ? col + (long long)S.nxs * S.ny * o : col + (long long)S.nxs * o);
  const double lo = __ldg(S.eig_o + o);
  const double sr = (__ldg(S.eig_x + (PACKED ? 2 * col : col)) + lo) * S.tri_h2;
  const double si = PACKED ? (__ldg(S.eig_x + 2 * col + 1) + lo) * S.tri_h2 : sr;
  const double rs = S.tri_rs, elo = S.tri_elo, ehi = S.tri_ehi;
  double* cmr = cm + l;
  double* cmi = PACKED ? cm + (long long)N * TRI_T + l : cmr;
  if (S.has_mean && col == 0 && o == 0) {  // the singular line
    double* x = reinterpret_cast<double*>(g);
    tri_real(x, 2 * st, N, sr, elo, ehi, rs, cmr, true, S.mean_dev ? S.mean_val * *S.mean_dev : S.mean_val);
    tri_real(x + 1, 2 * st, N, si, elo, ehi, rs, cmi, !PACKED, 0.0);
    return;
  }
  double mr = 0.0, mi = 0.0;
  double2 d = make_double2(0.0, 0.0);
#pragma unroll 4
  for (int j = 0; j < N; ++j) {
    double br = -2.0 + sr, bi = -2.0 + si;
    if (j == 0) { br += elo; bi += elo; }
    if (j == N - 1) { br += ehi; bi += ehi; }
    mr = 1.0 / (br - mr);
    if (PACKED) mi = 1.0 / (bi - mi);
    else mi = mr;
    const double2 r = g[(long long)j * st];
    d.x = fma(r.x, rs, -d.x) * mr;
    d.y = fma(r.y, rs, -d.y) * mi;
    g[(long long)j * st] = d;
    cmr[j * TRI_T] = mr;
    if (PACKED) cmi[j * TRI_T] = mi;
  }
  double2 p = d;
#pragma unroll 4
  for (int j = N - 2; j >= 0; --j) {
    const double2 x = g[(long long)j * st];
    p.x = fma(-cmr[j * TRI_T], p.x, x.x);
    p.y = fma(-cmi[j * TRI_T], p.y, x.y);
    g[(long long)j * st] = p;
  }
}

__global__ void __launch_bounds__(128) dense_x_fwd_kernel(SpecPlan S, DivArgs d, double2* __restrict__ spec) {
  extern __shared__ __align__(16) double xs_fwd[];
  dense_x_fwd_body(S, d, spec, xs_fwd, blockIdx.x);
}
__global__ void __launch_bounds__(128) dense_x_inv_kernel(SpecPlan S, const double2* __restrict__ spec, double* dp,
                                                          Layout L) {
  extern __shared__ __align__(16) double xs_inv[];
  dense_x_inv_body(S, spec, dp, L, xs_inv, blockIdx.x);
}
template <int AXIS, bool FWD>
__global__ void __launch_bounds__(128) dense_yz_kernel(SpecPlan S, double2* __restrict__ spec) {
  extern __shared__ __align__(16) double2 ls_yz[];
  dense_yz_body<AXIS, FWD>(S, spec, ls_yz, blockIdx.x);
}

template <int AXIS, bool PACKED>
__global__ void __launch_bounds__(TRI_T) tri_solve_kernel(SpecPlan S, double2* __restrict__ spec) {
  extern __shared__ __align__(16) double cm_tri[];
  tri_solve_body<AXIS, PACKED>(S, spec, cm_tri, blockIdx.x, blockIdx.y);
}


// ---------------------------------------------------------------------------
// Twisted, table-driven line solve (the session's wall axis, 1 or 2, and
// the batch's z axis).  Line
// t = col + nxs o (o: z for y lines, y for z lines) of N rows; k = N/2.  Its
// table holds m_j = 1/(b_j - m_{j-1}) for j < k (top-down, as tri_solve_body),
// n_j = 1/(b_j - n_{j+1}) for j > k (bottom-up) and the middle pivot
// 1/(b_k - m_{k-1} - n_{k+1}).  Lanes l and l + 16 of a warp take line l:
// the top lane forms d_j = (rs r_j - d_{j-1}) m_j downwards, the bottom lane
// e_j = (rs r_j - e_{j+1}) n_j upwards; the middle row gives
// x_k = (rs r_k - d_{k-1} - e_{k+1}) piv, and the lanes substitute outwards,
// x_j = d_j - m_j x_{j+1} above and x_j = e_j - n_j x_{j-1} below.  No
// division in the solve, twice the lines' lanes in flight and half the
// recurrence length of the one-lane Thomas solve; the sums round
// differently.  The singular line takes the general path on its top lane.
// ---------------------------------------------------------------------------
struct TwLine {
  long long base, st;
  int col, o;
  bool valid;
};
template <int AXIS>
__device__ __forceinline__ TwLine tw_line(const SpecPlan& S, int t) {
  TwLine L;
  L.valid = t < S.nxs * (AXIS == 1 ? S.nz : S.ny);
  if (!L.valid) t = 0;
  L.col = t % S.nxs;
  L.o = t / S.nxs;
  if (AXIS == 1) { L.base = L.col + (long long)S.nxs * S.ny * L.o; L.st = S.nxs; }
  else { L.base = t; L.st = (long long)S.nxs * S.ny; }
  return L;
}

template <int AXIS, bool PACKED>
__global__ void __launch_bounds__(128) tri_twist_table_kernel(SpecPlan S, double2* __restrict__ tab) {
  const TwLine ln = tw_line<AXIS>(S, blockIdx.x * 128 + threadIdx.x);
  if (!ln.valid) return;
  const int N = AXIS == 1 ? S.ny : S.nz, k = N / 2;
  const double lo = __ldg(S.eig_o + ln.o);
  const double sr = (__ldg(S.eig_x + (PACKED ? 2 * ln.col : ln.col)) + lo) * S.tri_h2;
  const double si = PACKED ? (__ldg(S.eig_x + 2 * ln.col + 1) + lo) * S.tri_h2 : sr;
  const double elo = S.tri_elo, ehi = S.tri_ehi;
  auto bj = [&](int j, double s) {
    double b = -2.0 + s;
    if (j == 0) b += elo;
    if (j == N - 1) b += ehi;
    return b;
  };
  double2* g = tab + ln.base;
  double mr = 0.0, mi = 0.0;
  for (int j = 0; j < k; ++j) {
    mr = 1.0 / (bj(j, sr) - mr);
    mi = PACKED ? 1.0 / (bj(j, si) - mi) : mr;
    g[(long long)j * ln.st] = make_double2(mr, mi);
  }
  double nr = 0.0, ni = 0.0;
  for (int j = N - 1; j > k; --j) {
    nr = 1.0 / (bj(j, sr) - nr);
    ni = PACKED ? 1.0 / (bj(j, si) - ni) : nr;
    g[(long long)j * ln.st] = make_double2(nr, ni);
  }
  const double pr = 1.0 / (bj(k, sr) - mr - nr);
  const double pi = PACKED ? 1.0 / (bj(k, si) - mi - ni) : pr;
  g[(long long)k * ln.st] = make_double2(pr, pi);
}

// One 128-thread block bx of the twisted solve (64 lines); scr: scratch of
// 2 N TRI_T doubles for the singular line.
template <int AXIS, bool PACKED>
__device__ __forceinline__ void tri_twist_body(const SpecPlan& S, double2* __restrict__ spec, double* scr, int bx) {
  constexpr int TP = 4;  // rows and multipliers loaded ahead
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, h = lane >> 4;
  const int t0 = (bx * 4 + warp) * 16;
  if (t0 >= S.nxs * (AXIS == 1 ? S.nz : S.ny)) return;  // the whole warp
  const TwLine ln = tw_line<AXIS>(S, t0 + (lane & 15));
  const int N = AXIS == 1 ? S.ny : S.nz, k = N / 2;
  // The singular line (col 0, o 0: lane 0 of the first warp) of a Neumann
  // axis goes to the whole warp after the other lines (sing_line_warp); its
  // rhs is set aside in the scratch first, since the twisted lanes also run
  // over it (a packed box's second mode of that slot is a regular line).
  // Otherwise it takes the one-lane general path on its top lane.
  const bool warp_sing = t0 == 0 && S.has_mean && S.tri_elo == 1.0 && S.tri_ehi == 1.0 && N <= 512;
  const bool sing = ln.valid && S.has_mean && ln.col == 0 && ln.o == 0;
  const bool work = ln.valid && (!sing || warp_sing);
  if (warp_sing) {
    const double2* g0 = spec;  // line (0, 0)
    for (int j = lane; j < N; j += 32) {
      const double2 r = g0[(long long)j * (AXIS == 1 ? (long long)S.nxs : (long long)S.nxs * S.ny)];
      scr[j] = r.x;
      if (!PACKED) scr[N + j] = r.y;
    }
    __syncwarp();
  }
  double2* g = spec + ln.base;
  const double2* __restrict__ tm = S.tri_m + ln.base;
  const long long st = ln.st;
  const double rs = S.tri_rs;
  const int cnt = h ? N - 1 - k : k;
  auto row = [&](int q) { return h ? N - 1 - q : q; };
  const double2 z2 = make_double2(0.0, 0.0);
  // elimination towards the middle row
  double2 d = z2;
  if (work) {
    double2 rv[TP], mv[TP];
#pragma unroll
    for (int q = 0; q < TP; ++q) {
      const bool in = q < cnt;
      rv[q] = in ? g[(long long)row(q) * st] : z2;
      mv[q] = in ? __ldg(tm + (long long)row(q) * st) : z2;
    }
    for (int q0 = 0; q0 < cnt; q0 += TP) {
      double2 rn[TP], mn[TP];
#pragma unroll
      for (int q = 0; q < TP; ++q) {
        const int qq = q0 + TP + q;
        const bool in = qq < cnt;
        rn[q] = in ? g[(long long)row(qq) * st] : z2;
        mn[q] = in ? __ldg(tm + (long long)row(qq) * st) : z2;
      }
#pragma unroll
      for (int q = 0; q < TP; ++q)
        if (q0 + q < cnt) {
          d.x = fma(rv[q].x, rs, -d.x) * mv[q].x;
          d.y = fma(rv[q].y, rs, -d.y) * mv[q].y;
          g[(long long)row(q0 + q) * st] = d;
        }
#pragma unroll
      for (int q = 0; q < TP; ++q) {
        rv[q] = rn[q];
        mv[q] = mn[q];
      }
    }
  }
  // the middle row, on the top lane, with the bottom lane's e_{k+1}
  const double ex = __shfl_xor_sync(0xffffffffu, d.x, 16), ey = __shfl_xor_sync(0xffffffffu, d.y, 16);
  double2 xk = z2;
  if (work && h == 0) {
    const double2 r = g[(long long)k * st];
    const double2 pv = __ldg(tm + (long long)k * st);
    xk.x = (fma(r.x, rs, -d.x) - ex) * pv.x;
    xk.y = (fma(r.y, rs, -d.y) - ey) * pv.y;
    g[(long long)k * st] = xk;
  }
  xk.x = __shfl_sync(0xffffffffu, xk.x, lane & 15);
  xk.y = __shfl_sync(0xffffffffu, xk.y, lane & 15);
  // substitution away from the middle row (row index cnt - 1 - q)
  if (work) {
    double2 p = xk;
    double2 rv[TP], mv[TP];
#pragma unroll
    for (int q = 0; q < TP; ++q) {
      const int qq = cnt - 1 - q;
      const bool in = qq >= 0;
      rv[q] = in ? g[(long long)row(qq) * st] : z2;
      mv[q] = in ? __ldg(tm + (long long)row(qq) * st) : z2;
    }
    for (int q0 = 0; q0 < cnt; q0 += TP) {
      double2 rn[TP], mn[TP];
#pragma unroll
      for (int q = 0; q < TP; ++q) {
        const int qq = cnt - 1 - (q0 + TP + q);
        const bool in = qq >= 0;
        rn[q] = in ? g[(long long)row(qq) * st] : z2;
        mn[q] = in ? __ldg(tm + (long long)row(qq) * st) : z2;
      }
#pragma unroll
      for (int q = 0; q < TP; ++q) {
        const int qq = cnt - 1 - (q0 + q);
        if (qq >= 0) {
          p.x = fma(-mv[q].x, p.x, rv[q].x);
          p.y = fma(-mv[q].y, p.y, rv[q].y);
          g[(long long)row(qq) * st] = p;
        }
      }
#pragma unroll
      for (int q = 0; q < TP; ++q) {
        rv[q] = rn[q];
        mv[q] = mn[q];
      }
    }
  }
  const double target = S.mean_dev ? S.mean_val * *S.mean_dev : S.mean_val;
  if (warp_sing) {
    __syncwarp();
    const long long st0 = AXIS == 1 ? (long long)S.nxs : (long long)S.nxs * S.ny;
    double* x0 = reinterpret_cast<double*>(spec);
    sing_line_warp(scr, x0, 2 * st0, N, rs, target);
    if (!PACKED) sing_line_warp(scr + N, x0 + 1, 2 * st0, N, rs, 0.0);
  } else if (sing && h == 0) {
    const double lo = __ldg(S.eig_o);
    const double sr = (__ldg(S.eig_x) + lo) * S.tri_h2;
    const double si = PACKED ? (__ldg(S.eig_x + 1) + lo) * S.tri_h2 : sr;
    double* x = reinterpret_cast<double*>(g);
    tri_real(x, 2 * st, N, sr, S.tri_elo, S.tri_ehi, rs, scr, true, target);
    tri_real(x + 1, 2 * st, N, si, S.tri_elo, S.tri_ehi, rs, scr + (long long)N * TRI_T, !PACKED, 0.0);
  }
}

template <int AXIS, bool PACKED>
__global__ void __launch_bounds__(128) tri_twist_solve_kernel(SpecPlan S, double2* __restrict__ spec) {
  tri_twist_body<AXIS, PACKED>(S, spec, S.sing_cm, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Batched passes: persistent CTAs walk (subdomain, block) work items; the
// subdomain's arguments are staged in shared memory once per item.
// PASS: 0 x forward, 1 x inverse, 2 y forward, 3 y inverse, 4 tridiagonal z (packed x,
// the twisted solve from the subdomain's table).
// A subdomain whose plan sets dct_x / dct_y (an axis of 24, 32, 48 or 64
// points, pressure code 2 or 3) takes the FFT-based line bodies of
// ns_fft_core.cuh there, with 128 / R1 lines per item so that all 128
// threads work; the others take the dense products.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int batch_dct_lpc(int n) {
  return 128 / (n == 64 ? Split<64>::R1 : n == 48 ? Split<48>::R1 : n == 32 ? Split<32>::R1 : Split<24>::R1);
}

template <int N, int PB>
__device__ __forceinline__ void batch_dct(int pass, const BatchSpecArgs& a, double2* sb, int bx) {
  constexpr int LPC = batch_dct_lpc(N);
  const FOne c{a.d.one, a.d.mzero};
  const int l = threadIdx.x % LPC, t = threadIdx.x / LPC;
  if (pass == 0) dct_x_fwd_body<N, PB, false, LPC>(a.S, nullptr, a.spec, sb, bx, l, t, c);
  else if (pass == 1) dct_x_inv_body<N, PB, LPC>(a.S, a.spec, a.dp, a.L, sb, bx, l, t, c);
  else if (pass == 2) dct_y_body<N, true, PB, LPC>(a.S, a.spec, sb, bx, l, t, c);
  else dct_y_body<N, false, PB, LPC>(a.S, a.spec, sb, bx, l, t, c);
}

template <int PASS>
__device__ __forceinline__ void batch_dct_dispatch(const BatchSpecArgs& a, double2* sb, int bx) {
  const int n = PASS < 2 ? a.S.nx : a.S.ny;
  const int pb = PASS < 2 ? a.S.dct_x : a.S.dct_y;
  if (n == 64) {
    if (pb == 2) batch_dct<64, 2>(PASS, a, sb, bx);
    else batch_dct<64, 3>(PASS, a, sb, bx);
  } else if (n == 48) {
    if (pb == 2) batch_dct<48, 2>(PASS, a, sb, bx);
    else batch_dct<48, 3>(PASS, a, sb, bx);
  } else if (n == 32) {
    if (pb == 2) batch_dct<32, 2>(PASS, a, sb, bx);
    else batch_dct<32, 3>(PASS, a, sb, bx);
  } else {
    if (pb == 2) batch_dct<24, 2>(PASS, a, sb, bx);
    else batch_dct<24, 3>(PASS, a, sb, bx);
  }
}

template <int PASS>
__global__ void __launch_bounds__(128) spec_batch_kernel(const BatchSpecArgs* __restrict__ tab,
                                                         const BatchItem* __restrict__ items, int n_items) {
  extern __shared__ __align__(16) double sm_b[];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    // the subdomain's arguments from the read-only table (a copy in shared
    // memory would be reloaded after every barrier of the passes)
    const BatchSpecArgs& a = tab[w.sub];
    if (PASS == 0) dense_x_fwd_body(a.S, a.d, a.spec, sm_b, w.bx);
    if (PASS == 1) dense_x_inv_body(a.S, a.spec, a.dp, a.L, sm_b, w.bx);
    if (PASS == 2) dense_yz_body<1, true>(a.S, a.spec, reinterpret_cast<double2*>(sm_b), w.bx);
    if (PASS == 3) dense_yz_body<1, false>(a.S, a.spec, reinterpret_cast<double2*>(sm_b), w.bx);
    if (PASS == 4) tri_twist_body<2, true>(a.S, a.spec, sm_b, w.bx);
    __syncthreads();
  }
}

template <int PASS>
__global__ void __launch_bounds__(128) spec_batch_dct_kernel(const BatchSpecArgs* __restrict__ tab,
                                                             const BatchItem* __restrict__ items, int n_items) {
  extern __shared__ __align__(16) double2 sm_d[];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    batch_dct_dispatch<PASS>(tab[w.sub], sm_d, w.bx);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kDivChunk) spec_batch_div_kernel(const BatchSpecArgs* __restrict__ tab,
                                                                   const BatchItem* __restrict__ items, int n_items) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const BatchSpecArgs& a = tab[w.sub];
    const unsigned N = (unsigned)a.S.nx;
    const unsigned e = (unsigned)w.bx * kDivChunk + threadIdx.x;  // a subdomain box holds < 2^31 cells
    if (e < N * (unsigned)a.S.ny * (unsigned)a.S.nz) {
      const int row = (int)(e / N), i = (int)(e - (unsigned)row * N);
      const FOne c{a.d.one, a.d.mzero};
      const DivArgs& d = a.d;
      double v;
      if (d.rhs) {
        v = d.rhs[d.L.at(i + 1, 1 + row % a.S.ny, 1 + row / a.S.ny)];
      } else {  // the divergence; the boundary cells' terms follow in spec_batch_bc_kernel
        const long long g = d.L.at(i + 1, 1 + row % a.S.ny, 1 + row / a.S.ny);
        v = fmul(c, fsub(c, d.us[g + 1], d.us[g]), d.cdx);
        v = fma(fsub(c, d.vs[g + d.L.sy], d.vs[g]), d.cdy, v);
        v = fma(fsub(c, d.ws[g + d.L.sz], d.ws[g]), d.cdz, v);
        v = v + 0.0;
      }
      reinterpret_cast<double*>(a.spec)[e] = v;
    }
  }
}

// The pressure-BC terms of those subdomains' boundary cells, added to their
// divergence rows (item (sub, q): boundary cells [kDivChunk q, kDivChunk (q+1))
// in the order of SpecPlan::bc_cell).
__global__ void __launch_bounds__(kDivChunk) spec_batch_bc_kernel(const BatchSpecArgs* __restrict__ tab,
                                                                  const BatchItem* __restrict__ items, int n_items) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const BatchSpecArgs& a = tab[w.sub];
    const long long q = (long long)w.bx * kDivChunk + threadIdx.x;
    if (q < a.S.bc_cells()) {
      int i, j, k;
      a.S.bc_cell(q, i, j, k);
      double* out = reinterpret_cast<double*>(a.spec);
      const long long e = (long long)a.S.nx * ((j - 1) + (long long)a.S.ny * (k - 1)) + (i - 1);
      out[e] = out[e] + a.S.bc_term_edge(i, j, k);
    }
  }
}

cudaError_t launch_spec_batch_bc(const BatchSpecArgs* tab, const BatchItem* items, int n_items, int grid,
                                 cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  if (grid <= 0) grid = 8 * 152;
  if (grid > n_items) grid = n_items;
  spec_batch_bc_kernel<<<grid, kDivChunk, 0, st>>>(tab, items, n_items);
  return cudaGetLastError();
}

cudaError_t launch_spec_batch_div(const BatchSpecArgs* tab, const BatchItem* items, int n_items, int grid,
                                  cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  if (grid <= 0) {
    int per_sm = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spec_batch_div_kernel, kDivChunk, 0);
    grid = (per_sm > 0 ? per_sm : 1) * nsm;
  }
  if (grid > n_items) grid = n_items;
  spec_batch_div_kernel<<<grid, kDivChunk, 0, st>>>(tab, items, n_items);
  return cudaGetLastError();
}

bool spec_pass_dct(int pass, const SpecPlan& S) {
  return ((pass == 0 || pass == 1) && S.dct_x) || ((pass == 2 || pass == 3) && S.dct_y);
}

// Work-item grid of one pass for one subdomain.
void spec_pass_grid(int pass, const SpecPlan& S, int& gx, int& gy) {
  gy = 1;
  if ((pass == 0 || pass == 1) && S.dct_x) gx = (S.ny * S.nz + 2 * batch_dct_lpc(S.nx) - 1) / (2 * batch_dct_lpc(S.nx));
  else if ((pass == 2 || pass == 3) && S.dct_y) gx = (S.nxs * S.nz + batch_dct_lpc(S.ny) - 1) / batch_dct_lpc(S.ny);
  else if (pass == 0 || pass == 1) {
    const int per = 128 / (pass == 0 ? dense_x_group(S.nx) : dense_x_inv_group(S.sym[0], S.nx));
    gx = (S.ny * S.nz + per - 1) / per;
  }
  else if (pass == 2 || pass == 3) gx = (S.nxs * S.nz + 15) / 16;  // dense_yz_body: 16 lines per item
  else gx = (S.nxs * S.ny + 63) / 64;  // tri_twist_body: 64 lines per item
}

size_t spec_pass_smem(int pass, const SpecPlan& S) {
  if ((pass == 0 || pass == 1) && S.dct_x) {
    const size_t L = batch_dct_lpc(S.nx);
    return (size_t)S.nx * L * sizeof(double2) + L * (S.nx + 1) * sizeof(double2);
  }
  if ((pass == 2 || pass == 3) && S.dct_y) return (size_t)S.ny * batch_dct_lpc(S.ny) * sizeof(double2);
  if (pass == 0) return (size_t)(128 / dense_x_group(S.nx)) * S.nx * sizeof(double);
  if (pass == 1) return (size_t)(128 / dense_x_inv_group(S.sym[0], S.nx)) * S.nx * sizeof(double);
  if (pass == 2 || pass == 3) return (size_t)S.ny * 16 * sizeof(double2);
  return (size_t)S.nz * TRI_T * sizeof(double) * 2;
}

cudaError_t launch_spec_batch(int pass, bool dct, const BatchSpecArgs* tab, const BatchItem* items, int n_items,
                              size_t smem, int grid, cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  if (dct && (pass < 0 || pass > 3)) return cudaErrorInvalidValue;
  auto kern = dct ? (pass == 0 ? spec_batch_dct_kernel<0>
                   : pass == 1 ? spec_batch_dct_kernel<1>
                   : pass == 2 ? spec_batch_dct_kernel<2>
                               : spec_batch_dct_kernel<3>)
            : pass == 0 ? spec_batch_kernel<0>
            : pass == 1 ? spec_batch_kernel<1>
            : pass == 2 ? spec_batch_kernel<2>
            : pass == 3 ? spec_batch_kernel<3>
                        : spec_batch_kernel<4>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (grid <= 0) {
    int per_sm = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
    grid = (per_sm > 0 ? per_sm : 1) * nsm;
  }
  if (grid > n_items) grid = n_items;
  kern<<<grid, 128, smem, st>>>(tab, items, n_items);
  return cudaGetLastError();
}

cudaError_t launch_dense_x(bool fwd, const SpecPlan& S, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                           cudaStream_t st) {
  const int lines = S.ny * S.nz, per = 128 / (fwd ? dense_x_group(S.nx) : dense_x_inv_group(S.sym[0], S.nx));
  const size_t sm = (size_t)per * S.nx * sizeof(double);
  if (fwd) dense_x_fwd_kernel<<<(lines + per - 1) / per, 128, sm, st>>>(S, d, spec);
  else dense_x_inv_kernel<<<(lines + per - 1) / per, 128, sm, st>>>(S, spec, dp, L);
  return cudaGetLastError();
}

int dense_symmetry(int n, const std::vector<double>& F, const std::vector<double>& G) {
  if (n < 2 || n % 2) return 0;
  double fm = 0.0, gm = 0.0;
  for (double x : F) fm = std::fmax(fm, std::fabs(x));
  for (double x : G) gm = std::fmax(gm, std::fabs(x));
  bool fs = true, gs = true;
  for (int r = 0; r < n && (fs || gs); ++r)
    for (int q = 0; q < n; ++q) {
      const double sg_r = (r & 1) ? -1.0 : 1.0, sg_q = (q & 1) ? -1.0 : 1.0;
      if (std::fabs(F[(size_t)r * n + (n - 1 - q)] - sg_r * F[(size_t)r * n + q]) > 4e-16 * fm) fs = false;
      if (std::fabs(G[(size_t)(n - 1 - r) * n + q] - sg_q * G[(size_t)r * n + q]) > 4e-16 * gm) gs = false;
    }
  int bits = (fs ? 1 : 0) | (gs ? 2 : 0);
  // Second level: within the modes of one parity, over the first H = n/2
  // points, F[k][H-1-q] = s_k F[k][q] and G[H-1-q][k] = s_k G[q][k] with
  // s_k = (-1)^((k >> 1) & 1).  DCT-II has it on its even modes (a half-size
  // DCT-II), DST-II on its odd ones.
  const int H = n / 2;
  if (H % 2 == 0) {
    bool f1[2] = {fs, fs}, g1[2] = {gs, gs};
    for (int k = 0; k < n; ++k) {
      const double sg = ((k >> 1) & 1) ? -1.0 : 1.0;
      for (int q = 0; q < H; ++q) {
        if (std::fabs(F[(size_t)k * n + (H - 1 - q)] - sg * F[(size_t)k * n + q]) > 4e-16 * fm) f1[k & 1] = false;
        if (std::fabs(G[(size_t)(H - 1 - q) * n + k] - sg * G[(size_t)q * n + k]) > 4e-16 * gm) g1[k & 1] = false;
      }
    }
    bits |= (f1[0] ? 4 : 0) | (f1[1] ? 8 : 0) | (g1[0] ? 16 : 0) | (g1[1] ? 32 : 0);
  }
  return bits;
}

cudaError_t launch_dense_yz(int axis, bool fwd, const SpecPlan& S, double2* spec, cudaStream_t st) {
  const int N = axis == 1 ? S.ny : S.nz;
  if (N > 512) return cudaErrorInvalidValue;
  // 16 lines of N complex values staged in shared memory: 32 KB at N = 128,
  // 128 KB at 512 (past the 48 KB default: opt in)
  const size_t sm = (size_t)N * 16 * sizeof(double2);
  dim3 grid((S.nxs * (axis == 1 ? S.nz : S.ny) + 15) / 16);
  auto kern = (axis == 1) ? (fwd ? dense_yz_kernel<1, true> : dense_yz_kernel<1, false>)
                          : (fwd ? dense_yz_kernel<2, true> : dense_yz_kernel<2, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  kern<<<grid, 128, sm, st>>>(S, spec);
  return cudaGetLastError();
}



cudaError_t launch_tri_twist_table(int axis, const SpecPlan& S, double2* tab, cudaStream_t st) {
  const bool packed = S.kind[0] != 0;
  const int nlines = S.nxs * (axis == 1 ? S.nz : S.ny);
  const int grid = (nlines + 127) / 128;
  if (axis == 1) {
    if (packed) tri_twist_table_kernel<1, true><<<grid, 128, 0, st>>>(S, tab);
    else tri_twist_table_kernel<1, false><<<grid, 128, 0, st>>>(S, tab);
  } else {
    if (packed) tri_twist_table_kernel<2, true><<<grid, 128, 0, st>>>(S, tab);
    else tri_twist_table_kernel<2, false><<<grid, 128, 0, st>>>(S, tab);
  }
  return cudaGetLastError();
}

cudaError_t launch_tri_solve(int axis, const SpecPlan& S, double2* spec, cudaStream_t st) {
  const int N = axis == 1 ? S.ny : S.nz;
  const int n_other = axis == 1 ? S.nz : S.ny;
  const bool packed = S.kind[0] != 0;
  if (S.tri_tw && S.tri_m && S.sing_cm) {
    const int grid = (S.nxs * n_other + 63) / 64;
    if (axis == 1) {
      if (packed) tri_twist_solve_kernel<1, true><<<grid, 128, 0, st>>>(S, spec);
      else tri_twist_solve_kernel<1, false><<<grid, 128, 0, st>>>(S, spec);
    } else {
      if (packed) tri_twist_solve_kernel<2, true><<<grid, 128, 0, st>>>(S, spec);
      else tri_twist_solve_kernel<2, false><<<grid, 128, 0, st>>>(S, spec);
    }
    return cudaGetLastError();
  }
  const size_t sm = (size_t)N * TRI_T * sizeof(double) * (packed ? 2 : 1);
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  const int nreg = packed ? S.nxs : S.nxs - 1;
  const int nblk = (nreg + TRI_T - 1) / TRI_T;
  dim3 grid(nblk + (packed ? 0 : 1), n_other);
  auto kern = axis == 1 ? (packed ? tri_solve_kernel<1, true> : tri_solve_kernel<1, false>)
                        : (packed ? tri_solve_kernel<2, true> : tri_solve_kernel<2, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  kern<<<grid, TRI_T, sm, st>>>(S, spec);
  return cudaGetLastError();
}

}  // namespace ns
