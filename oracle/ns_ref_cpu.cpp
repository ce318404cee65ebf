// CPU restatement of the reference's periodic time step, C++17 + OpenMP
// (test infrastructure and the timed CPU baseline; never part of the product).
//
// THIS FILE IS TEST INFRASTRUCTURE.  Only tests/ and bench.py's CPU legs load
// the library built from it (oracle/libns_ref_cpu.so), as the checker or the
// timed baseline.  libns_gpu.so never calls it.
//
// It restates, loop by loop, the NumPy oracle (oracle/ns_oracle.py), which
// in turn restates the reference (zzwz02/NS_3D_Staggered_dp) step of
// big_periodic_3D.f90:326-567 on a triply periodic box:
//   cal_conv (NS_functions.f90:53-158) and cal_diff (:161-210) from the
//   two-point means and differences of FD_functions.f90:222-527;
//   the Euler / AB2 / AB2-CN predictor and history (big_periodic_3D.f90:350-423);
//   the CN-ADI sweeps as the reference runs them: dense mat_CN matrices
//   (NS_functions.f90:1245-1294) factored once with partial pivoting (getrf,
//   big_periodic_3D.f90:171-187) and applied to every line of a plane at once
//   (getrs with nrhs = the plane's lines, :425-489);
//   the FFT pressure Poisson solve (r2c 3D DFT, divide by the eigenvalues,
//   c2r with 1/N; :215-256, :498-548), the gauge and the correction (:562-567).
// Arrays are the reference's padded Fortran-order shapes.  Parallel loops use
// every OpenMP thread (OMP_NUM_THREADS).
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

namespace {

using cd = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;

// A Fortran-order 3D array (0-based indices).
struct A3 {
  double* d;
  int e0, e1, e2;
  double& operator()(int i, int j, int k) const { return d[i + (size_t)e0 * (j + (size_t)e1 * k)]; }
  size_t size() const { return (size_t)e0 * e1 * e2; }
};

// ---------------------------------------------------------------------------
// FFT: iterative radix-2 complex transform of one contiguous line.
// ---------------------------------------------------------------------------
struct Fft {
  int n = 0, lg = 0;
  std::vector<cd> tw;       // exp(-2 pi i m / n), m < n/2
  std::vector<int> rev;
  void init(int n_) {
    n = n_;
    lg = 0;
    while ((1 << lg) < n) ++lg;
    tw.resize(n / 2 > 0 ? n / 2 : 1);
    for (int m = 0; m < n / 2; ++m) tw[m] = std::polar(1.0, -2.0 * kPi * m / n);
    rev.resize(n);
    for (int i = 0; i < n; ++i) {
      int r = 0;
      for (int b = 0; b < lg; ++b) r |= ((i >> b) & 1) << (lg - 1 - b);
      rev[i] = r;
    }
  }
  // in place; inverse: conjugate twiddles, no scaling
  void run(cd* x, bool inverse) const {
    for (int i = 0; i < n; ++i)
      if (rev[i] > i) std::swap(x[i], x[rev[i]]);
    for (int len = 2; len <= n; len <<= 1) {
      const int half = len / 2, step = n / len;
      for (int s = 0; s < n; s += len)
        for (int q = 0; q < half; ++q) {
          const cd w = inverse ? std::conj(tw[q * step]) : tw[q * step];
          const cd a = x[s + q], b = w * x[s + q + half];
          x[s + q] = a + b;
          x[s + q + half] = a - b;
        }
    }
  }
};

// Periodic pressure Poisson solve of R (nx, ny, nz) into out (same shape):
// rfftn, divide by lambda (lambda(0) = +Inf), irfftn with 1/N.
struct Poisson {
  int nx, ny, nz, nxh;
  Fft fx2, fy, fz;               // nx/2-point (packed r2c), ny-, nz-point
  std::vector<cd> wr;            // r2c split twiddles exp(-2 pi i k / nx), k <= nx/2
  std::vector<double> eig;       // lambda per (kx, ky, kz)
  std::vector<cd> spec;          // (nxh, ny, nz)
  void init(int nx_, int ny_, int nz_, double dx, double dy, double dz) {
    nx = nx_; ny = ny_; nz = nz_; nxh = nx / 2 + 1;
    fx2.init(nx / 2); fy.init(ny); fz.init(nz);
    wr.resize(nxh);
    for (int k = 0; k < nxh; ++k) wr[k] = std::polar(1.0, -2.0 * kPi * k / nx);
    eig.resize((size_t)nxh * ny * nz);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nxh; ++i) {
          const double ex = std::pow(std::sin(kPi * i / nx) / dx, 2);
          const double ey = std::pow(std::sin(kPi * j / ny) / dy, 2);
          const double ez = std::pow(std::sin(kPi * k / nz) / dz, 2);
          eig[i + (size_t)nxh * (j + (size_t)ny * k)] = -4.0 * ((ex + ey) + ez);
        }
    spec.resize((size_t)nxh * ny * nz);
  }
  void solve(const double* R, double* out) {
    const int M = nx / 2;
    // x: r2c of every line through an M-point complex FFT of the packed samples
#pragma omp parallel
    {
      std::vector<cd> z(M);
#pragma omp for schedule(static)
      for (long long l = 0; l < (long long)ny * nz; ++l) {
        const double* x = R + (size_t)nx * l;
        for (int m = 0; m < M; ++m) z[m] = cd(x[2 * m], x[2 * m + 1]);
        fx2.run(z.data(), false);
        cd* o = spec.data() + (size_t)nxh * l;
        for (int k = 0; k <= M; ++k) {
          const cd zk = z[k % M], zm = std::conj(z[(M - k) % M]);
          const cd E = 0.5 * (zk + zm), O = cd(0.0, -0.5) * (zk - zm);
          o[k] = E + wr[k] * O;
        }
      }
    }
    // y and z: complex FFTs of the strided lines, divide, inverse
    auto pass = [&](int axis, bool inverse) {
      const int n = axis == 1 ? ny : nz;
      const Fft& F = axis == 1 ? fy : fz;
      const long long lines = axis == 1 ? (long long)nxh * nz : (long long)nxh * ny;
#pragma omp parallel
      {
        std::vector<cd> t(n);
#pragma omp for schedule(static)
        for (long long l = 0; l < lines; ++l) {
          const int i = (int)(l % nxh);
          const int o2 = (int)(l / nxh);
          const size_t base = axis == 1 ? i + (size_t)nxh * ny * o2 : i + (size_t)nxh * o2;
          const size_t st = axis == 1 ? (size_t)nxh : (size_t)nxh * ny;
          for (int e = 0; e < n; ++e) t[e] = spec[base + st * e];
          F.run(t.data(), inverse);
          for (int e = 0; e < n; ++e) spec[base + st * e] = t[e];
        }
      }
    };
    pass(1, false);
    pass(2, false);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)spec.size(); ++q) spec[q] = q == 0 ? cd(0.0, 0.0) : spec[q] / eig[q];
    pass(2, true);
    pass(1, true);
    // x: c2r, and the 1/N of the backward transform
    const double scale = 1.0 / ((double)nx * ny * nz);
#pragma omp parallel
    {
      std::vector<cd> z(M);
#pragma omp for schedule(static)
      for (long long l = 0; l < (long long)ny * nz; ++l) {
        const cd* X = spec.data() + (size_t)nxh * l;
        for (int k = 0; k < M; ++k) {
          const cd xk = X[k], xm = std::conj(X[M - k]);
          const cd E = xk + xm, O = (xk - xm) * std::conj(wr[k]);
          z[k] = E + cd(0.0, 1.0) * O;
        }
        fx2.run(z.data(), true);
        double* x = out + (size_t)nx * l;
        // z now holds nx * ny * nz times the packed samples (2 E, 2 O and the
        // unnormalised M-point inverse contribute 2 M = nx)
        for (int m = 0; m < M; ++m) {
          x[2 * m] = z[m].real() * scale;
          x[2 * m + 1] = z[m].imag() * scale;
        }
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Dense CN matrices and their LU (mat_CN, NS_functions.f90:1245-1294; getrf)
// ---------------------------------------------------------------------------
struct DenseLU {
  int m = 0;
  std::vector<double> a;  // row-major LU factors (unit lower L below the diagonal)
  std::vector<int> piv;   // row interchanged with row i at step i
  void factor(std::vector<double> A, int m_) {
    m = m_;
    piv.assign(m, 0);
    for (int c = 0; c < m; ++c) {
      int p = c;
      for (int r = c + 1; r < m; ++r)
        if (std::fabs(A[(size_t)r * m + c]) > std::fabs(A[(size_t)p * m + c])) p = r;
      piv[c] = p;
      if (p != c)
        for (int q = 0; q < m; ++q) std::swap(A[(size_t)c * m + q], A[(size_t)p * m + q]);
      const double d = A[(size_t)c * m + c];
      for (int r = c + 1; r < m; ++r) {
        const double l = A[(size_t)r * m + c] / d;
        A[(size_t)r * m + c] = l;
        if (l != 0.0)
          for (int q = c + 1; q < m; ++q) A[(size_t)r * m + q] -= l * A[(size_t)c * m + q];
      }
    }
    a = std::move(A);
  }
  // Solve for NB right-hand sides held row-major: X[e * NB + t].
  template <int NB>
  void solve(double* X) const {
    for (int i = 0; i < m; ++i)
      if (piv[i] != i)
        for (int t = 0; t < NB; ++t) std::swap(X[(size_t)i * NB + t], X[(size_t)piv[i] * NB + t]);
    // row i accumulates in registers over the rows above (below) it
    for (int i = 1; i < m; ++i) {
      double acc[NB];
      double* xi = X + (size_t)i * NB;
      for (int t = 0; t < NB; ++t) acc[t] = xi[t];
      const double* __restrict__ li = a.data() + (size_t)i * m;
      for (int l = 0; l < i; ++l) {
        const double c = li[l];
        const double* __restrict__ xl = X + (size_t)l * NB;
#pragma omp simd
        for (int t = 0; t < NB; ++t) acc[t] -= c * xl[t];
      }
      for (int t = 0; t < NB; ++t) xi[t] = acc[t];
    }
    for (int i = m - 1; i >= 0; --i) {
      double acc[NB];
      double* xi = X + (size_t)i * NB;
      for (int t = 0; t < NB; ++t) acc[t] = xi[t];
      const double* __restrict__ ui = a.data() + (size_t)i * m;
      for (int l = i + 1; l < m; ++l) {
        const double c = ui[l];
        const double* __restrict__ xl = X + (size_t)l * NB;
#pragma omp simd
        for (int t = 0; t < NB; ++t) acc[t] -= c * xl[t];
      }
      const double d = ui[i];
      for (int t = 0; t < NB; ++t) xi[t] = acc[t] / d;
    }
  }
};

// A (n+1, normal component) and B (n+2, tangential) of a periodic axis.
void mat_cn(int n, double dx2, double dt, double nu, std::vector<double>& A, std::vector<double>& B) {
  const double idx2 = 1.0 / dx2;
  const double dg = 1.0 + 0.5 * dt * nu * 2.0 * idx2;
  const double of = -0.5 * dt * nu * 1.0 * idx2;
  const int ma = n + 1, mb = n + 2;
  A.assign((size_t)ma * ma, 0.0);
  B.assign((size_t)mb * mb, 0.0);
  auto a = [&](int r, int c) -> double& { return A[(size_t)r * ma + c]; };
  auto b = [&](int r, int c) -> double& { return B[(size_t)r * mb + c]; };
  for (int i = 1; i < n; ++i) { a(i, i) = dg; a(i, i - 1) = of; a(i, i + 1) = of; }
  for (int i = 1; i <= n; ++i) { b(i, i) = dg; b(i, i - 1) = of; b(i, i + 1) = of; }
  a(0, 0) = dg; a(0, 1) = of; a(0, n) = of;   // the reference's row 1 closes on face n+1
  a(n, n) = 1.0; a(n, 0) = -1.0;
  b(0, 0) = 1.0; b(0, n) = -1.0;
  b(n + 1, n + 1) = 1.0; b(n + 1, 1) = -1.0;
}

constexpr int NB = 16;  // lines per block of the multi-line solves

// Solve every line of array X along axis ax with the LU of an m-unknown system.
void sweep(const A3& X, int ax, const DenseLU& lu) {
  const int m = lu.m;
  const int e[3] = {X.e0, X.e1, X.e2};
  // lines are indexed by the two other axes; blocks of NB lines run along the
  // fastest other axis (x for the y and z sweeps, y for the x sweep)
  const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
  const int n1 = e[o1], n2 = e[o2];
  const int nblk1 = (n1 + NB - 1) / NB;
#pragma omp parallel
  {
    std::vector<double> buf((size_t)m * NB);
#pragma omp for schedule(static)
    for (long long q = 0; q < (long long)nblk1 * n2; ++q) {
      const int b1 = (int)(q % nblk1), c2 = (int)(q / nblk1);
      const int t0 = b1 * NB, nt = std::min(NB, n1 - t0);
      auto at = [&](int el, int t) -> double& {
        int idx[3];
        idx[ax] = el; idx[o1] = t0 + t; idx[o2] = c2;
        return X(idx[0], idx[1], idx[2]);
      };
      for (int el = 0; el < m; ++el)
        for (int t = 0; t < NB; ++t) buf[(size_t)el * NB + t] = t < nt ? at(el, t) : 0.0;
      lu.solve<NB>(buf.data());
      for (int el = 0; el < m; ++el)
        for (int t = 0; t < nt; ++t) at(el, t) = buf[(size_t)el * NB + t];
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// The step
// ---------------------------------------------------------------------------
struct cpu_session {
  int nx, ny, nz, scheme, dp_flag, gauge;
  double dx, dy, dz, nu, dt;
  DenseLU lu[3][2];  // [axis][0 normal, 1 tangential]
  Poisson poisson;
  std::vector<double> cx, cy, cz, fx, fy, fz, us, vs, ws, R, dpi, dp;
};

extern "C" {

int cpu_threads(void) { return omp_get_max_threads(); }
// The host threads later steps use (n >= 1); returns the new count.
int cpu_set_threads(int n) {
  if (n >= 1) omp_set_num_threads(n);
  return omp_get_max_threads();
}

cpu_session* cpu_create(int nx, int ny, int nz, double lx, double ly, double lz, double nu, double dt, int scheme,
                        int dp_flag, int gauge) {
  auto pow2 = [](int n) { return n >= 4 && (n & (n - 1)) == 0; };
  if (!pow2(nx) || !pow2(ny) || !pow2(nz) || scheme < 0 || scheme > 2) return nullptr;
  cpu_session* s = new cpu_session();
  s->nx = nx; s->ny = ny; s->nz = nz; s->scheme = scheme; s->dp_flag = dp_flag; s->gauge = gauge;
  s->dx = lx / nx; s->dy = ly / ny; s->dz = lz / nz; s->nu = nu; s->dt = dt;
  const int n3[3] = {nx, ny, nz};
  const double h[3] = {s->dx, s->dy, s->dz};
  for (int a = 0; a < 3; ++a) {
    std::vector<double> A, B;
    mat_cn(n3[a], h[a] * h[a], dt, nu, A, B);
    s->lu[a][0].factor(A, n3[a] + 1);
    s->lu[a][1].factor(B, n3[a] + 2);
  }
  s->poisson.init(nx, ny, nz, s->dx, s->dy, s->dz);
  const size_t c = (size_t)nx * ny * nz;
  for (auto* v : {&s->cx, &s->cy, &s->cz, &s->fx, &s->fy, &s->fz, &s->R, &s->dpi}) v->assign(c, 0.0);
  s->us.assign((size_t)(nx + 1) * (ny + 2) * (nz + 2), 0.0);
  s->vs.assign((size_t)(nx + 2) * (ny + 1) * (nz + 2), 0.0);
  s->ws.assign((size_t)(nx + 2) * (ny + 2) * (nz + 1), 0.0);
  s->dp.assign((size_t)(nx + 2) * (ny + 2) * (nz + 2), 0.0);
  return s;
}

void cpu_destroy(cpu_session* s) { delete s; }

// One step in place on the reference arrays (history arrays in/out; zero
// outside their interior ranges on output).  first: the Euler start of
// AB2 / AB2-CN (big_periodic_3D.f90:377).
int cpu_step(cpu_session* s, double* up, double* vp, double* wp, double* pp, double* hxp, double* hyp, double* hzp,
             int first) {
  if (!s) return 1;
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double dx = s->dx, dy = s->dy, dz = s->dz, nu = s->nu, dt = s->dt;
  const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
  const double dpf = s->dp_flag;
  A3 u{up, nx + 1, ny + 2, nz + 2}, v{vp, nx + 2, ny + 1, nz + 2}, w{wp, nx + 2, ny + 2, nz + 1};
  A3 p{pp, nx + 2, ny + 2, nz + 2};
  A3 hx{hxp, nx + 1, ny + 2, nz + 2}, hy{hyp, nx + 2, ny + 1, nz + 2}, hz{hzp, nx + 2, ny + 2, nz + 1};
  A3 cx{s->cx.data(), nx, ny, nz}, cy{s->cy.data(), nx, ny, nz}, cz{s->cz.data(), nx, ny, nz};
  A3 fx{s->fx.data(), nx, ny, nz}, fy{s->fy.data(), nx, ny, nz}, fz{s->fz.data(), nx, ny, nz};
  A3 us{s->us.data(), nx + 1, ny + 2, nz + 2}, vs{s->vs.data(), nx + 2, ny + 1, nz + 2};
  A3 ws{s->ws.data(), nx + 2, ny + 2, nz + 1}, dp{s->dp.data(), nx + 2, ny + 2, nz + 2};
  // two-point means of FD_functions.f90 avg (bc 1: periodic wrap of the first entry)
  auto ux = [&](int a, int J, int K) { return a == 0 ? (u(nx, J, K) + u(nx - 1, J, K)) / 2.0 : (u(a, J, K) + u(a - 1, J, K)) / 2.0; };
  auto uy = [&](int a, int b, int K) { return (u(a, b + 1, K) + u(a, b, K)) / 2.0; };
  auto uz = [&](int a, int J, int c) { return (u(a, J, c + 1) + u(a, J, c)) / 2.0; };
  auto vx = [&](int a, int b, int K) { return (v(a + 1, b, K) + v(a, b, K)) / 2.0; };
  auto vy = [&](int I, int b, int K) { return b == 0 ? (v(I, ny, K) + v(I, ny - 1, K)) / 2.0 : (v(I, b, K) + v(I, b - 1, K)) / 2.0; };
  auto vz = [&](int I, int b, int c) { return (v(I, b, c + 1) + v(I, b, c)) / 2.0; };
  auto wx = [&](int a, int J, int c) { return (w(a + 1, J, c) + w(a, J, c)) / 2.0; };
  auto wy = [&](int I, int b, int c) { return (w(I, b + 1, c) + w(I, b, c)) / 2.0; };
  auto wz = [&](int I, int J, int c) { return c == 0 ? (w(I, J, nz) + w(I, J, nz - 1)) / 2.0 : (w(I, J, c) + w(I, J, c - 1)) / 2.0; };
  // cal_conv and cal_diff at the interior outputs
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int I = i + 1, J = j + 1, K = k + 1;
        double t;
        {  // conv_x
          const double a1 = ux(i + 1, J, K), a0 = ux(i, J, K);
          t = (a1 * a1 - a0 * a0) / dx;
          t = t + (uy(i, j + 1, K) * vx(i, j + 1, K) - uy(i, j, K) * vx(i, j, K)) / dy;
          t = t + (uz(i, J, k + 1) * wx(i, J, k + 1) - uz(i, J, k) * wx(i, J, k)) / dz;
          cx(i, j, k) = t;
        }
        {  // conv_y
          t = (vx(i + 1, j, K) * uy(i + 1, j, K) - vx(i, j, K) * uy(i, j, K)) / dx;
          const double b1 = vy(I, j + 1, K), b0 = vy(I, j, K);
          t = t + (b1 * b1 - b0 * b0) / dy;
          t = t + (vz(I, j, k + 1) * wy(I, j, k + 1) - vz(I, j, k) * wy(I, j, k)) / dz;
          cy(i, j, k) = t;
        }
        {  // conv_z
          t = (wx(i + 1, J, k) * uz(i + 1, J, k) - wx(i, J, k) * uz(i, J, k)) / dx;
          t = t + (wy(I, j + 1, k) * vz(I, j + 1, k) - wy(I, j, k) * vz(I, j, k)) / dy;
          const double c1 = wz(I, J, k + 1), c0 = wz(I, J, k);
          t = t + (c1 * c1 - c0 * c0) / dz;
          cz(i, j, k) = t;
        }
        {  // diff_x: periodic diff2 along x of u(:, J, K), plain along y and z
          const double xm = i == 0 ? u(nx - 1, J, K) : u(i - 1, J, K);
          t = (xm - 2.0 * u(i, J, K) + u(i + 1, J, K)) / dx2;
          t = t + (u(i, j, K) - 2.0 * u(i, j + 1, K) + u(i, j + 2, K)) / dy2;
          t = t + (u(i, J, k) - 2.0 * u(i, J, k + 1) + u(i, J, k + 2)) / dz2;
          fx(i, j, k) = t;
        }
        {  // diff_y
          t = (v(i, j, K) - 2.0 * v(i + 1, j, K) + v(i + 2, j, K)) / dx2;
          const double ym = j == 0 ? v(I, ny - 1, K) : v(I, j - 1, K);
          t = t + (ym - 2.0 * v(I, j, K) + v(I, j + 1, K)) / dy2;
          t = t + (v(I, j, k) - 2.0 * v(I, j, k + 1) + v(I, j, k + 2)) / dz2;
          fy(i, j, k) = t;
        }
        {  // diff_z
          t = (w(i, J, k) - 2.0 * w(i + 1, J, k) + w(i + 2, J, k)) / dx2;
          t = t + (w(I, j, k) - 2.0 * w(I, j + 1, k) + w(I, j + 2, k)) / dy2;
          const double zm = k == 0 ? w(I, J, nz - 1) : w(I, J, k - 1);
          t = t + (zm - 2.0 * w(I, J, k) + w(I, J, k + 1)) / dz2;
          fz(i, j, k) = t;
        }
      }
  // predictor over the full arrays and the AB2 history (big_periodic_3D.f90:350-423)
  const int sch = s->scheme;
  auto predict = [&](const A3& F, const A3& FS, const A3& H, const A3& C, const A3& D, int ax) {
    const int e[3] = {F.e0, F.e1, F.e2};
#pragma omp parallel for collapse(2) schedule(static)
    for (int c = 0; c < e[2]; ++c)
      for (int b = 0; b < e[1]; ++b)
        for (int a = 0; a < e[0]; ++a) {
          // interior range X of this component: own axis 0..n-1, others 1..n
          const int idx[3] = {a, b, c};
          const int nn[3] = {nx, ny, nz};
          bool in = true;
          int ci[3];
          for (int q = 0; q < 3; ++q) {
            const int lo = q == ax ? 0 : 1;
            in = in && idx[q] >= lo && idx[q] < lo + nn[q];
            ci[q] = idx[q] - lo;
          }
          double rx = 0.0;
          if (in) {
            const double cc = C(ci[0], ci[1], ci[2]), ff = D(ci[0], ci[1], ci[2]);
            if (sch == 2) rx = first ? 0.5 * nu * ff - cc : 0.5 * nu * ff - 1.5 * cc;
            else rx = nu * ff - cc;
          }
          int pi[3] = {a, b, c};
          pi[ax] += 1;
          const double dpd = (p(pi[0], pi[1], pi[2]) - p(a, b, c)) / (ax == 0 ? dx : (ax == 1 ? dy : dz));
          const double px = H(a, b, c);
          double r;
          if (sch == 0) r = dt * (1.0 * rx - dpf * dpd) + F(a, b, c);
          else if (sch == 1) r = first ? dt * (1.0 * rx - dpf * dpd) + F(a, b, c)
                                       : dt * (1.5 * rx - 0.5 * px - dpf * dpd) + F(a, b, c);
          else r = first ? dt * (rx - dpf * dpd) + F(a, b, c) : dt * (rx - 0.5 * px - dpf * dpd) + F(a, b, c);
          FS(a, b, c) = r;
          // history: Euler 0, AB2 rhs, AB2-CN -conv; zero outside the interior range
          double hn = 0.0;
          if (in) hn = sch == 0 ? 0.0 : (sch == 1 ? rx : -C(ci[0], ci[1], ci[2]));
          H(a, b, c) = hn;
        }
  };
  predict(u, us, hx, cx, fx, 0);
  predict(v, vs, hy, cy, fy, 1);
  predict(w, ws, hz, cz, fz, 2);
  if (sch == 2) {
    // CN-ADI: the periodic BC rows are zero (vel_bc_staggered_CN2), then the sweeps
    auto zero = [&](const A3& X, int ax, int idx) {
      const int e[3] = {X.e0, X.e1, X.e2};
      const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
#pragma omp parallel for schedule(static)
      for (int c = 0; c < e[o2]; ++c)
        for (int b = 0; b < e[o1]; ++b) {
          int q[3];
          q[ax] = idx; q[o1] = b; q[o2] = c;
          X(q[0], q[1], q[2]) = 0.0;
        }
    };
    for (int ax = 0; ax < 3; ++ax) {
      const A3* F[3] = {&us, &vs, &ws};
      for (int f = 0; f < 3; ++f) {
        const int e = ax == 0 ? F[f]->e0 : (ax == 1 ? F[f]->e1 : F[f]->e2);
        if (f == ax) zero(*F[f], ax, e - 1);             // the duplicate face row
        else { zero(*F[f], ax, 0); zero(*F[f], ax, e - 1); }  // the two ghost rows
      }
      for (int f = 0; f < 3; ++f) sweep(*F[f], ax, s->lu[ax][f == ax ? 0 : 1]);
    }
  } else {
    // vel_bc_staggered, periodic copies (NS_functions.f90:213-310)
    auto copy_plane = [&](const A3& X, int ax, int dst, int src) {
      const int e[3] = {X.e0, X.e1, X.e2};
      const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
#pragma omp parallel for schedule(static)
      for (int c = 0; c < e[o2]; ++c)
        for (int b = 0; b < e[o1]; ++b) {
          int qd[3], qs[3];
          qd[ax] = dst; qs[ax] = src; qd[o1] = qs[o1] = b; qd[o2] = qs[o2] = c;
          X(qd[0], qd[1], qd[2]) = X(qs[0], qs[1], qs[2]);
        }
    };
    const A3* F[3] = {&us, &vs, &ws};
    const int n3[3] = {nx, ny, nz};
    for (int ax = 0; ax < 3; ++ax)
      for (int f = 0; f < 3; ++f) {
        if (f == ax) copy_plane(*F[f], ax, n3[ax], 0);   // face n+1 <- face 1
        else { copy_plane(*F[f], ax, 0, n3[ax]); copy_plane(*F[f], ax, n3[ax] + 1, 1); }
      }
  }
  // divergence right-hand side, FFT Poisson solve, pr_bc_staggered, gauge, correction
  A3 R{s->R.data(), nx, ny, nz};
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int I = i + 1, J = j + 1, K = k + 1;
        double r = (us(i + 1, J, K) - us(i, J, K)) / dx;
        r = r + (vs(I, j + 1, K) - vs(I, j, K)) / dy;
        r = r + (ws(I, J, k + 1) - ws(I, J, k)) / dz;
        R(i, j, k) = r / dt;
      }
  s->poisson.solve(s->R.data(), s->dpi.data());
  A3 dpi{s->dpi.data(), nx, ny, nz};
  std::fill(s->dp.begin(), s->dp.end(), 0.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) dp(i + 1, j + 1, k + 1) = dpi(i, j, k);
  for (int ax = 0; ax < 3; ++ax) {
    const int e[3] = {dp.e0, dp.e1, dp.e2};
    const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
    const int n = e[ax] - 2;
    for (int c = 0; c < e[o2]; ++c)
      for (int b = 0; b < e[o1]; ++b) {
        int q0[3], qn[3], q1[3], qe[3];
        q0[ax] = 0; qn[ax] = n; q1[ax] = 1; qe[ax] = n + 1;
        q0[o1] = qn[o1] = q1[o1] = qe[o1] = b;
        q0[o2] = qn[o2] = q1[o2] = qe[o2] = c;
        dp(q0[0], q0[1], q0[2]) = dp(qn[0], qn[1], qn[2]);
        dp(qe[0], qe[1], qe[2]) = dp(q1[0], q1[1], q1[2]);
      }
  }
  if (s->gauge) {
    const double g0 = dp(0, 0, 0);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)dp.size(); ++q) dp.d[q] = dp.d[q] - g0;
  }
  auto correct = [&](const A3& F, const A3& FS, int ax, double h) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int c = 0; c < F.e2; ++c)
      for (int b = 0; b < F.e1; ++b)
        for (int a = 0; a < F.e0; ++a) {
          int q[3] = {a, b, c};
          q[ax] += 1;
          F(a, b, c) = -dt * (dp(q[0], q[1], q[2]) - dp(a, b, c)) / h + FS(a, b, c);
        }
  };
  correct(u, us, 0, dx);
  correct(v, vs, 1, dy);
  correct(w, ws, 2, dz);
#pragma omp parallel for schedule(static)
  for (long long q = 0; q < (long long)p.size(); ++q) p.d[q] = dpf * p.d[q] + dp.d[q];
  return 0;
}

}  // extern "C"
