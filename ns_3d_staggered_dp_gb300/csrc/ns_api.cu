// C ABI of libns_gpu.so: sessions, state transfer, boundary faces, the time
// step and the routine tier.  See include/ns_gpu.h for the contract and the
// reference routine each entry point replaces.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"
#include "ns_session.cuh"

using namespace ns;

namespace {

// LU factors (no pivoting) of tridiag(a, b, c), a[0] and c[m-1] unused.
void thomas_factor(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& c,
                   HostLineSys& S) {
  const int m = (int)b.size();
  S.l.assign(m, 0.0); S.dinv.assign(m, 0.0); S.cu.assign(m, 0.0);
  double d = b[0];
  S.dinv[0] = 1.0 / d;
  S.cu[0] = m > 1 ? c[0] / d : 0.0;
  for (int i = 1; i < m; ++i) {
    S.l[i] = a[i] / d;
    d = b[i] - S.l[i] * c[i - 1];
    S.dinv[i] = 1.0 / d;
    S.cu[i] = (i + 1 < m) ? c[i] / d : 0.0;
  }
}

std::vector<double> thomas_solve(const HostLineSys& S, std::vector<double> r) {
  const int m = (int)r.size();
  for (int i = 1; i < m; ++i) r[i] -= S.l[i] * r[i - 1];
  r[m - 1] *= S.dinv[m - 1];
  for (int i = m - 2; i >= 0; --i) r[i] = r[i] * S.dinv[i] - S.cu[i] * r[i + 1];
  return r;
}

}  // namespace

namespace ns {
// CN system of one sweep axis (mat_CN, NS_functions.f90:1245-1294).
// normal: the swept field is staggered along the axis (A matrix, n+1
// unknowns); otherwise tangential (B matrix, n+2 unknowns).
// transposed (periodic only): the system M^T of the adjoint sweep, whose
// corner entries are those of M exchanged.
HostLineSys build_cn_system(int n, int bc, double h, double dt, double nu, bool normal, int closure,
                            bool transposed) {
  const double idx2 = 1.0 / (h * h);
  const double dg = 1.0 + 0.5 * dt * nu * 2.0 * idx2;
  const double of = -0.5 * dt * nu * 1.0 * idx2;
  HostLineSys S;
  S.n = n;
  if (bc == 1) {
    // Reduced cyclic system on slots 1..n.
    std::vector<double> a(n, of), b(n, dg), c(n, of);
    double tr = of, bl = of;  // M[0][n-1], M[n-1][0]
    if (normal && closure == 0) {
      // A(1,n+1) ties face 1 to the duplicate face n+1 = face 1 (reference closure)
      b[0] = dg + of;
      tr = 0.0;
    }
    if (transposed) std::swap(tr, bl);
    const double gam = -b[0];
    b[0] -= gam;
    b[n - 1] -= tr * bl / gam;
    HostLineSys T;
    thomas_factor(a, b, c, T);
    std::vector<double> u(n, 0.0);
    u[0] = gam;
    u[n - 1] += bl;
    std::vector<double> z = thomas_solve(T, u);
    const double vlast = tr / gam;
    const double fac = 1.0 + z[0] + vlast * z[n - 1];
    S.l = T.l; S.dinv = T.dinv; S.cu = T.cu; S.z = z;
    S.s0 = 1.0 / fac;
    S.s1 = vlast / fac;
    double zmax = 0;
    for (double q : z) zmax = std::fmax(zmax, std::fabs(q));
    const double thr = 1e-18 * zmax;
    int zA = 0, zB = n;
    for (int i = 0; i < n / 2; ++i)
      if (std::fabs(z[i]) >= thr) zA = i + 1;
    for (int i = n - 1; i >= n / 2; --i)
      if (std::fabs(z[i]) >= thr) zB = i;
    S.zA = zA; S.zB = zB;
    S.lo = 1; S.hi = n; S.periodic = 1;
    return S;
  }
  const int m = normal ? n + 1 : n + 2;
  std::vector<double> a(m, of), b(m, dg), c(m, of);
  if (normal) {  // rows 1 and n+1: identity (bc 2 and 4)
    b[0] = 1.0; c[0] = 0.0;
    b[m - 1] = 1.0; a[m - 1] = 0.0;
    S.lo = 1; S.hi = n + 1;
  } else {
    if (bc == 2) {
      b[0] = 0.5; c[0] = 0.5;
      b[m - 1] = 0.5; a[m - 1] = 0.5;
    } else {
      b[0] = 1.0; c[0] = 0.0;
      b[m - 1] = 1.0; a[m - 1] = 0.0;
    }
    S.lo = 0; S.hi = n + 1;
  }
  a[0] = 0.0; c[m - 1] = 0.0;
  thomas_factor(a, b, c, S);
  S.periodic = 0;
  S.z.assign(1, 0.0);
  return S;
}
}  // namespace ns

namespace ns {

// Dense transform pair of one non-periodic axis of n cells, from the MKL
// trigonometric transforms DCT_poisson_solver applies (NS_functions.f90:1526-1625):
//   pbc 3: F = backward staggered cosine (DCT-II / 2), G = forward staggered cosine
//   pbc 2: sign flip of the odd (1-based) inputs, pbc-3 transform, reversal (and back)
//   pbc 4: F = DST-I / 2 on n points, G = DST-I / (n + 1)
// F[k][n'] (mode k from sample n'), G[n'][k] = F^-1, angles in long double.
void dense_pair(int n, int pb, std::vector<double>& F, std::vector<double>& G) {
  const long double pi = 3.141592653589793238462643383279502884L;
  F.assign((size_t)n * n, 0.0);
  G.assign((size_t)n * n, 0.0);
  auto cosq = [&](long long m, long long q) {  // cos(pi m / q), m reduced mod 2q
    m %= 2 * q;
    return cosl(pi * (long double)m / (long double)q);
  };
  auto sinq = [&](long long m, long long q) {
    m %= 2 * q;
    return sinl(pi * (long double)m / (long double)q);
  };
  for (int k = 0; k < n; ++k)
    for (int s = 0; s < n; ++s) {
      long double f, g;
      if (pb == 3 || pb == 2) {
        const int kk = (pb == 2) ? n - 1 - k : k;  // reversal of the modes
        const long double sg = (pb == 2 && s % 2 == 0) ? -1.0L : 1.0L;  // odd 1-based samples flipped
        const long double cs = cosq((long long)kk * (2 * s + 1), 2LL * n);
        f = sg * cs;
        g = sg * cs * (kk == 0 ? 1.0L : 2.0L) / (long double)n;
      } else {
        const long double sn = sinq((long long)(k + 1) * (s + 1), n + 1);
        f = sn;
        g = 2.0L * sn / (long double)(n + 1);
      }
      F[(size_t)k * n + s] = (double)f;
      G[(size_t)s * n + k] = (double)g;
    }
}

// Eigenvalue sin^2(..)/h^2 of mode m (0-based) of one axis: FFT bins for pbc 1
// (big_periodic_3D.f90:242-255), the trigonometric-transform modes otherwise
// (re_simulation_sub_tstep_interBC_combine.f90:320-353).
double axis_eig(int n, int pb, int m, double h) {
  const double pi = 3.1415926535897932;
  double s;
  if (pb == 1) s = std::sin(pi * m / n);
  else if (pb == 2) s = std::sin((m + 1) * pi / 2 / n);
  else if (pb == 3) s = std::sin(m * pi / 2 / n);
  else s = std::sin((m + 1) * pi / 2 / (n + 1));
  return s * s / (h * h);
}

}  // namespace ns

namespace {

int fail(ns_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define NS_CUDA(h, call)                                                                     \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail((h), NS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

// Internal slot offset per field and axis: face axis -> 0, cell axis -> -1.
// field 0 u (face x), 1 v (face y), 2 w (face z), 3 p (cells).
inline int slot_off(int field, int axis) { return (field == axis) ? 0 : -1; }
// Reference extent of a field along an axis.
inline int ext_of(const ns_config& c, int field, int axis) {
  const int n = axis == 0 ? c.nx : (axis == 1 ? c.ny : c.nz);
  return (field == axis) ? n + 1 : n + 2;
}

// Host <-> device field transfers.  A reference-shaped array moves as ONE
// flat copy between host memory and a device staging buffer (full link
// bandwidth; a pitched 3D copy issues one DMA per 2 KB row), and a kernel
// scatters it into, or gathers it from, the padded slot layout.  On the way
// out, entries outside [lo, hi] per axis (0-based reference indices) can be
// written as zero (the history outside its interior ranges).
struct PackArgs {
  Layout L;
  double* field;
  double* stage;
  int ex, ey, ez;   // reference extents
  int ox, oy, oz;   // slot of reference index 0 per axis
  int to_field;     // 1: stage -> field, 0: field -> stage
  int lo[3], hi[3]; // kept range on the way out (others zero)
  int z_lo, z_hi;   // reference planes [z_lo, z_hi) moved
};

// IDX: the index type of the flat reference index (32-bit divisions where
// the moved planes hold fewer than 2^32 entries; 64-bit emulated ones cost
// more than the copy itself).
template <typename IDX>
__global__ void __launch_bounds__(256) field_pack_kernel(PackArgs a) {
  const IDX ex = (IDX)a.ex, ey = (IDX)a.ey;
  const IDX n = ex * ey * (IDX)(a.z_hi - a.z_lo);
  const long long base = (long long)a.ex * a.ey * a.z_lo;  // flat index of the first moved entry
  for (IDX q = blockIdx.x * (IDX)blockDim.x + threadIdx.x; q < n; q += (IDX)gridDim.x * blockDim.x) {
    const IDX r = q / ex;
    const int i = (int)(q - r * ex);
    const IDX kk = r / ey;
    const int j = (int)(r - kk * ey);
    const int k = a.z_lo + (int)kk;
    const long long t = base + (long long)q;
    const long long g = a.L.at(a.ox + i, a.oy + j, a.oz + k);
    if (a.to_field) {
      a.field[g] = a.stage[t];
    } else {
      const bool keep = i >= a.lo[0] && i <= a.hi[0] && j >= a.lo[1] && j <= a.hi[1] && k >= a.lo[2] && k <= a.hi[2];
      a.stage[t] = keep ? a.field[g] : 0.0;
    }
  }
}

// The extra face slot 0 of u along x and of v along y (periodic axes) on
// z slots [z0, z1): the slab-wise part of launch_extra_slots.
__global__ void __launch_bounds__(256) extra_xy_kernel(Layout L, double* u, double* v, int perx, int pery, int z0,
                                                       int z1) {
  const int nyp = L.ny + 2, nxp = L.nx + 2, per = nyp + nxp;
  const long long n = (long long)(z1 - z0) * per;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int k = z0 + (int)(t / per);
    const int r = (int)(t % per);
    if (r < nyp) {
      if (perx) u[L.at(0, r, k)] = u[L.at(L.nx, r, k)];
    } else if (pery) {
      const int i = r - nyp;
      v[L.at(i, 0, k)] = v[L.at(i, L.ny, k)];
    }
  }
}

cudaError_t ensure_stage(ns_handle* h) {
  if (h->stage) return cudaSuccess;
  const size_t n = (size_t)(h->cfg.nx + 2) * (h->cfg.ny + 2) * (h->cfg.nz + 2);
  return cudaMalloc(&h->stage, n * sizeof(double));
}

// The second staging buffer, the copy stream and its events (multi-field transfers).
cudaError_t ensure_xfer(ns_handle* h) {
  cudaError_t e = ensure_stage(h);
  if (e != cudaSuccess || h->stage2) return e;
  const size_t n = (size_t)(h->cfg.nx + 2) * (h->cfg.ny + 2) * (h->cfg.nz + 2);
  if ((e = cudaMalloc(&h->stage2, n * sizeof(double))) != cudaSuccess) return e;
  if ((e = cudaStreamCreateWithFlags(&h->xfer, cudaStreamNonBlocking)) != cudaSuccess) return e;
  int least = 0, greatest = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess) return e;
  (void)least;
  if ((e = cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
  if ((e = cudaStreamCreateWithPriority(&h->prio, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
  if ((e = cudaStreamCreateWithPriority(&h->scat, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
  for (int b = 0; b < 2; ++b) {
    if ((e = cudaEventCreateWithFlags(&h->ev_full[b], cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&h->ev_free[b], cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&h->ev_aux[b], cudaEventDisableTiming)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The history's interior ranges (0-based reference indices) of field f:
// entries outside them are returned as zero.
void hist_range(const ns_config& c, int f, int lo[3], int hi[3]) {
  for (int ax = 0; ax < 3; ++ax) {
    const int na = ax == 0 ? c.nx : (ax == 1 ? c.ny : c.nz);
    if (ax == f) { lo[ax] = c.bc[ax] == 1 ? 0 : 1; hi[ax] = na - 1; }
    else { lo[ax] = 1; hi[ax] = na; }
  }
}



cudaError_t pack_launch(ns_handle* h, double* field, double* stage, int f, bool to_field, const int* lo = nullptr,
                        const int* hi = nullptr, cudaStream_t stream = nullptr, int z_lo = 0, int z_hi = -1) {
  const ns_config& c = h->cfg;
  PackArgs a{};
  a.L = h->L;
  a.field = field;
  a.stage = stage;
  a.ex = ext_of(c, f, 0); a.ey = ext_of(c, f, 1); a.ez = ext_of(c, f, 2);
  a.ox = 1 + slot_off(f, 0); a.oy = 1 + slot_off(f, 1); a.oz = 1 + slot_off(f, 2);
  a.to_field = to_field ? 1 : 0;
  const int ext[3] = {a.ex, a.ey, a.ez};
  for (int q = 0; q < 3; ++q) {
    a.lo[q] = lo ? lo[q] : 0;
    a.hi[q] = hi ? hi[q] : ext[q] - 1;
  }
  a.z_lo = z_lo;
  a.z_hi = z_hi < 0 ? a.ez : z_hi;
  if (a.z_hi <= a.z_lo) return cudaSuccess;
  const long long n = (long long)a.ex * a.ey * (a.z_hi - a.z_lo);
  const int grid = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  if (n + (long long)grid * 256 < (1LL << 32))
    field_pack_kernel<unsigned><<<grid, 256, 0, stream ? stream : h->stream>>>(a);
  else
    field_pack_kernel<unsigned long long><<<grid, 256, 0, stream ? stream : h->stream>>>(a);
  return cudaGetLastError();
}

inline size_t field_bytes(const ns_config& c, int f) {
  return sizeof(double) * ext_of(c, f, 0) * ext_of(c, f, 1) * ext_of(c, f, 2);
}

// n fields in: copies on the copy stream, scatters on the handle's stream,
// two staging buffers in turn so the copy of one field overlaps the scatter
// of the previous one.
cudaError_t h2d_fields(ns_handle* h, int n, double* const* dst, const double* const* src, const int* fid) {
  cudaError_t e = ensure_xfer(h);
  if (e != cudaSuccess) return e;
  double* buf[2] = {h->stage, h->stage2};
  for (int b = 0; b < 2; ++b)
    if ((e = cudaEventRecord(h->ev_free[b], h->stream)) != cudaSuccess) return e;
  for (int q = 0; q < n; ++q) {
    const int b = q & 1;
    if ((e = cudaStreamWaitEvent(h->xfer, h->ev_free[b], 0)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(buf[b], src[q], field_bytes(h->cfg, fid[q]), cudaMemcpyHostToDevice, h->xfer)) !=
        cudaSuccess)
      return e;
    if ((e = cudaEventRecord(h->ev_full[b], h->xfer)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(h->stream, h->ev_full[b], 0)) != cudaSuccess) return e;
    if ((e = pack_launch(h, dst[q], buf[b], fid[q], true)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(h->ev_free[b], h->stream)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// n fields out: gathers on the handle's stream, copies on the copy stream;
// returns after the last copy has landed.  zero_hist[q]: zero the entries
// outside the history's interior ranges.
cudaError_t d2h_fields(ns_handle* h, int n, double* const* dst, const double* const* src, const int* fid,
                       const bool* zero_hist) {
  cudaError_t e = ensure_xfer(h);
  if (e != cudaSuccess) return e;
  const ns_config& c = h->cfg;
  double* buf[2] = {h->stage, h->stage2};
  for (int b = 0; b < 2; ++b)
    if ((e = cudaEventRecord(h->ev_free[b], h->xfer)) != cudaSuccess) return e;
  for (int q = 0; q < n; ++q) {
    const int b = q & 1, f = fid[q];
    if ((e = cudaStreamWaitEvent(h->stream, h->ev_free[b], 0)) != cudaSuccess) return e;
    int lo[3], hi[3];
    hist_range(c, f, lo, hi);
    const bool z = zero_hist && zero_hist[q];
    if ((e = pack_launch(h, const_cast<double*>(src[q]), buf[b], f, false, z ? lo : nullptr, z ? hi : nullptr)) !=
        cudaSuccess)
      return e;
    if ((e = cudaEventRecord(h->ev_full[b], h->stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(h->xfer, h->ev_full[b], 0)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(dst[q], buf[b], field_bytes(c, f), cudaMemcpyDeviceToHost, h->xfer)) != cudaSuccess)
      return e;
    if ((e = cudaEventRecord(h->ev_free[b], h->xfer)) != cudaSuccess) return e;
  }
  return cudaStreamSynchronize(h->xfer);
}

// Copy a Fortran array (reference shape) into the padded device field.
cudaError_t h2d_field(ns_handle* h, double* dst, const double* src, int field) {
  const ns_config& c = h->cfg;
  const size_t bytes = sizeof(double) * ext_of(c, field, 0) * ext_of(c, field, 1) * ext_of(c, field, 2);
  cudaError_t e = ensure_stage(h);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(h->stage, src, bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess) return e;
  return pack_launch(h, dst, h->stage, field, true);
}

cudaError_t d2h_field(ns_handle* h, double* dst, const double* src, int field) {
  const ns_config& c = h->cfg;
  const size_t bytes = sizeof(double) * ext_of(c, field, 0) * ext_of(c, field, 1) * ext_of(c, field, 2);
  cudaError_t e = ensure_stage(h);
  if (e != cudaSuccess) return e;
  if ((e = pack_launch(h, const_cast<double*>(src), h->stage, field, false)) != cudaSuccess) return e;
  return cudaMemcpyAsync(dst, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream);
}

// Plane size of face planes for an axis (full box extent of the two other axes).
inline int plane_n1(const Layout& L, int axis) { return axis == 0 ? L.ny + 2 : L.nx + 2; }
inline int plane_n2(const Layout& L, int axis) { return axis == 2 ? L.ny + 2 : L.nz + 2; }
inline size_t plane_size(const Layout& L, int axis) { return (size_t)plane_n1(L, axis) * plane_n2(L, axis); }

// Offsets of a face plane inside face_buf.
size_t face_offset(const Layout& L, int set, int axis, int field, int side) {
  size_t off = 0;
  for (int s = 0; s < 4; ++s)
    for (int a = 0; a < 3; ++a)
      for (int f = 0; f < 4; ++f)
        for (int d = 0; d < 2; ++d) {
          if (s == set && a == axis && f == field && d == side) return off;
          off += plane_size(L, a);
        }
  return off;
}
size_t face_total(const Layout& L) {
  size_t t = 0;
  for (int a = 0; a < 3; ++a) t += 4 * 8 * plane_size(L, a);
  return t;
}

// Convert one reference face array (2D, Fortran order over the two other
// axes of the field) into a device plane in internal slot order.
void face_to_plane(const ns_config& c, const Layout& L, int axis, int field, const double* src, double* plane) {
  const int a1 = axis == 0 ? 1 : 0;
  const int a2 = axis == 2 ? 1 : 2;
  const int e1 = ext_of(c, field, a1), e2 = ext_of(c, field, a2);
  const int o1 = 1 + slot_off(field, a1), o2 = 1 + slot_off(field, a2);
  const int n1 = plane_n1(L, axis);
  for (int q = 0; q < e2; ++q)
    for (int r = 0; r < e1; ++r) plane[(size_t)(r + o1) + (size_t)n1 * (q + o2)] = src[r + (size_t)e1 * q];
}

int validate(const ns_config& c, std::string& msg) {
  if (c.nx < 4 || c.ny < 4 || c.nz < 4) { msg = "grid too small"; return NS_ERR_SHAPE; }
  if (c.scheme < 0 || c.scheme > 2) { msg = "scheme must be 0 (Euler), 1 (AB2) or 2 (AB2-CN)"; return NS_ERR_ARG; }
  if (c.poisson_z != 0 && c.poisson_z != 1) { msg = "poisson_z must be 0 (cyclic line solves) or 1 (z FFT)"; return NS_ERR_ARG; }
  if (c.keep_sweeps != 0 && c.keep_sweeps != 1) { msg = "keep_sweeps must be 0 or 1"; return NS_ERR_ARG; }
  for (int a = 0; a < 3; ++a) {
    if (c.bc[a] != 1 && c.bc[a] != 2 && c.bc[a] != 4) {
      msg = "velocity bc must be 1, 2 or 4 (3 leaves the ghosts undefined in the reference)";
      return NS_ERR_UNSUPPORTED_BC;
    }
    if (c.pbc[a] < 1 || c.pbc[a] > 4) { msg = "pbc must be 1..4"; return NS_ERR_UNSUPPORTED_BC; }
    if ((c.bc[a] == 1) != (c.pbc[a] == 1)) { msg = "bc and pbc must agree on periodicity"; return NS_ERR_UNSUPPORTED_BC; }
  }
  // Poisson: FFT on periodic axes, dense trigonometric transforms on the others.
  if (c.pbc[0] != 1 && (c.pbc[1] == 1 || c.pbc[2] == 1)) {
    msg = "a non-periodic x pressure axis needs non-periodic y and z as well";
    return NS_ERR_UNSUPPORTED_BC;
  }
  auto pow2 = [](int n) { return n == 16 || n == 32 || n == 64 || n == 128 || n == 256 || n == 512; };
  const int n3[3] = {c.nx, c.ny, c.nz};
  // Wall axes: a wall z (else a wall y) is solved line by line (tridiagonal),
  // a wall y in front of a wall z and a wall x are dense transforms.
  const int sax = c.pbc[2] != 1 ? 2 : (c.pbc[1] != 1 ? 1 : 0);
  for (int a = 0; a < 3; ++a) {
    if (c.pbc[a] == 1 && !pow2(n3[a])) { msg = "FFT (periodic) axes must be powers of two in [16, 512]"; return NS_ERR_SHAPE; }
    if (c.pbc[a] == 1) continue;
    if (a == sax && n3[a] > (c.pbc[0] != 1 ? 256 : 512)) {
      msg = "the wall axis solved by lines is limited to 512 cells (256 with a wall x)";
      return NS_ERR_SHAPE;
    }
    if (a == 1 && a != sax && n3[a] > 512) { msg = "a wall y in front of a wall z is limited to 512 cells"; return NS_ERR_SHAPE; }
    if (a == 0 && (n3[a] % 2 != 0 || n3[a] > 1024)) {
      msg = "a non-periodic x axis needs an even cell count <= 1024";
      return NS_ERR_SHAPE;
    }
  }
  if (!(c.dt > 0) || !(c.nu >= 0) || !(c.lx > 0) || !(c.ly > 0) || !(c.lz > 0)) { msg = "dt, nu, lengths"; return NS_ERR_ARG; }
  return NS_OK;
}

// After every kernel launch: count it and, while profiling, record an event.
void mark(ns_handle* h, const char* name, int nkernels = 1) {
  h->launches += nkernels;
  if (h->profiling) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) == cudaSuccess) {
      cudaEventRecord(e, h->stream);
      h->prof_events.emplace_back(name, e);
    }
  }
}
void mark_cb(void* ctx, const char* name) { mark(static_cast<ns_handle*>(ctx), name); }

// Phase trace of ns_step_host: a timed event on stream st (NS_TRACE only),
// named name, or "name s [lo,hi)" for a slab.
void trace_mark(ns_handle* h, cudaStream_t st, const char* name, int s = -1, int lo = 0, int hi = 0) {
  if (!h->trace) return;
  char buf[96];
  if (s >= 0) std::snprintf(buf, sizeof buf, "%s %d [%d,%d)", name, s, lo, hi);
  else std::snprintf(buf, sizeof buf, "%s", name);
  const size_t n = h->trace_names.size();
  if (n == h->trace_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    h->trace_pool.push_back(e);
  }
  if (cudaEventRecord(h->trace_pool[n], st) == cudaSuccess) h->trace_names.push_back(buf);
}

// Print the phases recorded since the first trace_mark, in ms from it, and reset.
void trace_flush(ns_handle* h) {
  if (!h->trace || h->trace_names.empty()) return;
  cudaDeviceSynchronize();
  for (size_t i = 0; i < h->trace_names.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->trace_pool[0], h->trace_pool[i]);
    std::fprintf(stderr, "ns_trace %-22s %9.3f ms\n", h->trace_names[i].c_str(), ms);
  }
  h->trace_names.clear();
}
Marker marker(ns_handle* h) {
  Marker m;
  m.fn = mark_cb;
  m.ctx = h;
  return m;
}

PredictArgs predict_args(ns_handle* h) {
  const ns_config& c = h->cfg;
  PredictArgs a{};
  a.L = h->L;
  a.u = h->u; a.v = h->v; a.w = h->w; a.p = h->p;
  a.us = h->us; a.vs = h->vs; a.ws = h->ws;
  a.hx = h->hx; a.hy = h->hy; a.hz = h->hz;
  a.err = h->dev_err;
  set_predict_coeffs(a, c.bc, h->dx, h->dy, h->dz, c.dt, c.nu);
  return a;
}

}  // namespace

namespace ns {

void set_predict_coeffs(PredictArgs& a, const int bc[3], double dx, double dy, double dz, double dt, double nu) {
  a.one = 1.0; a.mzero = -0.0;
  a.ulo = bc[0] == 1 ? 1 : 2;
  a.vlo = bc[1] == 1 ? 1 : 2;
  a.wlo = bc[2] == 1 ? 1 : 2;
  a.cx = -0.25 / dx; a.cy = -0.25 / dy; a.cz = -0.25 / dz;
  const double ix2 = 1.0 / (dx * dx), iy2 = 1.0 / (dy * dy), iz2 = 1.0 / (dz * dz);
  a.kx = nu * ix2; a.ky = nu * iy2; a.kz = nu * iz2;
  a.k0 = -2.0 * nu * (ix2 + iy2 + iz2);
  const double hnd = 0.5 * nu * dt;
  a.ca = hnd * ix2; a.cb = hnd * iy2; a.cc = hnd * iz2;
  a.c0 = 1.0 - 2.0 * hnd * (ix2 + iy2 + iz2);
  a.cC = 1.5 * dt; a.cP = -0.5 * dt;
  a.dt = dt; a.e1 = 1.5 * dt; a.e2 = -0.5 * dt;
  a.gpx = -dt / dx; a.gpy = -dt / dy; a.gpz = -dt / dz;
  a.ix2 = ix2; a.iy2 = iy2; a.iz2 = iz2; a.lap0 = -2.0 * (ix2 + iy2 + iz2);
}

}  // namespace ns

namespace {

// The three sweeps with fixed buffer roles: x reads A (the predictor's
// output) and writes B, y reads B and writes A, z reads A and writes B, so
// the final u*, v*, w* are in B on every step (and in every captured graph).
// With keep_sweeps the x sweep writes C instead (and y reads C), so after a
// step C holds u* after the x sweep, A after the y sweep, B after the z sweep.
AdiArgs adi_args(ns_handle* h, int ax) {
  double* A[3] = {h->us, h->vs, h->ws};
  double* B[3] = {h->us2, h->vs2, h->ws2};
  double* X[3] = {h->us3 ? h->us3 : h->us2, h->vs3 ? h->vs3 : h->vs2, h->ws3 ? h->ws3 : h->ws2};
  AdiArgs a{};
  a.L = h->L;
  for (int f = 0; f < 3; ++f) {
    a.src[f] = (ax == 1) ? X[f] : A[f];
    a.dst[f] = (ax == 1) ? A[f] : (ax == 0 ? X[f] : B[f]);
    a.sys[f] = h->sys[ax][f];
    a.face_lo[f] = h->face_set_nonzero[1 + ax] ? h->faces[1 + ax].ax[ax].f[f][0] : nullptr;
    a.face_hi[f] = h->face_set_nonzero[1 + ax] ? h->faces[1 + ax].ax[ax].f[f][1] : nullptr;
  }
  return a;
}

int enqueue_adi(ns_handle* h) {
  for (int ax = 0; ax < 3; ++ax) {
    NS_CUDA(h, launch_adi(ax, adi_args(h, ax), h->stream));
    mark(h, ax == 0 ? "adi_x" : (ax == 1 ? "adi_y" : "adi_z"));
  }
  return NS_OK;
}

// u*, v*, w* after the explicit predictor + BC fill or after the ADI sweeps.
inline void final_star(ns_handle* h, const double** fs) {
  const bool cn = h->cfg.scheme == NS_AB2_CN;
  fs[0] = cn ? h->us2 : h->us;
  fs[1] = cn ? h->vs2 : h->vs;
  fs[2] = cn ? h->ws2 : h->ws;
}

DivArgs div_args(ns_handle* h, const double* rhs) {
  const ns_config& c = h->cfg;
  DivArgs d{};
  d.rhs = rhs;
  d.L = h->L;
  const double* fs[3];
  final_star(h, fs);
  d.us = fs[0]; d.vs = fs[1]; d.ws = fs[2];
  d.cdx = 1.0 / (h->dx * c.dt); d.cdy = 1.0 / (h->dy * c.dt); d.cdz = 1.0 / (h->dz * c.dt);
  d.one = 1.0; d.mzero = -0.0;
  return d;
}

CorrectArgs correct_args(ns_handle* h) {
  const ns_config& c = h->cfg;
  CorrectArgs ca{};
  ca.L = h->L;
  const double* fs[3];
  final_star(h, fs);
  ca.us = fs[0]; ca.vs = fs[1]; ca.ws = fs[2]; ca.dp = h->dp;
  ca.u = h->u; ca.v = h->v; ca.w = h->w; ca.p = h->p;
  ca.gx = -c.dt / h->dx; ca.gy = -c.dt / h->dy; ca.gz = -c.dt / h->dz;
  ca.dp_flag = c.dp_flag; ca.gauge = c.gauge;
  for (int q = 0; q < 3; ++q) ca.per[q] = c.bc[q] == 1;
  ca.one = 1.0; ca.mzero = -0.0;
  return ca;
}

int enqueue_poisson(ns_handle* h, const double* rhs = nullptr) {
  const ns_config& c = h->cfg;
  const DivArgs d = div_args(h, rhs);
  NS_CUDA(h, launch_fft_poisson(h->plan, d, h->spec, h->dp, h->L, h->stream, marker(h)));
  NS_CUDA(h, launch_pr_bc(h->L, h->dp, h->faces[0], c.pbc, h->dx, h->dy, h->dz, h->stream));
  mark(h, "pr_bc", 3);
  return NS_OK;
}

// Everything after the predictor: the ADI sweeps (x and y unless already
// done plane by plane) or the BC fill, the Poisson solve, the correction.
int enqueue_tail(ns_handle* h, bool adi_xy_done);

int enqueue_step(ns_handle* h, bool first, cudaEvent_t after_predict = nullptr) {
  const ns_config& c = h->cfg;
  PredictArgs a = predict_args(h);
  NS_CUDA(h, launch_predict(a, c.scheme, first, c.dp_flag != 0, 0, h->stream, &h->tma));
  mark(h, "predict");
  if (after_predict) NS_CUDA(h, cudaEventRecord(after_predict, h->stream));
  return enqueue_tail(h, false);
}

// The viscous part after the predictor: the ADI sweeps (x and y unless
// already done plane by plane) or the velocity BC fill.
int enqueue_viscous(ns_handle* h, bool adi_xy_done) {
  const ns_config& c = h->cfg;
  if (c.scheme == NS_AB2_CN) {
    for (int ax = adi_xy_done ? 2 : 0; ax < 3; ++ax) {
      NS_CUDA(h, launch_adi(ax, adi_args(h, ax), h->stream));
      mark(h, ax == 0 ? "adi_x" : (ax == 1 ? "adi_y" : "adi_z"));
    }
  } else {
    NS_CUDA(h, launch_vel_bc(h->L, h->us, h->vs, h->ws, h->faces[0], c.bc, h->stream));
    mark(h, "vel_bc", 3);
  }
  return NS_OK;
}

int enqueue_tail(ns_handle* h, bool adi_xy_done) {
  int s = enqueue_viscous(h, adi_xy_done);
  if (s) return s;
  s = enqueue_poisson(h);
  if (s) return s;
  NS_CUDA(h, launch_correct(correct_args(h), h->stream));
  mark(h, "correct");
  return NS_OK;
}

// Out-copy of the slots [k0, k1) along z of field fid (0..2 u/v/w-type, 3
// p-type) into the host array dst: gathered on the compute stream into the
// staging buffer (at the array's own offsets; zero_hist zeroes the history's
// entries outside its interior ranges), then copied on the copy stream, which
// thus carries nothing but copies.
cudaError_t out_planes(ns_handle* h, const double* field, double* dst, int fid, int k0, int k1, double* stage,
                       bool zero_hist, cudaEvent_t ev) {
  const ns_config& c = h->cfg;
  const int off = fid == 2 ? 1 : 0;  // w-type: slot k is reference plane k - 1
  const int r0 = std::max(k0 - off, 0), r1 = std::min(k1 - off, ext_of(c, fid, 2));
  if (r1 <= r0) return cudaSuccess;
  int lo[3], hi[3];
  hist_range(c, fid, lo, hi);
  cudaError_t e = pack_launch(h, const_cast<double*>(field), stage, fid, false, zero_hist ? lo : nullptr,
                              zero_hist ? hi : nullptr, h->stream, r0, r1);
  if (e != cudaSuccess) return e;
  if ((e = cudaEventRecord(ev, h->stream)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(h->xfer, ev, 0)) != cudaSuccess) return e;
  const size_t pd = (size_t)ext_of(c, fid, 0) * ext_of(c, fid, 1);
  return cudaMemcpyAsync(dst + pd * r0, stage + pd * r0, sizeof(double) * pd * (r1 - r0), cudaMemcpyDeviceToHost,
                         h->xfer);
}

// The tail of ns_step_host in z-slabs (plans whose inverse passes work plane
// by plane), after the viscous part.  The forward passes and the line solve
// cover the whole box.  Then the inverse passes, the pressure ghosts and the
// correction run slab by slab [tb[s], tb[s+1]) (slots), and each slab's u, v,
// w, p are gathered and copied out on the copy stream while the next slab is
// computed.  Cell planes nz-1 and nz come first: slot 0 of the face fields
// (its periodic image) and the gauge corner dp(0,0,0) read them.  The z pass
// of the ghost fill runs with slab 0, once planes 1 and nz are final.  Every
// value is computed by the same kernels from the same inputs as in
// enqueue_tail, so the result has the same bits.
int step_host_slab_tail(ns_handle* h, const std::vector<int>& tb, double* uo, double* vo, double* wo, double* po,
                        int ev0) {
  const ns_config& c = h->cfg;
  const Layout& L = h->L;
  const int nz = c.nz;
  const DivArgs d = div_args(h, nullptr);
  NS_CUDA(h, launch_poisson_fwd(h->plan, d, h->spec, h->dp, L, h->stream, marker(h)));
  // A middle inverse pass that needs whole z lines (the z FFT of a y-wall
  // box, or a dense y transform) runs on the whole box first; the x inverse
  // pass, the ghost fill and the correction then go slab by slab.
  const bool mid_planes = poisson_inv_by_planes(h->plan);
  if (!mid_planes) NS_CUDA(h, launch_poisson_inv_mid(h->plan, d, h->spec, L, h->stream, marker(h), 1, nz + 1));
  trace_mark(h, h->stream, "poisson fwd");
  auto inv = [&](int k0, int k1) -> cudaError_t {
    cudaError_t e = mid_planes ? launch_poisson_inv_mid(h->plan, d, h->spec, L, h->stream, marker(h), k0, k1)
                               : cudaSuccess;
    if (e == cudaSuccess) e = launch_poisson_inv_x(h->plan, d, h->spec, h->dp, L, h->stream, marker(h), k0, k1);
    return e;
  };
  const CorrectArgs ca = correct_args(h);
  const int top = std::max(1, nz - 1);
  NS_CUDA(h, inv(top, nz + 1));
  NS_CUDA(h, launch_pr_bc_planes(L, h->dp, h->faces[0], c.pbc, h->dx, h->dy, top, nz + 1, h->stream));
  mark(h, "pr_bc", 2);
  double* want[4] = {uo, vo, wo, po};
  const double* have[4] = {h->u, h->v, h->w, h->p};
  const int ntail = (int)tb.size() - 1;
  for (int s = 0; s < ntail; ++s) {
    const int lo = tb[s], hi = tb[s + 1];
    const int k0 = std::max(lo, 1), k1 = std::min(hi, top);
    if (k1 > k0) {
      NS_CUDA(h, inv(k0, k1));
      NS_CUDA(h, launch_pr_bc_planes(L, h->dp, h->faces[0], c.pbc, h->dx, h->dy, k0, k1, h->stream));
      mark(h, "pr_bc", 2);
    }
    if (s == 0) {
      NS_CUDA(h, launch_pr_bc_z(L, h->dp, h->faces[0], c.pbc[2], h->dz, h->stream));
      mark(h, "pr_bc");
    }
    NS_CUDA(h, launch_correct_planes(ca, lo, hi, h->stream));
    mark(h, "correct");
    trace_mark(h, h->stream, "tail slab", s, lo, hi);
    for (int q = 0; q < 4; ++q)
      if (want[q]) NS_CUDA(h, out_planes(h, have[q], want[q], q, lo, hi, h->stage_f[q], false, h->ev_slab[ev0 + 4 * s + q]));
    trace_mark(h, h->xfer, "d2h slab", s, lo, hi);
  }
  return NS_OK;
}

int build_plans(ns_handle* h) {
  const ns_config& c = h->cfg;
  const int nx = c.nx, ny = c.ny, nz = c.nz, M = nx / 2, nxh = M + 1;
  const int n3[3] = {nx, ny, nz};
  const double hs[3] = {h->dx, h->dy, h->dz};
  FftPlan& P = h->plan;
  P = FftPlan{};
  // Axis roles: FFT on periodic axes; a wall z (else a wall y) is the
  // tridiagonal solve axis; the other wall axes get dense transforms.
  for (int a = 0; a < 3; ++a) P.kind[a] = c.pbc[a] == 1 ? 0 : 1;
  int sax = 0;  // solve axis (0: the fused FFT z solve)
  if (P.kind[2] == 1) sax = 2;
  else if (P.kind[1] == 1) sax = 1;
  if (sax) P.kind[sax] = 2;
  const bool xper = P.kind[0] == 0;
  const int nxs = xper ? nxh : nx / 2;
  // Twiddles W_N^m = exp(-2 pi i m / N), computed in long double (FFT axes only).
  auto twid = [](int N, int count, std::vector<double2>& out) {
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int m = 0; m < count; ++m) {
      const long double th = 2.0L * pi * (long double)m / (long double)N;
      out.push_back(make_double2((double)cosl(th), (double)(-sinl(th))));
    }
  };
  std::vector<double2> tw;
  size_t o_xr = 0, o_y = 0, o_z = 0;
  if (xper) {
    twid(M, M, tw);
    o_xr = tw.size();
    twid(nx, M / 2 + 1, tw);
  }
  o_y = tw.size();
  if (P.kind[1] == 0) twid(ny, ny, tw);
  o_z = tw.size();
  if (P.kind[2] == 0) twid(nz, nz, tw);
  // A dense y (in front of a wall z) of length 24, 48 or a power of two from
  // 32 to 512 with pbc 2 or 3 goes through an FFT: its twiddles and the DCT
  // pre/post-twiddles.  (NS_DENSE_Y in the environment keeps the dense
  // products, for comparison.)
  auto dct_len = [](int m) { return m == 24 || m == 48 || (m >= 32 && m <= 512 && (m & (m - 1)) == 0); };
  P.dct_y = 0;
  size_t o_dtw = 0, o_dwf = 0, o_dwi = 0;
  if (P.kind[1] == 1 && (c.pbc[1] == 2 || c.pbc[1] == 3) && dct_len(ny) && !std::getenv("NS_DENSE_Y")) {
    P.dct_y = c.pbc[1];
    const long double pi = 3.141592653589793238462643383279502884L;
    o_dtw = tw.size();
    twid(ny, ny, tw);
    o_dwf = tw.size();
    for (int k = 0; k <= ny; ++k) {
      const long double th = pi * (long double)k / (2.0L * ny);
      tw.push_back(make_double2((double)(cosl(th) / 2.0L), (double)(-sinl(th) / 2.0L)));
    }
    o_dwi = tw.size();
    for (int k = 0; k < ny; ++k) {
      const long double th = pi * (long double)k / (2.0L * ny);
      tw.push_back(make_double2((double)(cosl(th) / ny), (double)(sinl(th) / ny)));
    }
  }
  // The same for a wall x axis (NS_DENSE_X keeps the dense products).
  P.dct_x = 0;
  size_t o_xtw = 0, o_xwf = 0, o_xwi = 0;
  if (P.kind[0] == 1 && (c.pbc[0] == 2 || c.pbc[0] == 3) && dct_len(nx) && !std::getenv("NS_DENSE_X")) {
    P.dct_x = c.pbc[0];
    const long double pi = 3.141592653589793238462643383279502884L;
    o_xtw = tw.size();
    twid(nx, nx, tw);
    o_xwf = tw.size();
    for (int k = 0; k <= nx; ++k) {
      const long double th = pi * (long double)k / (2.0L * nx);
      tw.push_back(make_double2((double)(cosl(th) / 2.0L), (double)(-sinl(th) / 2.0L)));
    }
    o_xwi = tw.size();
    for (int k = 0; k < nx; ++k) {
      const long double th = pi * (long double)k / (2.0L * nx);
      tw.push_back(make_double2((double)(cosl(th) / nx), (double)(sinl(th) / nx)));
    }
  }
  if (tw.empty()) tw.push_back(make_double2(1.0, 0.0));
  NS_CUDA(h, cudaMalloc(&h->tw, tw.size() * sizeof(double2)));
  NS_CUDA(h, cudaMemcpyAsync(h->tw, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  // Per-axis eigenvalues lambda = -4 sin^2(..)/h^2 of each mode.
  std::vector<double> e3[3];
  for (int a = 0; a < 3; ++a) {
    const int cnt = (a == 0 && xper) ? nxh : n3[a];
    e3[a].resize(cnt);
    for (int m = 0; m < cnt; ++m) e3[a][m] = -4.0 * axis_eig(n3[a], c.pbc[a], m, hs[a]);
  }
  // Scale of the unnormalised FFT passes (x: 2 nx for the r2c/c2r pair); the
  // dense pairs are exact inverses.
  double scale = 1.0;
  if (xper) scale /= 2.0 * nx;
  if (P.kind[1] == 0) scale /= ny;
  if (P.kind[2] == 0) scale /= nz;
  const bool allper = c.pbc[0] == 1 && c.pbc[1] == 1 && c.pbc[2] == 1;
  bool singular = true;
  for (int a = 0; a < 3; ++a) singular = singular && (c.pbc[a] == 1 || c.pbc[a] == 3);
  // The singular mode: zero mean for the all-periodic FFT solve
  // (big_periodic_3D.f90:242-255), mean_dp otherwise (NS_functions.f90:1576-1577).
  P.has_mean = (singular && !allper) ? 1 : 0;
  // Device tables: dense matrices (x stored transposed: F^T, G^T), then the
  // eigenvalue tables of the tridiagonal solve, or the 1/lambda table of the
  // FFT z solve.
  std::vector<double> tab;
  size_t o_f[3] = {0, 0, 0}, o_g[3] = {0, 0, 0}, o_ex = 0, o_eo = 0, o_il = 0;
  for (int a = 0; a < 3; ++a) {
    if (P.kind[a] != 1) continue;
    std::vector<double> F, G;
    dense_pair(n3[a], c.pbc[a], F, G);
    const int n = n3[a];
    P.sym[a] = dense_symmetry(n, F, G);
    if (a == 0) {
      std::vector<double> Ft((size_t)n * n), Gt((size_t)n * n);
      for (int r = 0; r < n; ++r)
        for (int q = 0; q < n; ++q) {
          Ft[(size_t)q * n + r] = F[(size_t)r * n + q];
          Gt[(size_t)q * n + r] = G[(size_t)r * n + q];
        }
      F.swap(Ft);
      G.swap(Gt);
    }
    o_f[a] = tab.size();
    tab.insert(tab.end(), F.begin(), F.end());
    o_g[a] = tab.size();
    tab.insert(tab.end(), G.begin(), G.end());
  }
  const size_t nspec = (size_t)nxs * ny * nz;
  if (sax) {
    const int oax = 3 - sax;
    o_ex = tab.size();
    tab.insert(tab.end(), e3[0].begin(), e3[0].end());
    o_eo = tab.size();
    tab.insert(tab.end(), e3[oax].begin(), e3[oax].end());
    const double hh = hs[sax];
    const int pb = c.pbc[sax];
    const double e_end = pb == 2 ? -1.0 : (pb == 3 ? 1.0 : 0.0);
    P.tri_h2 = hh * hh;
    P.tri_rs = hh * hh * scale;
    P.tri_elo = P.tri_ehi = e_end;
    double dense_other = 1.0;
    for (int a = 0; a < 3; ++a)
      if (a != sax && P.kind[a] == 1) dense_other *= n3[a];
    // mean of the singular line: dense_other * mean_dp, mean_dp read on the
    // device so that ns_set_mean_dp changes it without a new plan or graph
    if (!h->mean_dev) NS_CUDA(h, cudaMalloc(&h->mean_dev, sizeof(double)));
    NS_CUDA(h, cudaMemcpyAsync(h->mean_dev, &c.mean_dp, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    P.mean_val = dense_other;
    P.mean_dev = h->mean_dev;
  } else if (allper && c.poisson_z == 0) {
    // cyclic z solve: the x and y eigenvalues give each z line's diagonal
    o_ex = tab.size();
    tab.insert(tab.end(), e3[0].begin(), e3[0].end());
    o_eo = tab.size();
    tab.insert(tab.end(), e3[1].begin(), e3[1].end());
    P.mean_val = 0.0;
  } else {
    o_il = tab.size();
    tab.resize(tab.size() + nspec);
    double* il = tab.data() + o_il;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nxh; ++i) {
          const double lam = (e3[0][i] + e3[1][j]) + e3[2][k];
          il[i + (size_t)nxh * (j + (size_t)ny * k)] = (i == 0 && j == 0 && k == 0) ? 0.0 : scale / lam;
        }
    P.mean_val = 0.0;
  }
  if (tab.empty()) tab.push_back(0.0);
  NS_CUDA(h, cudaMalloc(&h->inv_lam, tab.size() * sizeof(double)));
  NS_CUDA(h, cudaMemcpyAsync(h->inv_lam, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  NS_CUDA(h, cudaMalloc(&h->spec, nspec * sizeof(double2)));
  const double* t0 = h->inv_lam;
  P.nx = nx; P.ny = ny; P.nz = nz; P.nxh = nxh; P.nxs = nxs;
  P.tw_x = h->tw; P.tw_xr = h->tw + o_xr; P.tw_y = h->tw + o_y; P.tw_z = h->tw + o_z;
  P.dct_tw = P.dct_y ? h->tw + o_dtw : nullptr;
  P.dct_wf = P.dct_y ? h->tw + o_dwf : nullptr;
  P.dct_wi = P.dct_y ? h->tw + o_dwi : nullptr;
  P.dctx_tw = P.dct_x ? h->tw + o_xtw : nullptr;
  P.dctx_wf = P.dct_x ? h->tw + o_xwf : nullptr;
  P.dctx_wi = P.dct_x ? h->tw + o_xwi : nullptr;
  const bool zcyc = !sax && allper && c.poisson_z == 0;
  P.inv_lam = (sax || zcyc) ? nullptr : t0 + o_il;
  P.eig_x = (sax || zcyc) ? t0 + o_ex : nullptr;
  P.eig_o = (sax || zcyc) ? t0 + o_eo : nullptr;
  for (int a = 0; a < 3; ++a) {
    P.fwd[a] = P.kind[a] == 1 ? t0 + o_f[a] : nullptr;
    P.inv[a] = P.kind[a] == 1 ? t0 + o_g[a] : nullptr;
  }
  // pr_bc_staggered_modify_rhs coefficients (NS_functions.f90:1345-1400) and
  // the set-0 pressure face planes they read.
  for (int a = 0; a < 3; ++a) {
    const double hh = hs[a];
    P.mod_lo[a] = P.mod_hi[a] = 0.0;
    if (c.pbc[a] == 2) { P.mod_lo[a] = -2.0 / (hh * hh); P.mod_hi[a] = -2.0 / (hh * hh); }
    else if (c.pbc[a] == 3) { P.mod_lo[a] = 1.0 / hh; P.mod_hi[a] = -1.0 / hh; }
    else if (c.pbc[a] == 4) { P.mod_lo[a] = -1.0 / (hh * hh); P.mod_hi[a] = -1.0 / (hh * hh); }
    P.face_lo[a] = h->faces[0].ax[a].f[3][0];
    P.face_hi[a] = h->faces[0].ax[a].f[3][1];
  }
  if (zcyc) {
    P.zcyc = 1;
    P.cyc_h2 = h->dz * h->dz;
    P.cyc_rs = h->dz * h->dz * scale * nz;
    NS_CUDA(h, cudaMalloc(&h->cyc_buf, cyc_table_doubles(P) * sizeof(double)));
    NS_CUDA(h, launch_cyc_table(P, h->cyc_buf, h->stream));
    NS_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  // The wall-axis line solve: the twisted factorisation from a table of its
  // multipliers made once here (no division in the solve, two lanes per
  // line).  The one-lane Thomas solve that computes its multipliers stays
  // for lines shorter than 8 (NS_TRI_THOMAS keeps it, for comparison).
  P.tri_m = nullptr;
  P.sing_cm = nullptr;
  P.tri_tw = 0;
  const int nsax = sax == 1 ? ny : nz;
  if (sax != 0 && nsax >= 8 && !std::getenv("NS_TRI_THOMAS")) {
    NS_CUDA(h, cudaMalloc(&h->tri_tab, (size_t)nxs * ny * nz * sizeof(double2)));
    NS_CUDA(h, cudaMalloc(&h->sing_cm, (size_t)2 * nsax * 32 * sizeof(double)));
    NS_CUDA(h, launch_tri_twist_table(sax, P, h->tri_tab, h->stream));
    NS_CUDA(h, cudaStreamSynchronize(h->stream));
    P.tri_m = h->tri_tab;
    P.sing_cm = h->sing_cm;
    P.tri_tw = 1;
  }
  return NS_OK;
}

constexpr int kAdiPad = 8;  // zero padding on each side of the factor tables

// Factor tables of the nine line systems (3 sweeps x 3 fields) in one device
// buffer *buf; transposed: the systems of the adjoint sweeps.
int build_line_tables(ns_handle* h, bool transposed, LineSys sys[3][3], double** buf) {
  const ns_config& c = h->cfg;
  const int ns_[3] = {c.nx, c.ny, c.nz};
  const double hs[3] = {h->dx, h->dy, h->dz};
  HostLineSys hs_sys[3][3];
  size_t total = 0;
  for (int ax = 0; ax < 3; ++ax)
    for (int f = 0; f < 3; ++f) {
      hs_sys[ax][f] =
          build_cn_system(ns_[ax], c.bc[ax], hs[ax], c.dt, c.nu, f == ax, c.cn_periodic_closure, transposed);
      total += (hs_sys[ax][f].l.size() + 2 * kAdiPad) * 3 + hs_sys[ax][f].z.size();
    }
  NS_CUDA(h, cudaMalloc(buf, total * sizeof(double)));
  std::vector<double> host(total, 0.0);
  size_t off = 0;
  for (int ax = 0; ax < 3; ++ax)
    for (int f = 0; f < 3; ++f) {
      const HostLineSys& S = hs_sys[ax][f];
      LineSys& D = sys[ax][f];
      const size_t m = S.l.size(), mp = m + 2 * kAdiPad;
      std::memcpy(&host[off + kAdiPad], S.l.data(), m * sizeof(double)); D.l = *buf + off; off += mp;
      std::memcpy(&host[off + kAdiPad], S.dinv.data(), m * sizeof(double)); D.dinv = *buf + off; off += mp;
      std::memcpy(&host[off + kAdiPad], S.cu.data(), m * sizeof(double)); D.cu = *buf + off; off += mp;
      std::memcpy(&host[off], S.z.data(), S.z.size() * sizeof(double)); D.z = *buf + off; off += S.z.size();
      D.s0 = S.s0; D.s1 = S.s1; D.zA = S.zA; D.zB = S.zB; D.lo = S.lo; D.hi = S.hi;
      D.periodic = S.periodic; D.n = S.n; D.pad = kAdiPad;
    }
  NS_CUDA(h, cudaMemcpyAsync(*buf, host.data(), total * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int build_adi(ns_handle* h) {
  if (h->cfg.scheme != NS_AB2_CN) return NS_OK;
  return build_line_tables(h, false, h->sys, &h->adi_buf);
}

void free_all(ns_handle* h) {
  ns::api_free_adjoint(h);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  double* bufs[] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz, h->us, h->vs, h->ws, h->dp, h->inv_lam, h->adi_buf, h->face_buf,
                    h->us2, h->vs2, h->ws2, h->us3, h->vs3, h->ws3};
  for (double* b : bufs)
    if (b) cudaFree(b);
  if (h->spec) cudaFree(h->spec);
  if (h->mean_dev) cudaFree(h->mean_dev);
  if (h->tri_tab) cudaFree(h->tri_tab);
  if (h->sing_cm) cudaFree(h->sing_cm);
  if (h->cyc_buf) cudaFree(h->cyc_buf);
  if (h->stage) cudaFree(h->stage);
  if (h->stage2) cudaFree(h->stage2);
  if (h->xfer) cudaStreamDestroy(h->xfer);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->prio) cudaStreamDestroy(h->prio);
  if (h->scat) cudaStreamDestroy(h->scat);
  for (int b = 0; b < 2; ++b) {
    if (h->ev_full[b]) cudaEventDestroy(h->ev_full[b]);
    if (h->ev_free[b]) cudaEventDestroy(h->ev_free[b]);
    if (h->ev_aux[b]) cudaEventDestroy(h->ev_aux[b]);
  }
  for (double* b : h->stage_f)
    if (b) cudaFree(b);
  for (cudaEvent_t e : h->ev_slab) cudaEventDestroy(e);
  for (cudaEvent_t e : h->trace_pool) cudaEventDestroy(e);
  if (h->tw) cudaFree(h->tw);
  if (h->diag_bits) cudaFree(h->diag_bits);
  if (h->dev_err) cudaFree(h->dev_err);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
}

}  // namespace

// Session internals shared with the adjoint tier (ns_adjoint.cu).
namespace ns {
int api_fail(ns_handle* h, int code, const std::string& msg) { return fail(h, code, msg); }
cudaError_t api_h2d_field(ns_handle* h, double* dst, const double* src, int field) {
  return h2d_field(h, dst, src, field);
}
cudaError_t api_d2h_field(ns_handle* h, double* dst, const double* src, int field) {
  return d2h_field(h, dst, src, field);
}
void api_mark(ns_handle* h, const char* name, int nkernels) { mark(h, name, nkernels); }
Marker api_marker(ns_handle* h) { return marker(h); }
int api_build_line_tables(ns_handle* h, bool transposed, LineSys sys[3][3], double** buf) {
  return build_line_tables(h, transposed, sys, buf);
}
}  // namespace ns

extern "C" {

const char* ns_version(void) { return "ns_gpu 0.1 (sm_103a, FP64)"; }

int ns_selftest_wait_timeout(double limit_ms, double* waited_ms) {
  if (!(limit_ms > 0.0) || limit_ms > 1000.0) return NS_ERR_ARG;
  int* d_gave = nullptr;
  unsigned long long* d_ns = nullptr;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NS_ERR_CUDA;
  int status = NS_OK;
  if (cudaMalloc(&d_gave, sizeof(int)) != cudaSuccess || cudaMalloc(&d_ns, sizeof(unsigned long long)) != cudaSuccess)
    status = NS_ERR_NOMEM;
  int gave = 0;
  unsigned long long ns = 0;
  if (!status && launch_wait_selftest((unsigned long long)(limit_ms * 1e6), d_gave, d_ns, st) != cudaSuccess)
    status = NS_ERR_CUDA;
  if (!status && (cudaMemcpyAsync(&gave, d_gave, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                  cudaMemcpyAsync(&ns, d_ns, sizeof(ns), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                  cudaStreamSynchronize(st) != cudaSuccess))
    status = NS_ERR_CUDA;
  if (d_gave) cudaFree(d_gave);
  if (d_ns) cudaFree(d_ns);
  cudaStreamDestroy(st);
  if (status) return status;
  if (waited_ms) *waited_ms = (double)ns * 1e-6;
  return gave ? NS_ERR_TIMEOUT : NS_OK;
}

const char* ns_status_string(int s) {
  switch (s) {
    case NS_OK: return "ok";
    case NS_ERR_SHAPE: return "unsupported grid shape";
    case NS_ERR_CUDA: return "CUDA error";
    case NS_ERR_NONFINITE: return "non-finite value";
    case NS_ERR_TIMEOUT: return "device wait timed out";
    case NS_ERR_UNSUPPORTED_BC: return "unsupported boundary condition";
    case NS_ERR_ARG: return "bad argument";
    case NS_ERR_NOMEM: return "out of device memory";
    case NS_ERR_IO: return "file read/write failed or the file is outside the HDF5 subset";
    default: return "unknown status";
  }
}

int ns_config_default(ns_config* c, int nx, int ny, int nz) {
  if (!c) return NS_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  const double pi = 3.1415926535897932;
  c->nx = nx; c->ny = ny; c->nz = nz;
  c->lx = 2.0 * pi; c->ly = 2.0 * pi; c->lz = 2.0 * pi;
  c->nu = 0.002; c->dt = 2.5e-4;
  c->scheme = NS_AB2;
  for (int a = 0; a < 3; ++a) { c->bc[a] = 1; c->pbc[a] = 1; }
  c->dp_flag = 0; c->gauge = 1; c->mean_dp = 0.0;
  c->cn_periodic_closure = 0;
  c->use_graph = 1;
  return NS_OK;
}

int ns_create(const ns_config* cfg, ns_handle** out) {
  if (!cfg || !out) return NS_ERR_ARG;
  *out = nullptr;
  std::string msg;
  int s = validate(*cfg, msg);
  if (s) {
    std::fprintf(stderr, "ns_create: %s\n", msg.c_str());
    return s;
  }
  ns_handle* h = new ns_handle();
  h->cfg = *cfg;
  h->trace = std::getenv("NS_TRACE") != nullptr;
  h->L = make_layout(cfg->nx, cfg->ny, cfg->nz);
  h->dx = cfg->lx / cfg->nx; h->dy = cfg->ly / cfg->ny; h->dz = cfg->lz / cfg->nz;
  auto bail = [&](int code) { free_all(h); delete h; return code; };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(NS_ERR_CUDA);
  h->own_stream = true;
  if (cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(NS_ERR_CUDA);
  double** fields[] = {&h->u, &h->v, &h->w, &h->p, &h->hx, &h->hy, &h->hz, &h->us, &h->vs, &h->ws, &h->dp,
                       &h->us2, &h->vs2, &h->ws2};
  for (double** f : fields) {
    if (cudaMalloc(f, h->L.fsize * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
    if (cudaMemsetAsync(*f, 0, h->L.fsize * sizeof(double), h->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  }
  if (cfg->keep_sweeps && cfg->scheme == NS_AB2_CN) {
    double** kept[] = {&h->us3, &h->vs3, &h->ws3};
    for (double** f : kept) {
      if (cudaMalloc(f, h->L.fsize * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
      if (cudaMemsetAsync(*f, 0, h->L.fsize * sizeof(double), h->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
    }
  }
  const size_t ft = face_total(h->L);
  if (cudaMalloc(&h->face_buf, ft * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMemsetAsync(h->face_buf, 0, ft * sizeof(double), h->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  for (int set = 0; set < 4; ++set)
    for (int a = 0; a < 3; ++a)
      for (int f = 0; f < 4; ++f)
        for (int d = 0; d < 2; ++d) h->faces[set].ax[a].f[f][d] = h->face_buf + face_offset(h->L, set, a, f, d);
  if (cudaMalloc(&h->diag_bits, sizeof(unsigned long long)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMalloc(&h->dev_err, sizeof(int)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMemsetAsync(h->dev_err, 0, sizeof(int), h->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  // The predictor stages its tiles with cp.async.  NS_PREDICT_TMA=1 in the
  // environment selects the tensor-memory-access loader instead (the same
  // bits; measured 3.3 ms against 2.1 ms per 256^3 launch, so not the default).
  // A requested loader that cannot be set up fails ns_create rather than
  // running the other one silently.
  const char* tma_env = std::getenv("NS_PREDICT_TMA");
  if (tma_env && tma_env[0] == '1' && !ns::make_pred_tma(h->tma, h->L, h->u, h->v, h->w)) {
    h->err = "NS_PREDICT_TMA=1: the tile loader's tensor maps could not be encoded";
    std::fprintf(stderr, "ns_create: %s\n", h->err.c_str());
    return bail(NS_ERR_CUDA);
  }
  if ((s = build_plans(h)) != NS_OK) { std::fprintf(stderr, "ns_create: %s\n", h->err.c_str()); return bail(s); }
  if ((s = build_adi(h)) != NS_OK) { std::fprintf(stderr, "ns_create: %s\n", h->err.c_str()); return bail(s); }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  *out = h;
  return NS_OK;
}

int ns_destroy(ns_handle* h) {
  if (!h) return NS_ERR_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return NS_OK;
}

const char* ns_last_error(const ns_handle* h) { return h ? h->err.c_str() : "null handle"; }

int ns_set_stream(ns_handle* h, void* stream) {
  if (!h) return NS_ERR_ARG;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->stream = (cudaStream_t)stream;
  h->own_stream = false;
  if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
  return NS_OK;
}

int ns_synchronize(ns_handle* h) {
  if (!h) return NS_ERR_ARG;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int ns_set_state(ns_handle* h, const double* u, const double* v, const double* w, const double* p, const double* hx,
                 const double* hy, const double* hz) {
  if (!h || !u || !v || !w || !p) return fail(h, NS_ERR_ARG, "u, v, w, p are required");
  const bool hist = hx && hy && hz;
  double* dst[7] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz};
  const double* src[7] = {u, v, w, p, hx, hy, hz};
  const int fid[7] = {0, 1, 2, 3, 0, 1, 2};
  NS_CUDA(h, h2d_fields(h, hist ? 7 : 4, dst, src, fid));
  // The extra face slot 0 of a periodic axis mirrors face n.
  NS_CUDA(h, launch_extra_slots(h->L, h->u, h->v, h->w, h->cfg.bc, h->stream));
  if (!hist) {
    NS_CUDA(h, cudaMemsetAsync(h->hx, 0, h->L.fsize * sizeof(double), h->stream));
    NS_CUDA(h, cudaMemsetAsync(h->hy, 0, h->L.fsize * sizeof(double), h->stream));
    NS_CUDA(h, cudaMemsetAsync(h->hz, 0, h->L.fsize * sizeof(double), h->stream));
  }
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  h->first_pending = !hist;
  h->steps = 0;
  return NS_OK;
}

int ns_get_state(ns_handle* h, double* u, double* v, double* w, double* p, double* hx, double* hy, double* hz) {
  if (!h) return NS_ERR_ARG;
  double* const all_dst[7] = {u, v, w, p, hx, hy, hz};
  const double* all_src[7] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz};
  double* dst[7];
  const double* src[7];
  int fid[7];
  bool zero[7];
  int n = 0;
  for (int q = 0; q < 7; ++q) {
    if (!all_dst[q]) continue;
    dst[n] = all_dst[q];
    src[n] = all_src[q];
    fid[n] = q < 4 ? q : q - 4;
    zero[n] = q >= 4;  // history outside the interior ranges is returned as zero
    ++n;
  }
  NS_CUDA(h, d2h_fields(h, n, dst, src, fid, zero));
  return NS_OK;
}

int ns_step_host(ns_handle* h, const double* u, const double* v, const double* w, const double* p, const double* hx,
                 const double* hy, const double* hz, double* uo, double* vo, double* wo, double* po, double* hxo,
                 double* hyo, double* hzo) {
  if (!h || !u || !v || !w) return fail(h, NS_ERR_ARG, "u, v, w are required");
  const ns_config& c = h->cfg;
  if (c.dp_flag && !p) return fail(h, NS_ERR_ARG, "p is required with dp_flag = 1");
  NS_CUDA(h, ensure_xfer(h));
  const Layout& L = h->L;
  const int nz = c.nz;
  const bool hist = hx && hy && hz;
  // state in: the fields the step reads (p only with dp_flag = 1), one staging buffer each
  struct In { double* dev; const double* host; int fid; int q; };
  std::vector<In> in = {{h->u, u, 0, 0}, {h->v, v, 1, 1}, {h->w, w, 2, 2}};
  if (hist) { in.push_back({h->hx, hx, 0, 4}); in.push_back({h->hy, hy, 1, 5}); in.push_back({h->hz, hz, 2, 6}); }
  if (c.dp_flag) in.push_back({h->p, p, 3, 3});
  // state out; staging buffer q serves field q in and out (disjoint planes at any time)
  double* const out[7] = {uo, vo, wo, po, hxo, hyo, hzo};
  const double* const out_dev[7] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz};
  bool need_stage[7] = {false, false, false, false, false, false, false};
  for (const In& f : in) need_stage[f.q] = true;
  for (int q = 0; q < 7; ++q) need_stage[q] = need_stage[q] || out[q];
  for (int q = 0; q < 7; ++q)
    if (need_stage[q] && !h->stage_f[q]) NS_CUDA(h, cudaMalloc(&h->stage_f[q], field_bytes(c, q < 4 ? q : q - 4)));
  // z-slabs: copy, scatter, predict, x and y sweeps of slab s run while slab
  // s+1 is being copied.  The first slab holds one predictor chunk (and the
  // two planes above it that the predictor reads), so compute starts early;
  // then 4 chunks a slab (2-chunk slabs left each launch under one wave of
  // CTAs); the compute of the last slab is not hidden, so the slabs shrink
  // towards the top: half the rest (whole chunks, rounded down) once less
  // than two full slabs remain (18, 64, 64, 48, 32, 16, 16 planes at 256).
  const int KC = predict_chunk_planes();
  const int S = 4 * KC;
  std::vector<int> fb = {0, std::min(nz + 2, KC + 2)};
  while (fb.back() < nz + 2) {
    const int r = nz + 2 - fb.back();
    int take = r;
    if (r >= 2 * S) take = S;
    else if (r > KC + 2) take = std::max(KC, r / 2 / KC * KC);
    fb.push_back(fb.back() + take);
  }
  const int nslab = (int)fb.size() - 1;
  // The tail in z-slabs as well when the inverse passes work plane by plane:
  // each slab's u, v, w, p leave while the next slab is computed.  The first
  // slab is small (its compute comes before any of the tail's copies).
  const bool slab_tail = poisson_inv_x_by_planes(h->plan);
  std::vector<int> tb = {0};
  if (slab_tail) {
    // sizes doubling from KC/2 + 1 up to S: each slab's compute about as
    // long as the copy of the one before
    int sz = KC / 2 + 1;
    while (tb.back() < nz + 2) {
      tb.push_back(std::min(nz + 2, tb.back() + sz));
      sz = std::min(S, tb.size() == 2 ? KC : 2 * sz);
    }
  }
  while (tb.back() < nz + 2) tb.push_back(std::min(nz + 2, tb.back() + S));
  const int ntail = (int)tb.size() - 1;
  // events: front slabs (copy done), start, history out (3 per front slab),
  // state out (4 per tail slab), predictor done (per front slab), sweeps
  // done, the periodic-image prelude done, scatter done (per front slab)
  const int ev_start = nslab, ev_hist = nslab + 1, ev_tail = ev_hist + 3 * nslab, ev_pred = ev_tail + 4 * ntail;
  const int ev_sweeps = ev_pred + nslab, ev_pre = ev_sweeps + 1, ev_scat = ev_pre + 1;
  while ((int)h->ev_slab.size() < ev_scat + nslab) {
    cudaEvent_t e;
    NS_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->ev_slab.push_back(e);
  }
  // The compute runs on two greatest-priority streams of the handle (after
  // the caller's stream): the predictor chain on one, the x and y sweeps of
  // each finished slab beside it on the other, ahead of any other work on the
  // device.  (With the sweeps at the lowest priority they fell a slab behind;
  // in line after the predictor, the slab's sliced sweeps made the chain as
  // slow as the copies.)
  trace_mark(h, h->stream, "start");
  NS_CUDA(h, cudaEventRecord(h->ev_slab[ev_start], h->stream));
  NS_CUDA(h, cudaStreamWaitEvent(h->xfer, h->ev_slab[ev_start], 0));
  NS_CUDA(h, cudaStreamWaitEvent(h->prio, h->ev_slab[ev_start], 0));
  NS_CUDA(h, cudaStreamWaitEvent(h->scat, h->ev_slab[ev_start], 0));
  struct StreamSwap {
    ns_handle* h;
    cudaStream_t saved;
    ~StreamSwap() { h->stream = saved; }
  } swap{h, h->stream};
  h->stream = h->prio;
  if (!hist) {
    NS_CUDA(h, cudaMemsetAsync(h->hx, 0, L.fsize * sizeof(double), h->stream));
    NS_CUDA(h, cudaMemsetAsync(h->hy, 0, L.fsize * sizeof(double), h->stream));
    NS_CUDA(h, cudaMemsetAsync(h->hz, 0, L.fsize * sizeof(double), h->stream));
  }
  auto plane_bytes = [&](int fid) {
    return sizeof(double) * (size_t)ext_of(c, fid, 0) * ext_of(c, fid, 1);
  };
  // reference planes [r0, r1) of field f that hold z slots [lo, hi)
  auto ref_range = [&](const In& f, int lo, int hi, int& r0, int& r1) {
    const int off = (f.fid == 2) ? 1 : 0;  // w-type fields: slot k is reference plane k - 1
    const int ez = ext_of(c, f.fid, 2);
    r0 = std::max(lo - off, 0);
    r1 = std::min(hi - off, ez);
  };
  auto copy_in = [&](const In& f, int r0, int r1) -> cudaError_t {
    if (r1 <= r0) return cudaSuccess;
    const size_t pb = plane_bytes(f.fid), pd = pb / sizeof(double);
    return cudaMemcpyAsync(h->stage_f[f.q] + pd * r0, f.host + pd * r0, pb * (r1 - r0), cudaMemcpyHostToDevice,
                           h->xfer);
  };
  // The periodic image w(slot 0) = w(slot nz) is read by the first chunk:
  // bring the w plane of slot nz in ahead of the slabs.
  const bool zper = c.bc[2] == 1;
  if (zper) {
    NS_CUDA(h, copy_in(in[2], nz - 1, nz));
    NS_CUDA(h, cudaEventRecord(h->ev_full[0], h->xfer));
    NS_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_full[0], 0));
    NS_CUDA(h, pack_launch(h, h->w, h->stage_f[2], 2, true, nullptr, nullptr, nullptr, nz - 1, nz));
    const int zonly[3] = {0, 0, 1};
    NS_CUDA(h, launch_extra_slots(L, h->u, h->v, h->w, zonly, h->stream));
    // the last slab's scatter rewrites slot nz (same bits) after this read of it
    NS_CUDA(h, cudaEventRecord(h->ev_slab[ev_pre], h->stream));
    NS_CUDA(h, cudaStreamWaitEvent(h->scat, h->ev_slab[ev_pre], 0));
  }
  for (int s = 0; s < nslab; ++s) {
    const int lo = fb[s], hi = fb[s + 1];
    for (const In& f : in) {
      int r0, r1;
      ref_range(f, lo, hi, r0, r1);
      NS_CUDA(h, copy_in(f, r0, r1));
    }
    NS_CUDA(h, cudaEventRecord(h->ev_slab[s], h->xfer));
    trace_mark(h, h->xfer, "h2d slab", s, lo, hi);
  }
  const bool cn = c.scheme == NS_AB2_CN;
  const bool first = !hist && c.scheme != NS_EULER;
  int pred_done = 1, xy_done = 0, hist_done = 0;  // next cell plane to predict; slots swept / sent out
  PredictArgs pa = predict_args(h);
  // Every slab is scattered into the padded layout on its own stream as soon
  // as it lands: the scatter writes slots [lo, hi) only, above every plane
  // the previous slab's predictor launch reads (its prefetch stops at slot
  // hi_prev - 1) and the planes whose history is being sent out, so it runs
  // beside that launch instead of queueing behind it.
  for (int s = 0; s < nslab; ++s) {
    const int lo = fb[s], hi = fb[s + 1];
    NS_CUDA(h, cudaStreamWaitEvent(h->scat, h->ev_slab[s], 0));
    for (const In& f : in) {
      int r0, r1;
      ref_range(f, lo, hi, r0, r1);
      NS_CUDA(h, pack_launch(h, f.dev, h->stage_f[f.q], f.fid, true, nullptr, nullptr, h->scat, r0, r1));
    }
    {
      const long long n = (long long)(hi - lo) * (L.nx + L.ny + 4);
      extra_xy_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 1024), 256, 0, h->scat>>>(
          L, h->u, h->v, c.bc[0] == 1, c.bc[1] == 1, lo, hi);
      NS_CUDA(h, cudaGetLastError());
    }
    NS_CUDA(h, cudaEventRecord(h->ev_slab[ev_scat + s], h->scat));
    trace_mark(h, h->scat, "scatter", s, lo, hi);
  }
  for (int s = 0; s < nslab; ++s) {
    const int lo = fb[s], hi = fb[s + 1];
    NS_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_slab[ev_scat + s], 0));
    // cell planes whose stencil and the two planes above it (read by the
    // prefetch) have arrived; a quarter of the range per CTA, at most
    // KC planes: short ranges at the top spread over as many CTAs as a
    // full slab, so the compute left after the last copy is short.
    const int e = hi >= nz + 2 ? nz + 1 : std::min(nz + 1, hi - 2);
    if (e > pred_done) {
      const int kc = std::max(2, std::min(KC, (e - pred_done) / 4));
      NS_CUDA(h, launch_predict_planes(pa, c.scheme, first, c.dp_flag != 0, pred_done, e, kc, h->stream, &h->tma));
      mark(h, "predict");
      trace_mark(h, h->stream, "predict", s, lo, hi);
      pred_done = e;
      // the history of the finished planes is final: out on the copy stream
      // (after the copies in, in stream order)
      const int done = e == nz + 1 ? nz + 2 : e;
      for (int q = 0; q < 3; ++q)
        if (out[4 + q])
          NS_CUDA(h, out_planes(h, out_dev[4 + q], out[4 + q], q, hist_done, done, h->stage_f[4 + q], true,
                                h->ev_slab[ev_hist + 3 * s + q]));
      hist_done = done;
      if (cn) {
        // x and y sweeps of the planes the predictor has finished, on the
        // side stream: they touch only those planes of u*, v*, w* (and their
        // second buffers), which the next predictor launch neither reads nor
        // writes, so they fill the wave tails of the next slab's launches.
        NS_CUDA(h, cudaEventRecord(h->ev_slab[ev_pred + s], h->stream));
        NS_CUDA(h, cudaStreamWaitEvent(h->side, h->ev_slab[ev_pred + s], 0));
        for (int ax = 0; ax < 2; ++ax) {
          AdiArgs a = adi_args(h, ax);
          a.z0 = xy_done;
          a.z1 = done;
          NS_CUDA(h, launch_adi(ax, a, h->side));
          mark(h, ax == 0 ? "adi_x" : "adi_y");
          trace_mark(h, h->side, ax == 0 ? "adi_x" : "adi_y", s, lo, hi);
        }
        xy_done = done;
      }
    }
  }
  if (pred_done != nz + 1) return fail(h, NS_ERR_ARG, "internal: predictor planes left after the last slab");
  if (cn) {
    NS_CUDA(h, cudaEventRecord(h->ev_slab[ev_sweeps], h->side));
    NS_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_slab[ev_sweeps], 0));
  }
  if (hxo || hyo || hzo) trace_mark(h, h->xfer, "d2h history");
  int st = slab_tail ? enqueue_viscous(h, cn) : enqueue_tail(h, cn);
  if (st) return st;
  trace_mark(h, h->stream, slab_tail ? "viscous" : "tail");
  if (slab_tail) {
    st = step_host_slab_tail(h, tb, uo, vo, wo, po, ev_tail);
    if (st) return st;
  } else {
    for (int q = 0; q < 4; ++q)
      if (out[q])
        NS_CUDA(h, out_planes(h, out_dev[q], out[q], q, 0, nz + 2, h->stage_f[q], false, h->ev_slab[ev_tail + q]));
    trace_mark(h, h->xfer, "d2h state");
  }
  NS_CUDA(h, cudaStreamSynchronize(h->xfer));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  trace_flush(h);
  h->first_pending = false;
  h->steps = 1;
  return NS_OK;
}

int ns_set_faces(ns_handle* h, int set, const double* const faces[24]) {
  if (!h || set < 0 || set > 3 || !faces) return fail(h, NS_ERR_ARG, "set must be 0..3");
  // The 24 planes of a set are contiguous in face_buf: repack them into one
  // host buffer and send them with one stream-ordered copy (the copy from
  // pageable memory is staged before the call returns, so the buffer can be
  // reused).  Reference order: field-major (u, v, w, p), then x/y/z, then
  // low/high.
  const size_t base = face_offset(h->L, set, 0, 0, 0);
  size_t n_set = 0;
  for (int ax = 0; ax < 3; ++ax) n_set += 8 * plane_size(h->L, ax);
  h->face_host.assign(n_set, 0.0);
  bool any = false;
  for (int fld = 0; fld < 4; ++fld)
    for (int ax = 0; ax < 3; ++ax)
      for (int side = 0; side < 2; ++side) {
        const double* src = faces[fld * 6 + ax * 2 + side];
        if (!src) continue;
        face_to_plane(h->cfg, h->L, ax, fld, src, h->face_host.data() + (face_offset(h->L, set, ax, fld, side) - base));
        any = true;
      }
  NS_CUDA(h, cudaMemcpyAsync(h->face_buf + base, h->face_host.data(), n_set * sizeof(double), cudaMemcpyHostToDevice,
                             h->stream));
  // The captured step reads the faces from fixed device addresses; only a
  // change between all-zero (null face arguments) and given faces needs a new graph.
  if (h->face_set_nonzero[set] != any && h->graph) {
    NS_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  h->face_set_nonzero[set] = any;
  return NS_OK;
}

int ns_set_mean_dp(ns_handle* h, double mean_dp) {
  if (!h) return NS_ERR_ARG;
  h->cfg.mean_dp = mean_dp;
  if (h->mean_dev)
    NS_CUDA(h, cudaMemcpyAsync(h->mean_dev, &h->cfg.mean_dp, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  return NS_OK;
}

int ns_step(ns_handle* h, int nsteps) {
  if (!h || nsteps < 0) return NS_ERR_ARG;
  for (int it = 0; it < nsteps; ++it) {
    const bool first = h->first_pending && h->cfg.scheme != NS_EULER;
    if (first || !h->cfg.use_graph || !h->eager_done) {
      // Eager launch.  The first steady step also runs eagerly so that every
      // kernel's attributes are set before the step is captured.
      int s = enqueue_step(h, first);
      if (s) return s;
      if (!first) h->eager_done = true;
    } else {
      if (!h->graph) {
        // Capture on the handle's private stream (the caller's stream may be
        // the legacy default stream, which cannot be captured); the graph is
        // then replayed on the caller's stream.
        cudaGraph_t g = nullptr;
        NS_CUDA(h, cudaStreamSynchronize(h->stream));
        cudaStream_t user = h->stream;
        h->stream = h->cap_stream;
        cudaError_t eb = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (eb != cudaSuccess) { h->stream = user; return fail(h, NS_ERR_CUDA, cudaGetErrorString(eb)); }
        const long long before = h->launches;
        const int s = enqueue_step(h, false);
        h->graph_launches = h->launches - before;
        h->launches = before;
        const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        h->stream = user;
        if (s) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) return fail(h, NS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        const cudaError_t e2 = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) return fail(h, NS_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e2));
      }
      NS_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
      h->launches += h->graph_launches;
    }
    h->first_pending = false;
    h->steps++;
  }
  return NS_OK;
}

int ns_launch_count(const ns_handle* h, long long* launches) {
  if (!h || !launches) return NS_ERR_ARG;
  *launches = h->launches;
  return NS_OK;
}

int ns_profile(ns_handle* h, int nsteps, ns_kernel_time* out, int max_out, int* n_out) {
  if (!h || !out || !n_out || nsteps < 1 || max_out < 1) return NS_ERR_ARG;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  cudaEvent_t start;
  NS_CUDA(h, cudaEventCreate(&start));
  NS_CUDA(h, cudaEventRecord(start, h->stream));
  h->profiling = true;
  int s = NS_OK;
  for (int it = 0; it < nsteps && s == NS_OK; ++it) {
    const bool first = h->first_pending && h->cfg.scheme != NS_EULER;
    s = enqueue_step(h, first);
    h->first_pending = false;
    h->steps++;
  }
  h->profiling = false;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  int n = 0;
  cudaEvent_t prev = start;
  for (auto& pe : h->prof_events) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, prev, pe.second);
    int slot = -1;
    for (int q = 0; q < n; ++q)
      if (pe.first == out[q].name) slot = q;
    if (slot < 0 && n < max_out) {
      slot = n++;
      std::memset(&out[slot], 0, sizeof(out[slot]));
      std::strncpy(out[slot].name, pe.first.c_str(), sizeof(out[slot].name) - 1);
    }
    if (slot >= 0) {
      out[slot].ms += ms;
      out[slot].launches += 1;
    }
    prev = pe.second;
  }
  for (auto& pe : h->prof_events) cudaEventDestroy(pe.second);
  h->prof_events.clear();
  cudaEventDestroy(start);
  *n_out = n;
  if (s) return s;
  if (e != cudaSuccess) return fail(h, NS_ERR_CUDA, cudaGetErrorString(e));
  return NS_OK;
}

int ns_get_diag(ns_handle* h, ns_diag* d) {
  if (!h || !d) return NS_ERR_ARG;
  NS_CUDA(h, launch_diag(h->L, h->u, h->v, h->w, 1.0 / h->dx, 1.0 / h->dy, 1.0 / h->dz, h->diag_bits, h->stream));
  unsigned long long bits = 0;
  double probe = 0;
  NS_CUDA(h, cudaMemcpyAsync(&bits, h->diag_bits, sizeof(bits), cudaMemcpyDeviceToHost, h->stream));
  const ns_config& c = h->cfg;
  // u(nx/2, ny/2, nz/2) in Fortran indices -> slot (nx/2, ny/2-1, nz/2-1)
  const long long g = h->L.at(c.nx / 2, c.ny / 2 - 1, c.nz / 2 - 1);
  NS_CUDA(h, cudaMemcpyAsync(&probe, h->u + g, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int timed_out = 0;
  NS_CUDA(h, cudaMemcpyAsync(&timed_out, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  double md;
  std::memcpy(&md, &bits, sizeof(md));
  d->max_div = md;
  d->probe = probe;
  d->steps_done = h->steps;
  d->euler_start_pending = h->first_pending ? 1 : 0;
  d->reserved = 0;
  if (timed_out) return fail(h, NS_ERR_TIMEOUT, "a tile-loader wait of the predictor gave up; the state is invalid");
  if (!std::isfinite(md)) return fail(h, NS_ERR_NONFINITE, "non-finite divergence");
  return NS_OK;
}

// x[e] -= *g over a reference-shaped array (the gauge shift dp - dp(1,1,1),
// big_periodic_3D.f90:562, applied to an exported copy).
static __global__ void gauge_shift_kernel(double* __restrict__ x, long long n, const double* __restrict__ g) {
  const double g0 = *g;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    x[e] = __dsub_rn(x[e], g0);
}

int ns_get_stage(ns_handle* h, double* us, double* vs, double* ws, double* dp) {
  if (!h) return NS_ERR_ARG;
  if (h->steps == 0) return fail(h, NS_ERR_ARG, "no step taken since ns_set_state: no u* or dp to return");
  const ns_config& c = h->cfg;
  const bool cn = c.scheme == NS_AB2_CN;
  double* const dst[3] = {us, vs, ws};
  const double* src[3] = {cn ? h->us2 : h->us, cn ? h->vs2 : h->vs, cn ? h->ws2 : h->ws};
  for (int f = 0; f < 3; ++f)
    if (dst[f]) NS_CUDA(h, d2h_field(h, dst[f], src[f], f));
  if (dp) {
    NS_CUDA(h, ensure_stage(h));
    NS_CUDA(h, pack_launch(h, h->dp, h->stage, 3, false));
    const long long n = (long long)(c.nx + 2) * (c.ny + 2) * (c.nz + 2);
    if (c.gauge) {
      gauge_shift_kernel<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, h->stream>>>(
          h->stage, n, h->dp + h->L.at(0, 0, 0));
      NS_CUDA(h, cudaGetLastError());
      ++h->launches;
    }
    NS_CUDA(h, cudaMemcpyAsync(dp, h->stage, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  }
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int ns_get_sweeps(ns_handle* h, double* ux, double* vx, double* wx, double* uy, double* vy, double* wy) {
  if (!h) return NS_ERR_ARG;
  if (!h->us3) return fail(h, NS_ERR_ARG, "ns_get_sweeps needs an AB2-CN session created with keep_sweeps = 1");
  if (h->steps == 0) return fail(h, NS_ERR_ARG, "no step taken since ns_set_state");
  double* const dst[6] = {ux, vx, wx, uy, vy, wy};
  const double* src[6] = {h->us3, h->vs3, h->ws3, h->us, h->vs, h->ws};
  for (int q = 0; q < 6; ++q)
    if (dst[q]) NS_CUDA(h, d2h_field(h, dst[q], src[q], q % 3));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

// ---------------------------------------------------------------------------
// Routine tier
// ---------------------------------------------------------------------------
static int routine_conv_diff(ns_handle* h, const double* u, const double* v, const double* w, double* ox, double* oy,
                             double* oz, int mode) {
  if (!h || !u || !v || !w || !ox || !oy || !oz) return NS_ERR_ARG;
  const ns_config& c = h->cfg;
  // stage the inputs through the state buffers (the session state is saved around the call)
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<double*> save = {h->u, h->v, h->w};
  double *tu = nullptr, *tv = nullptr, *tw = nullptr;
  NS_CUDA(h, cudaMalloc(&tu, h->L.fsize * sizeof(double)));
  NS_CUDA(h, cudaMalloc(&tv, h->L.fsize * sizeof(double)));
  NS_CUDA(h, cudaMalloc(&tw, h->L.fsize * sizeof(double)));
  NS_CUDA(h, cudaMemsetAsync(tu, 0, h->L.fsize * sizeof(double), h->stream));
  NS_CUDA(h, cudaMemsetAsync(tv, 0, h->L.fsize * sizeof(double), h->stream));
  NS_CUDA(h, cudaMemsetAsync(tw, 0, h->L.fsize * sizeof(double), h->stream));
  NS_CUDA(h, h2d_field(h, tu, u, 0));
  NS_CUDA(h, h2d_field(h, tv, v, 1));
  NS_CUDA(h, h2d_field(h, tw, w, 2));
  // the extra periodic face slot mirrors face n
  NS_CUDA(h, launch_extra_slots(h->L, tu, tv, tw, c.bc, h->stream));
  PredictArgs a = predict_args(h);
  a.u = tu; a.v = tv; a.w = tw;
  NS_CUDA(h, launch_predict(a, 0, false, false, mode, h->stream));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  // gather the interior ranges into the reference shapes
  double* outs[3] = {ox, oy, oz};
  double* srcs[3] = {h->us, h->vs, h->ws};
  for (int f = 0; f < 3; ++f) {
    std::vector<double> full(h->L.fsize);
    NS_CUDA(h, cudaMemcpyAsync(full.data(), srcs[f], h->L.fsize * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    NS_CUDA(h, cudaStreamSynchronize(h->stream));
    const int ex = (c.bc[0] == 1 || f != 0) ? c.nx : c.nx - 1;
    const int ey = (c.bc[1] == 1 || f != 1) ? c.ny : c.ny - 1;
    const int ez = (c.bc[2] == 1 || f != 2) ? c.nz : c.nz - 1;
    const int x0 = (f == 0 && c.bc[0] != 1) ? 2 : 1;
    const int y0 = (f == 1 && c.bc[1] != 1) ? 2 : 1;
    const int z0 = (f == 2 && c.bc[2] != 1) ? 2 : 1;
    for (int k = 0; k < ez; ++k)
      for (int j = 0; j < ey; ++j)
        for (int i = 0; i < ex; ++i)
          outs[f][i + (size_t)ex * (j + (size_t)ey * k)] = full[h->L.at(x0 + i, y0 + j, z0 + k)];
  }
  cudaFree(tu); cudaFree(tv); cudaFree(tw);
  (void)save;
  return NS_OK;
}

int ns_cal_conv(ns_handle* h, const double* u, const double* v, const double* w, double* cx, double* cy, double* cz) {
  return routine_conv_diff(h, u, v, w, cx, cy, cz, 1);
}

int ns_cal_diff(ns_handle* h, const double* u, const double* v, const double* w, double* dx, double* dy, double* dz) {
  return routine_conv_diff(h, u, v, w, dx, dy, dz, 2);
}

int ns_poisson(ns_handle* h, const double* rhs, double* dp) {
  if (!h || !rhs || !dp) return NS_ERR_ARG;
  const ns_config& c = h->cfg;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  // Stage rhs into the cell slots of the dp buffer, then transform it.
  std::vector<double> full((size_t)h->L.fsize, 0.0);
  for (int k = 0; k < c.nz; ++k)
    for (int j = 0; j < c.ny; ++j)
      for (int i = 0; i < c.nx; ++i)
        full[h->L.at(i + 1, j + 1, k + 1)] = rhs[i + (size_t)c.nx * (j + (size_t)c.ny * k)];
  NS_CUDA(h, cudaMemcpyAsync(h->us, full.data(), full.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int s = enqueue_poisson(h, h->us);
  if (s) return s;
  NS_CUDA(h, d2h_field(h, dp, h->dp, 3));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int ns_adi(ns_handle* h, double* u_star, double* v_star, double* w_star) {
  if (!h || !u_star || !v_star || !w_star) return NS_ERR_ARG;
  if (h->cfg.scheme != NS_AB2_CN) return fail(h, NS_ERR_ARG, "ns_adi needs scheme AB2-CN (factors are built for it)");
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  NS_CUDA(h, h2d_field(h, h->us, u_star, 0));
  NS_CUDA(h, h2d_field(h, h->vs, v_star, 1));
  NS_CUDA(h, h2d_field(h, h->ws, w_star, 2));
  int s = enqueue_adi(h);
  if (s) return s;
  NS_CUDA(h, d2h_field(h, u_star, h->us2, 0));
  NS_CUDA(h, d2h_field(h, v_star, h->vs2, 1));
  NS_CUDA(h, d2h_field(h, w_star, h->ws2, 2));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int ns_vel_bc(ns_handle* h, double* u_star, double* v_star, double* w_star) {
  if (!h || !u_star || !v_star || !w_star) return NS_ERR_ARG;
  const ns_config& c = h->cfg;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  NS_CUDA(h, h2d_field(h, h->us, u_star, 0));
  NS_CUDA(h, h2d_field(h, h->vs, v_star, 1));
  NS_CUDA(h, h2d_field(h, h->ws, w_star, 2));
  NS_CUDA(h, launch_vel_bc(h->L, h->us, h->vs, h->ws, h->faces[0], c.bc, h->stream));
  NS_CUDA(h, d2h_field(h, u_star, h->us, 0));
  NS_CUDA(h, d2h_field(h, v_star, h->vs, 1));
  NS_CUDA(h, d2h_field(h, w_star, h->ws, 2));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

int ns_correct(ns_handle* h, const double* u_star, const double* v_star, const double* w_star, const double* dp,
               double* u, double* v, double* w, double* p) {
  if (!h || !u_star || !v_star || !w_star || !dp || !u || !v || !w || !p) return NS_ERR_ARG;
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  struct DevBuf {
    double* ptr = nullptr;
    ~DevBuf() { if (ptr) cudaFree(ptr); }
  } pt;
  NS_CUDA(h, cudaMalloc(&pt.ptr, h->L.fsize * sizeof(double)));
  NS_CUDA(h, cudaMemsetAsync(pt.ptr, 0, h->L.fsize * sizeof(double), h->stream));
  NS_CUDA(h, h2d_field(h, h->us, u_star, 0));
  NS_CUDA(h, h2d_field(h, h->vs, v_star, 1));
  NS_CUDA(h, h2d_field(h, h->ws, w_star, 2));
  NS_CUDA(h, h2d_field(h, h->dp, dp, 3));
  NS_CUDA(h, h2d_field(h, pt.ptr, p, 3));
  CorrectArgs ca = correct_args(h);
  ca.us = h->us; ca.vs = h->vs; ca.ws = h->ws; ca.dp = h->dp;
  ca.u = h->us2; ca.v = h->vs2; ca.w = h->ws2; ca.p = pt.ptr;
  NS_CUDA(h, launch_correct(ca, h->stream));
  NS_CUDA(h, d2h_field(h, u, h->us2, 0));
  NS_CUDA(h, d2h_field(h, v, h->vs2, 1));
  NS_CUDA(h, d2h_field(h, w, h->ws2, 2));
  NS_CUDA(h, d2h_field(h, p, pt.ptr, 3));
  NS_CUDA(h, cudaStreamSynchronize(h->stream));
  return NS_OK;
}

}  // extern "C"
