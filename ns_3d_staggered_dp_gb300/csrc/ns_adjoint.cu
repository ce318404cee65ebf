// Discrete adjoint of the periodic FP64 staggered step (AB2-CN, AB2, Euler;
// dp_flag = 0): the transpose of the tangent-linear model of one step of
// big_periodic_3D.f90:326-567, operator by operator.
//
// Forward step (slot form, C = -conv, g the step's coefficients):
//   u*  = c0 u + ca (u[i-1] + u[i+1]) + cb (..) + cc (..) + cC C(u) + cP h    (AB2-CN)
//   h'  = C(u)
//   u'  = P A^-1 u*,   A^-1 = Az^-1 Ay^-1 Ax^-1 (CN-ADI),  P = I - G L^+ D
// Backward step, given the adjoint l of u' and the adjoint m of h':
//   la  = P l                                  (P is symmetric: D = -G^T)
//   ls  = Ax^-T Ay^-T Az^-T la                 (transposed line systems, sweeps z, y, x)
//   g   = cC ls + m,   m = cP ls_next          (ls of the following step; 0 after the last)
//   l_u = c0 ls + ca (ls[i-1] + ls[i+1]) + .. + C'(u)^T g
//   m_h = cP ls                                (kept as ls_next of the previous step)
// AB2 / Euler: no ADI, g = e1 ls + m weights rhs = nu lap u + C, and
// l_u = ls + (nu lap)^T g + C'(u)^T g.
//
// C'(u)^T g, from C = -(cal_conv) (NS_functions.f90:53-158) written with
// SX(c) = u(c) + u(c+1) and QXY(i,J) = (u(i,J-1) + u(i,J)) (v(i-1,J) + v(i,J))
// (x-face i, y-face J), and likewise SY, SZ, QXZ, QYZ.  With ax = -1/(4dx):
//   weight of SX(c)^2:  ax (gx(c) - gx(c+1))
//   weight of QXY(i,J): ay (gx(i,J-1) - gx(i,J)) + ax (gy(i-1,J) - gy(i,J))
// then each product's weight times the other factor goes back to the two
// points of its sum: u(i) gets PX(i-1) + PX(i) (PX = 2 SX * weight),
// XYu(i,j) + XYu(i,j+1) (XYu = weight(QXY) * Vx), XZu(k) + XZu(k+1); v gets
// PY, XYv (x-faces i, i+1), YZv (z-faces k, k+1); w gets PZ, XZw, YZw.
//
// Tiling of adj_predict: a CTA owns 32 x-slots by 8 y-slots and marches
// along z.  Product positions are 33 x 9 per plane, one warp per row (the
// 33rd column by one extra pass of the last warp, lanes 0..8): the
// position (a, b) owns PX of cell a-1, PY of cell b-1, the XY edge at faces
// (a, b), the XZ edge at (x-face a, z-face K), the YZ edge at (y-face b,
// z-face K), and PZ of cell K-1.  An output at (i, j, k) then reads positions
// i, i+1 and j, j+1 only, and z-faces k, k+1 (a ring of two product planes).
// Inputs (the weights g and the forward u, v, w) are staged with a one-slot
// halo in a ring of two planes.  The Laplacian part reads ls through L1.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"
#include "ns_session.cuh"

namespace ns {

struct AdjArgs {
  Layout L;
  const double* ls[3];  // adjoint of u*, v*, w* (slots 0..n+1 hold periodic images)
  const double* ln[3];  // ls of the following step (unused when HAS_NEXT is false)
  const double* f[3];   // forward u, v, w at the start of the step
  double* out[3];       // adjoint of u, v, w: slots 1..n written
  double one, mzero;
  double wS, wN;        // g = wS ls + wN ln
  double ax, ay, az;    // -1/(4 dx) etc.
  double ax2, ay2, az2; // 2 ax etc.
  double l0, lx, ly, lz;  // Laplacian part: l0 X + lx (X[i-1] + X[i+1]) + ...
  int kc;               // z planes per CTA (set by the launcher)
};

namespace {

constexpr int AX = 32;       // output x-slots per row
constexpr int AY = 8;        // output rows
constexpr int IW = AX + 2;   // staged input row: x in [i0-1, i0+AX]
constexpr int IH = AY + 2;   // staged input rows: y in [j0-1, j0+AY]
constexpr int PW = AX + 1;   // product positions per row: x in [i0, i0+AX]
constexpr int PH = AY + 1;   // product rows: y in [j0, j0+AY]

struct AdjSmem {
  double g[3][2][IH][IW];  // weights, ring of planes (parity)
  double f[3][2][IH][IW];  // forward u, v, w
  double px[PH][PW], py[PH][PW], xyu[PH][PW], xyv[PH][PW];  // plane k
  double pz[2][PH][PW], xzu[2][PH][PW], xzw[2][PH][PW], yzv[2][PH][PW], yzw[2][PH][PW];  // z-faces k, k+1
};

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

template <bool HAS_NEXT>
__device__ __forceinline__ void adj_load_plane(AdjSmem& S, const AdjArgs& a, const FOne& c, int i0, int j0, int k) {
  const Layout& L = a.L;
  const int kk = clampi(k, 0, L.nz + 1);
  const int s = k & 1;
  const int nthr = blockDim.x * blockDim.y;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int e = tid; e < IW * IH; e += nthr) {
    const int xx = e % IW, yy = e / IW;
    const int gi = clampi(i0 - 1 + xx, 0, L.nx + 1);
    const int gj = clampi(j0 - 1 + yy, 0, L.ny + 1);
    const long long gg = L.at(gi, gj, kk);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double l = __ldg(a.ls[q] + gg);
      S.g[q][s][yy][xx] = HAS_NEXT ? fma(a.wN, __ldg(a.ln[q] + gg), fmul(c, a.wS, l)) : fmul(c, a.wS, l);
      S.f[q][s][yy][xx] = __ldg(a.f[q] + gg);
    }
  }
}

// Products of position (pa, pb) that live on plane k (cell products PX, PY
// and the XY edge), from ring slot s.
__device__ __forceinline__ void adj_products_xy(AdjSmem& S, const AdjArgs& a, const FOne& c, int pa, int pb, int s) {
  const int x = pa + 1, y = pb + 1;  // staged coordinates of the position
  const double (*gx)[IW] = S.g[0][s];
  const double (*gy)[IW] = S.g[1][s];
  const double (*U)[IW] = S.f[0][s];
  const double (*V)[IW] = S.f[1][s];
  // PX of x-cell a-1: 2 SX * ax (gx(a-1) - gx(a))
  const double sx = fadd(c, U[y][x - 1], U[y][x]);
  S.px[pb][pa] = fmul(c, sx, fmul(c, a.ax2, fsub(c, gx[y][x - 1], gx[y][x])));
  // PY of y-cell b-1
  const double sy = fadd(c, V[y - 1][x], V[y][x]);
  S.py[pb][pa] = fmul(c, sy, fmul(c, a.ay2, fsub(c, gy[y - 1][x], gy[y][x])));
  // XY edge at (x-face a, y-face b)
  double A = fmul(c, a.ay, fsub(c, gx[y - 1][x], gx[y][x]));
  A = fma(a.ax, fsub(c, gy[y][x - 1], gy[y][x]), A);
  S.xyu[pb][pa] = fmul(c, A, fadd(c, V[y][x - 1], V[y][x]));
  S.xyv[pb][pa] = fmul(c, A, fadd(c, U[y - 1][x], U[y][x]));
}

// Products on z-face K (PZ of cell K-1, the XZ and YZ edges) from ring
// slots s0 (plane K-1) and s1 (plane K), into product slot K & 1.
__device__ __forceinline__ void adj_products_z(AdjSmem& S, const AdjArgs& a, const FOne& c, int pa, int pb, int s0,
                                               int s1, int ps) {
  const int x = pa + 1, y = pb + 1;
  const double (*gx0)[IW] = S.g[0][s0];
  const double (*gx1)[IW] = S.g[0][s1];
  const double (*gy0)[IW] = S.g[1][s0];
  const double (*gy1)[IW] = S.g[1][s1];
  const double (*gz0)[IW] = S.g[2][s0];
  const double (*gz1)[IW] = S.g[2][s1];
  const double (*U0)[IW] = S.f[0][s0];
  const double (*U1)[IW] = S.f[0][s1];
  const double (*V0)[IW] = S.f[1][s0];
  const double (*V1)[IW] = S.f[1][s1];
  const double (*W0)[IW] = S.f[2][s0];
  const double (*W1)[IW] = S.f[2][s1];
  // PZ of z-cell K-1
  const double sz = fadd(c, W0[y][x], W1[y][x]);
  S.pz[ps][pb][pa] = fmul(c, sz, fmul(c, a.az2, fsub(c, gz0[y][x], gz1[y][x])));
  // XZ edge at (x-face a, z-face K)
  double A = fmul(c, a.az, fsub(c, gx0[y][x], gx1[y][x]));
  A = fma(a.ax, fsub(c, gz1[y][x - 1], gz1[y][x]), A);
  S.xzu[ps][pb][pa] = fmul(c, A, fadd(c, W1[y][x - 1], W1[y][x]));
  S.xzw[ps][pb][pa] = fmul(c, A, fadd(c, U0[y][x], U1[y][x]));
  // YZ edge at (y-face b, z-face K)
  double B = fmul(c, a.az, fsub(c, gy0[y][x], gy1[y][x]));
  B = fma(a.ay, fsub(c, gz1[y - 1][x], gz1[y][x]), B);
  S.yzv[ps][pb][pa] = fmul(c, B, fadd(c, W1[y - 1][x], W1[y][x]));
  S.yzw[ps][pb][pa] = fmul(c, B, fadd(c, V0[y][x], V1[y][x]));
}

// Laplacian part at slot g of component q: LAPG false -> X = ls (AB2-CN),
// true -> X = g = wS ls + wN ln, plus ls itself (AB2, Euler).
template <bool LAPG, bool HAS_NEXT>
__device__ __forceinline__ double adj_lap(const AdjArgs& a, const FOne& c, int q, long long g) {
  const Layout& L = a.L;
  const double* __restrict__ X = a.ls[q];
  const double* __restrict__ N = a.ln[q];
  auto val = [&](long long o) {
    const double l = __ldg(X + o);
    if (!LAPG) return l;
    return HAS_NEXT ? fma(a.wN, __ldg(N + o), fmul(c, a.wS, l)) : fmul(c, a.wS, l);
  };
  double t = fmul(c, a.l0, val(g));
  t = fma(a.lx, fadd(c, val(g - 1), val(g + 1)), t);
  t = fma(a.ly, fadd(c, val(g - L.sy), val(g + L.sy)), t);
  t = fma(a.lz, fadd(c, val(g - L.sz), val(g + L.sz)), t);
  if (LAPG) t = fadd(c, t, __ldg(X + g));
  return t;
}

}  // namespace

template <bool LAPG, bool HAS_NEXT>
__global__ void __launch_bounds__(32 * PH, 3) adj_predict_kernel(AdjArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  AdjSmem& S = *reinterpret_cast<AdjSmem*>(smem_raw);
  const Layout L = a.L;
  const FOne c{a.one, a.mzero};
  const int lane = threadIdx.x, wy = threadIdx.y;  // position (lane, wy)
  const int i0 = 1 + AX * blockIdx.x;
  const int j0 = 1 + AY * blockIdx.y;
  const int k0 = 1 + a.kc * blockIdx.z;
  const int k1 = min(k0 + a.kc, L.nz + 1);
  // warm-up: planes k0-1, k0 and the z-face products at k0
  adj_load_plane<HAS_NEXT>(S, a, c, i0, j0, k0 - 1);
  adj_load_plane<HAS_NEXT>(S, a, c, i0, j0, k0);
  __syncthreads();
  adj_products_z(S, a, c, lane, wy, (k0 - 1) & 1, k0 & 1, k0 & 1);
  const bool extra = wy == PH - 1 && lane < PH;  // column AX of row `lane`
  if (extra) adj_products_z(S, a, c, AX, lane, (k0 - 1) & 1, k0 & 1, k0 & 1);
  const int i = i0 + lane, j = j0 + wy;
  const bool out_ok = lane < AX && wy < AY && i <= L.nx && j <= L.ny;
  for (int k = k0; k < k1; ++k) {
    __syncthreads();  // previous outputs done with plane k-1's ring slot
    adj_load_plane<HAS_NEXT>(S, a, c, i0, j0, k + 1);
    __syncthreads();
    adj_products_xy(S, a, c, lane, wy, k & 1);
    adj_products_z(S, a, c, lane, wy, k & 1, (k + 1) & 1, (k + 1) & 1);
    if (extra) {
      adj_products_xy(S, a, c, AX, lane, k & 1);
      adj_products_z(S, a, c, AX, lane, k & 1, (k + 1) & 1, (k + 1) & 1);
    }
    __syncthreads();
    if (out_ok) {
      const long long g = L.at(i, j, k);
      const int p0 = k & 1, p1 = (k + 1) & 1;
      const int pa = lane, pb = wy;
      double u = fadd(c, S.px[pb][pa], S.px[pb][pa + 1]);
      u = fadd(c, u, fadd(c, S.xyu[pb][pa], S.xyu[pb + 1][pa]));
      u = fadd(c, u, fadd(c, S.xzu[p0][pb][pa], S.xzu[p1][pb][pa]));
      a.out[0][g] = fadd(c, u, adj_lap<LAPG, HAS_NEXT>(a, c, 0, g));
      double v = fadd(c, S.py[pb][pa], S.py[pb + 1][pa]);
      v = fadd(c, v, fadd(c, S.xyv[pb][pa], S.xyv[pb][pa + 1]));
      v = fadd(c, v, fadd(c, S.yzv[p0][pb][pa], S.yzv[p1][pb][pa]));
      a.out[1][g] = fadd(c, v, adj_lap<LAPG, HAS_NEXT>(a, c, 1, g));
      double w = fadd(c, S.pz[p0][pb][pa], S.pz[p1][pb][pa]);
      w = fadd(c, w, fadd(c, S.xzw[p0][pb][pa], S.xzw[p0][pb][pa + 1]));
      w = fadd(c, w, fadd(c, S.yzw[p0][pb][pa], S.yzw[p0][pb + 1][pa]));
      a.out[2][g] = fadd(c, w, adj_lap<LAPG, HAS_NEXT>(a, c, 2, g));
    }
  }
}

// z-chunk length: the number of chunks c that minimises the time of the
// grid in waves of resident CTAs, ceil(cols c / slots) * (ceil(nz / c) + 2),
// where the 2 stands for a chunk's warm-up (two planes loaded, one plane of
// products).  At 128^3 this gives 7 chunks of 19 planes (448 CTAs on 456
// slots) instead of 8 chunks (512 CTAs, 1.12 waves).
static int adj_chunk(int cols, int nz, int slots) {
  int best = nz;
  double best_t = 1e300;
  for (int c = 1; c <= nz; ++c) {
    const int kc = (nz + c - 1) / c;
    const int cc = (nz + kc - 1) / kc;  // chunks actually launched
    const double waves = std::ceil((double)cols * cc / slots);
    const double t = waves * (kc + 2);
    if (t < best_t - 1e-9) { best_t = t; best = kc; }
  }
  return best;
}

template <bool LAPG, bool HAS_NEXT>
static cudaError_t launch_adj_t(AdjArgs a, cudaStream_t st) {
  auto kern = adj_predict_kernel<LAPG, HAS_NEXT>;
  const size_t sm = sizeof(AdjSmem);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * PH, sm)) != cudaSuccess) return e;
  const int gx = (a.L.nx + AX - 1) / AX, gy = (a.L.ny + AY - 1) / AY;
  a.kc = adj_chunk(gx * gy, a.L.nz, std::max(1, per_sm) * std::max(1, nsm));
  dim3 grid(gx, gy, (a.L.nz + a.kc - 1) / a.kc);
  kern<<<grid, dim3(32, PH), sm, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adj_predict(const AdjArgs& a, bool lap_of_g, bool has_next, cudaStream_t st) {
  if (lap_of_g) return has_next ? launch_adj_t<true, true>(a, st) : launch_adj_t<true, false>(a, st);
  return has_next ? launch_adj_t<false, true>(a, st) : launch_adj_t<false, false>(a, st);
}

// Periodic images along AXIS of the three fields: X[0] = X[n], X[n+1] = X[1]
// over the full extent of the other two axes (ghosts included), so three
// passes x, y, z leave every ghost slot consistent.
template <int AXIS>
__global__ void __launch_bounds__(256) periodic_fill_kernel(Layout L, double* f0, double* f1, double* f2) {
  const int n1 = (AXIS == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (AXIS == 2) ? L.ny + 2 : L.nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  const int s1 = t % n1, s2 = t / n1;
  long long base, st;
  int n;
  if (AXIS == 0) { base = L.at(0, s1, s2); st = 1; n = L.nx; }
  else if (AXIS == 1) { base = L.at(s1, 0, s2); st = L.sy; n = L.ny; }
  else { base = L.at(s1, s2, 0); st = L.sz; n = L.nz; }
  double* f[3] = {f0, f1, f2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    double* x = f[q] + base;
    x[0] = x[(long long)n * st];
    x[(long long)(n + 1) * st] = x[st];
  }
}

// Transpose of the periodic images along AXIS (FOLD): X[n] += X[0],
// X[1] += X[n+1], then both ghosts zeroed; or (!FOLD) the ghosts zeroed
// only.  Three passes x, y, z carry a corner entry to its owner in hops.
template <int AXIS, bool FOLD>
__global__ void __launch_bounds__(256) periodic_fold_kernel(Layout L, double* f0, double* f1, double* f2) {
  const int n1 = (AXIS == 0) ? L.ny + 2 : L.nx + 2;
  const int n2 = (AXIS == 2) ? L.ny + 2 : L.nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  const int s1 = t % n1, s2 = t / n1;
  long long base, st;
  int n;
  if (AXIS == 0) { base = L.at(0, s1, s2); st = 1; n = L.nx; }
  else if (AXIS == 1) { base = L.at(s1, 0, s2); st = L.sy; n = L.ny; }
  else { base = L.at(s1, s2, 0); st = L.sz; n = L.nz; }
  double* f[3] = {f0, f1, f2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    double* x = f[q] + base;
    double* hi = x + (long long)(n + 1) * st;
    if (FOLD) {
      x[(long long)n * st] += x[0];
      x[st] += *hi;
    }
    x[0] = 0.0;
    *hi = 0.0;
  }
}

cudaError_t launch_periodic_fold(const Layout& L, double* f0, double* f1, double* f2, bool fold, cudaStream_t st) {
  for (int a = 0; a < 3; ++a) {
    const int n = plane_count(L, a);
    const dim3 grid((n + 255) / 256);
    if (a == 0) fold ? periodic_fold_kernel<0, true><<<grid, 256, 0, st>>>(L, f0, f1, f2)
                     : periodic_fold_kernel<0, false><<<grid, 256, 0, st>>>(L, f0, f1, f2);
    if (a == 1) fold ? periodic_fold_kernel<1, true><<<grid, 256, 0, st>>>(L, f0, f1, f2)
                     : periodic_fold_kernel<1, false><<<grid, 256, 0, st>>>(L, f0, f1, f2);
    if (a == 2) fold ? periodic_fold_kernel<2, true><<<grid, 256, 0, st>>>(L, f0, f1, f2)
                     : periodic_fold_kernel<2, false><<<grid, 256, 0, st>>>(L, f0, f1, f2);
  }
  return cudaGetLastError();
}

cudaError_t launch_periodic_fill(const Layout& L, double* f0, double* f1, double* f2, cudaStream_t st) {
  for (int a = 0; a < 3; ++a) {
    const int n = plane_count(L, a);
    const dim3 grid((n + 255) / 256);
    if (a == 0) periodic_fill_kernel<0><<<grid, 256, 0, st>>>(L, f0, f1, f2);
    if (a == 1) periodic_fill_kernel<1><<<grid, 256, 0, st>>>(L, f0, f1, f2);
    if (a == 2) periodic_fill_kernel<2><<<grid, 256, 0, st>>>(L, f0, f1, f2);
  }
  return cudaGetLastError();
}

}  // namespace ns

// ===========================================================================
// Host side: the adjoint tier of the C ABI.
// ===========================================================================
namespace ns {

struct AdjState {
  int nsteps = 0, ckpt = 0, nck = 0;
  bool ready = false;
  std::vector<double*> ck;    // nck x 6 fields: u, v, w, hx, hy, hz at steps 0, K, 2K, ...
  std::vector<int> ck_first;  // Euler start pending at each checkpoint
  double* fin[7] = {};        // state after the forward run: u, v, w, p, hx, hy, hz
  bool fin_first = false;
  long long fin_steps = 0;
  std::vector<double*> seg;   // K x 3 fields: u, v, w entering each step of a segment
  std::vector<int> seg_first;
  double* lam[3] = {};        // adjoint of u, v, w
  double* la[3] = {};         // projected adjoint
  double* ls[2][3] = {};      // adjoint of u*, v*, w*: ping-pong (this step / following step)
  int cur = 0;
  double* pscr = nullptr;     // p output of the adjoint projection (discarded)
  LineSys sys_t[3][3]{};      // transposed CN line systems (AB2-CN)
  double* sys_buf = nullptr;
};

namespace {

#define ADJ_CUDA(h, call)                                                                        \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return api_fail((h), NS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int adj_alloc(ns_handle* h, double** p) {
  if (cudaMalloc(p, h->L.fsize * sizeof(double)) != cudaSuccess) {
    *p = nullptr;
    return api_fail(h, NS_ERR_NOMEM, "adjoint: device allocation failed");
  }
  ADJ_CUDA(h, cudaMemsetAsync(*p, 0, h->L.fsize * sizeof(double), h->stream));
  return NS_OK;
}

void adj_free_vec(std::vector<double*>& v) {
  for (double* p : v)
    if (p) cudaFree(p);
  v.clear();
}

int adj_copy(ns_handle* h, double* dst, const double* src) {
  ADJ_CUDA(h, cudaMemcpyAsync(dst, src, h->L.fsize * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return NS_OK;
}

int adj_check_cfg(ns_handle* h) {
  const ns_config& c = h->cfg;
  for (int a = 0; a < 3; ++a)
    if (c.bc[a] != 1 || c.pbc[a] != 1)
      return api_fail(h, NS_ERR_UNSUPPORTED_BC, "adjoint: the triply periodic box only (bc = pbc = 1)");
  if (c.dp_flag != 0) return api_fail(h, NS_ERR_UNSUPPORTED_BC, "adjoint: dp_flag = 0 only");
  return NS_OK;
}

// Per-step work buffers, allocated once per handle.
int adj_ensure(ns_handle* h) {
  if (h->adj) return NS_OK;
  AdjState* A = new AdjState();
  h->adj = A;
  int s;
  for (int q = 0; q < 3; ++q) {
    if ((s = adj_alloc(h, &A->lam[q]))) return s;
    if ((s = adj_alloc(h, &A->la[q]))) return s;
    if ((s = adj_alloc(h, &A->ls[0][q]))) return s;
    if ((s = adj_alloc(h, &A->ls[1][q]))) return s;
  }
  if ((s = adj_alloc(h, &A->pscr))) return s;
  if (h->cfg.scheme == NS_AB2_CN && (s = api_build_line_tables(h, true, A->sys_t, &A->sys_buf))) return s;
  return NS_OK;
}

// Reference extent of field f (0 u, 1 v, 2 w) along axis a.
inline int ref_ext(const ns_config& c, int f, int a) {
  const int n = a == 0 ? c.nx : (a == 1 ? c.ny : c.nz);
  return f == a ? n + 1 : n + 2;
}

// Zero every entry that is a periodic copy (gradients are with respect to
// the independent values).
void zero_copies(const ns_config& c, int f, double* a) {
  const int ex = ref_ext(c, f, 0), ey = ref_ext(c, f, 1), ez = ref_ext(c, f, 2);
  const int n3[3] = {c.nx, c.ny, c.nz};
  auto own = [&](int r, int ax) {
    const bool face = f == ax;
    return face ? (r <= n3[ax] - 1) : (r >= 1 && r <= n3[ax]);
  };
  for (int k = 0; k < ez; ++k)
    for (int j = 0; j < ey; ++j)
      for (int i = 0; i < ex; ++i)
        if (!(own(i, 0) && own(j, 1) && own(k, 2))) a[i + (size_t)ex * (j + (size_t)ey * k)] = 0.0;
}

// One backward step over forward step n, whose input velocity is fwd[3].
int adj_backward_step(ns_handle* h, AdjState* A, double* const fwd[3], bool first, bool has_next) {
  const ns_config& c = h->cfg;
  const bool cn = c.scheme == NS_AB2_CN;
  double* const* cur = A->ls[A->cur];
  double* const* nxt = A->ls[1 - A->cur];
  // la = P lam: the forward projection applied to the adjoint
  DivArgs d{};
  d.L = h->L;
  d.us = A->lam[0]; d.vs = A->lam[1]; d.ws = A->lam[2];
  d.cdx = 1.0 / (h->dx * c.dt); d.cdy = 1.0 / (h->dy * c.dt); d.cdz = 1.0 / (h->dz * c.dt);
  d.one = 1.0; d.mzero = -0.0; d.rhs = nullptr;
  ADJ_CUDA(h, launch_fft_poisson(h->plan, d, h->spec, h->dp, h->L, h->stream, api_marker(h)));
  ADJ_CUDA(h, launch_pr_bc(h->L, h->dp, h->faces[0], c.pbc, h->dx, h->dy, h->dz, h->stream));
  api_mark(h, "adj_pr_bc", 3);
  CorrectArgs ca{};
  ca.L = h->L;
  ca.us = A->lam[0]; ca.vs = A->lam[1]; ca.ws = A->lam[2]; ca.dp = h->dp;
  double* const* pout = cn ? A->la : cur;
  ca.u = pout[0]; ca.v = pout[1]; ca.w = pout[2]; ca.p = A->pscr;
  ca.gx = -c.dt / h->dx; ca.gy = -c.dt / h->dy; ca.gz = -c.dt / h->dz;
  ca.dp_flag = 0; ca.gauge = 0;
  for (int q = 0; q < 3; ++q) ca.per[q] = 1;
  ca.one = 1.0; ca.mzero = -0.0;
  ADJ_CUDA(h, launch_correct(ca, h->stream));
  api_mark(h, "adj_correct", 1);
  // ls = Ax^-T Ay^-T Az^-T la: sweeps z (la -> lam), y (lam -> la), x (la -> cur)
  if (cn) {
    const int order[3] = {2, 1, 0};
    for (int st = 0; st < 3; ++st) {
      const int ax = order[st];
      AdiArgs a{};
      a.L = h->L;
      for (int f = 0; f < 3; ++f) {
        a.src[f] = st == 1 ? A->lam[f] : A->la[f];
        a.dst[f] = st == 0 ? A->lam[f] : (st == 1 ? A->la[f] : cur[f]);
        a.sys[f] = A->sys_t[ax][f];
        a.face_lo[f] = nullptr;
        a.face_hi[f] = nullptr;
      }
      ADJ_CUDA(h, launch_adi(ax, a, h->stream));
      api_mark(h, ax == 0 ? "adj_adi_x" : (ax == 1 ? "adj_adi_y" : "adj_adi_z"), 1);
    }
  }
  // l_u = (Laplacian part) + C'(u)^T g
  AdjArgs a{};
  a.L = h->L;
  for (int q = 0; q < 3; ++q) {
    a.ls[q] = cur[q];
    a.ln[q] = nxt[q];
    a.f[q] = fwd[q];
    a.out[q] = A->lam[q];
  }
  a.one = 1.0; a.mzero = -0.0;
  const double dt = c.dt, nu = c.nu;
  a.wS = (first || c.scheme == NS_EULER) ? dt : 1.5 * dt;
  a.wN = -0.5 * dt;
  a.ax = -0.25 / h->dx; a.ay = -0.25 / h->dy; a.az = -0.25 / h->dz;
  a.ax2 = 2.0 * a.ax; a.ay2 = 2.0 * a.ay; a.az2 = 2.0 * a.az;
  const double ix2 = 1.0 / (h->dx * h->dx), iy2 = 1.0 / (h->dy * h->dy), iz2 = 1.0 / (h->dz * h->dz);
  if (cn) {
    const double hnd = 0.5 * nu * dt;
    a.l0 = 1.0 - 2.0 * hnd * (ix2 + iy2 + iz2);
    a.lx = hnd * ix2; a.ly = hnd * iy2; a.lz = hnd * iz2;
  } else {
    a.l0 = -2.0 * nu * (ix2 + iy2 + iz2);
    a.lx = nu * ix2; a.ly = nu * iy2; a.lz = nu * iz2;
  }
  const bool next = has_next && c.scheme != NS_EULER;
  ADJ_CUDA(h, launch_adj_predict(a, !cn, next, h->stream));
  api_mark(h, "adj_predict", 1);
  ADJ_CUDA(h, launch_periodic_fill(h->L, A->lam[0], A->lam[1], A->lam[2], h->stream));
  api_mark(h, "adj_fill", 3);
  A->cur = 1 - A->cur;
  return NS_OK;
}

}  // namespace

void api_free_adjoint(ns_handle* h) {
  AdjState* A = h->adj;
  if (!A) return;
  adj_free_vec(A->ck);
  adj_free_vec(A->seg);
  for (double*& p : A->fin)
    if (p) { cudaFree(p); p = nullptr; }
  for (int q = 0; q < 3; ++q) {
    double* bufs[4] = {A->lam[q], A->la[q], A->ls[0][q], A->ls[1][q]};
    for (double* p : bufs)
      if (p) cudaFree(p);
  }
  if (A->pscr) cudaFree(A->pscr);
  if (A->sys_buf) cudaFree(A->sys_buf);
  delete A;
  h->adj = nullptr;
}

}  // namespace ns

using namespace ns;

extern "C" {

int ns_adj_forward(ns_handle* h, int nsteps, int ckpt_every) {
  if (!h) return NS_ERR_ARG;
  if (nsteps < 1 || ckpt_every < 1) return api_fail(h, NS_ERR_ARG, "adjoint: nsteps and ckpt_every must be >= 1");
  int s;
  if ((s = adj_check_cfg(h))) return s;
  if ((s = adj_ensure(h))) return s;
  AdjState* A = h->adj;
  A->ready = false;
  const int K = std::min(ckpt_every, nsteps);
  const int nck = (nsteps + K - 1) / K;
  // checkpoint and segment storage, kept across calls while the sizes hold
  if ((int)A->ck.size() != nck * 6) {
    adj_free_vec(A->ck);
    A->ck.assign((size_t)nck * 6, nullptr);
    for (double*& p : A->ck)
      if ((s = adj_alloc(h, &p))) return s;
  }
  if ((int)A->seg.size() != K * 3) {
    adj_free_vec(A->seg);
    A->seg.assign((size_t)K * 3, nullptr);
    for (double*& p : A->seg)
      if ((s = adj_alloc(h, &p))) return s;
  }
  for (double*& p : A->fin)
    if (!p && (s = adj_alloc(h, &p))) return s;
  A->ck_first.assign(nck, 0);
  A->seg_first.assign(K, 0);
  double* const st6[6] = {h->u, h->v, h->w, h->hx, h->hy, h->hz};
  for (int n = 0; n < nsteps; ++n) {
    if (n % K == 0) {
      for (int q = 0; q < 6; ++q)
        if ((s = adj_copy(h, A->ck[(size_t)(n / K) * 6 + q], st6[q]))) return s;
      A->ck_first[n / K] = h->first_pending ? 1 : 0;
    }
    if ((s = ns_step(h, 1))) return s;
  }
  double* const st7[7] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz};
  for (int q = 0; q < 7; ++q)
    if ((s = adj_copy(h, A->fin[q], st7[q]))) return s;
  A->fin_first = h->first_pending;
  A->fin_steps = h->steps;
  ADJ_CUDA(h, cudaStreamSynchronize(h->stream));
  A->nsteps = nsteps;
  A->ckpt = K;
  A->nck = nck;
  A->ready = true;
  return NS_OK;
}

int ns_adj_backward(ns_handle* h, const double* dJ_du, const double* dJ_dv, const double* dJ_dw, double* grad_u,
                    double* grad_v, double* grad_w, double* grad_hx, double* grad_hy, double* grad_hz) {
  if (!h) return NS_ERR_ARG;
  if (!dJ_du || !dJ_dv || !dJ_dw || !grad_u || !grad_v || !grad_w)
    return api_fail(h, NS_ERR_ARG, "adjoint: dJ_du/dv/dw and grad_u/v/w are required");
  AdjState* A = h->adj;
  if (!A || !A->ready) return api_fail(h, NS_ERR_ARG, "adjoint: call ns_adj_forward first");
  const ns_config& c = h->cfg;
  int s;
  // seed: dJ/du(T) with every periodic copy folded into its owner, then
  // the images refilled
  const double* seeds[3] = {dJ_du, dJ_dv, dJ_dw};
  for (int f = 0; f < 3; ++f) {
    ADJ_CUDA(h, cudaMemsetAsync(A->lam[f], 0, h->L.fsize * sizeof(double), h->stream));
    ADJ_CUDA(h, api_h2d_field(h, A->lam[f], seeds[f], f));
  }
  ADJ_CUDA(h, launch_periodic_fold(h->L, A->lam[0], A->lam[1], A->lam[2], true, h->stream));
  api_mark(h, "adj_fold", 3);
  ADJ_CUDA(h, launch_periodic_fill(h->L, A->lam[0], A->lam[1], A->lam[2], h->stream));
  api_mark(h, "adj_fill", 3);
  A->cur = 0;
  const int K = A->ckpt;
  const bool euler = c.scheme == NS_EULER;
  for (int sg = A->nck - 1; sg >= 0; --sg) {
    const int s0 = sg * K, s1 = std::min(s0 + K, A->nsteps);
    // recompute the segment from its checkpoint, keeping each step's input
    double* const st6[6] = {h->u, h->v, h->w, h->hx, h->hy, h->hz};
    for (int q = 0; q < 6; ++q)
      if ((s = adj_copy(h, st6[q], A->ck[(size_t)sg * 6 + q]))) return s;
    h->first_pending = A->ck_first[sg] != 0;
    for (int n = s0; n < s1; ++n) {
      for (int q = 0; q < 3; ++q)
        if ((s = adj_copy(h, A->seg[(size_t)(n - s0) * 3 + q], st6[q]))) return s;
      A->seg_first[n - s0] = (h->first_pending && !euler) ? 1 : 0;
      if (n + 1 < s1 && (s = ns_step(h, 1))) return s;
    }
    for (int n = s1 - 1; n >= s0; --n) {
      double* const fwd[3] = {A->seg[(size_t)(n - s0) * 3], A->seg[(size_t)(n - s0) * 3 + 1],
                              A->seg[(size_t)(n - s0) * 3 + 2]};
      const bool has_next = n + 1 < A->nsteps;
      if ((s = adj_backward_step(h, A, fwd, A->seg_first[n - s0] != 0, has_next))) return s;
    }
  }
  // gradients with respect to the independent values of u0, v0, w0 (the
  // periodic copies zeroed)
  ADJ_CUDA(h, launch_periodic_fold(h->L, A->lam[0], A->lam[1], A->lam[2], false, h->stream));
  api_mark(h, "adj_zero", 3);
  double* gr[3] = {grad_u, grad_v, grad_w};
  for (int f = 0; f < 3; ++f) ADJ_CUDA(h, api_d2h_field(h, gr[f], A->lam[f], f));
  // history input of step 0: cP ls of step 0 (zero after an Euler start)
  double* gh[3] = {grad_hx, grad_hy, grad_hz};
  const bool hist_used = !euler && !A->ck_first[0];
  for (int f = 0; f < 3; ++f)
    if (gh[f] && hist_used) ADJ_CUDA(h, api_d2h_field(h, gh[f], A->ls[1 - A->cur][f], f));
  ADJ_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int f = 0; f < 3; ++f) {
    if (!gh[f]) continue;
    const size_t n = (size_t)ref_ext(c, f, 0) * ref_ext(c, f, 1) * ref_ext(c, f, 2);
    if (!hist_used) {
      std::memset(gh[f], 0, n * sizeof(double));
      continue;
    }
    for (size_t e = 0; e < n; ++e) gh[f][e] *= -0.5 * c.dt;
    zero_copies(c, f, gh[f]);
  }
  // back to the state after the forward run
  double* const st7[7] = {h->u, h->v, h->w, h->p, h->hx, h->hy, h->hz};
  for (int q = 0; q < 7; ++q)
    if ((s = adj_copy(h, st7[q], A->fin[q]))) return s;
  ADJ_CUDA(h, cudaStreamSynchronize(h->stream));
  h->first_pending = A->fin_first;
  h->steps = A->fin_steps;
  return NS_OK;
}

}  // extern "C"
