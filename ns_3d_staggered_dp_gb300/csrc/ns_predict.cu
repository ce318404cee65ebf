// Fused predictor: convection (cal_conv, NS_functions.f90:53-158), diffusion
// (cal_diff, NS_functions.f90:161-210), pressure gradient, Euler/AB2/AB2-CN
// predictor and AB2 history update (big_periodic_3D.f90:340-423,
// re_simulation_sub_tstep_interBC_combine.f90:543-654), in one pass over HBM.
//
// The divergence-form convection is rebuilt from shared products.  With the
// factor 1/2 of every two-point mean folded into the constants:
//   SX[c]  = u[c] + u[c+1]                 (x-mean of u at cell c, times 2)
//   QXY    = (u[f,J-1] + u[f,J]) * (v[f-1,J] + v[f,J])   at x-face f, y-face J
//   conv_x = (SX[f]^2 - SX[f-1]^2)/(4dx) + (QXY[J+1]-QXY[J])/(4dy) + (QXZ[K+1]-QXZ[K])/(4dz)
// which is cal_conv's avg/product/diff sequence with the products shared
// between conv_x, conv_y and conv_z (uy*vx serves both conv_x and conv_y).
//
// Tiling: a CTA owns 32 x-cells by TY y-rows and marches along z through a
// chunk of KC planes.  Warp w (0..TY) is y-row j0-1+w; warp 0 only computes
// products: those of the low y-halo row and, in one extra pass with lane r
// on row r, the low x-halo position of every row.  Products are owned
// one-sided (cell a owns SX[a], and the face products at faces a+1), so an
// output cell needs products of its own and its lower neighbours only.  An
// FP64 warp instruction costs its full issue slot however many lanes are
// active, so no halo work is done by single lanes of the row warps.
// Every FP64 operation is issued in FMA form (see ns_internal.cuh).
#include <algorithm>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {

namespace {

constexpr int TX = 32;
constexpr int TY = 16;
constexpr int KC = 16;
constexpr int SXW = TX + 8;  // smem row width: column c is x = i0-2+c; columns 1..34 (x in
                             // [i0-1, i0+32]) are read, 0..35 loaded (a 320-byte row)
constexpr int SYH = TY + 2;  // smem rows: y in [j0-1, j0+TY]
constexpr int PXW = TX + 1;  // product row width: x in [i0-1, i0+31]
constexpr int PYH = TY + 1;  // product rows: y in [j0-1, j0+TY-1]

constexpr int RING = 4;       // planes k-1, k, k+1 in use, k+2 in flight

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

struct PredSmem {
  // u, v, w first: each ring slot (18 x 40 doubles, 5760 bytes) starts on a
  // 128-byte boundary for the tile loader
  double u[RING][SYH][SXW];
  double v[RING][SYH][SXW];
  double w[RING][SYH][SXW];
  double sx2[PYH][PXW];
  double sy2[PYH][PXW];
  double sz2[2][PYH][PXW];
  double qxy[PYH][PXW];
  double qxz[2][PYH][PXW];
  double qyz[2][PYH][PXW];
  unsigned long long bar[RING];  // tile loader: one mbarrier per ring slot
};
static_assert(sizeof(double) * SYH * SXW % 128 == 0, "ring slots of the tile loader stay 128-byte aligned");

// ---- tile loader (TMA): one thread fills a ring slot with three 40 x 18 x 1
// boxes (u, v, w) and arms the slot's mbarrier with their byte count ----
constexpr unsigned kTileBytes = 3u * SYH * SXW * sizeof(double);
constexpr int kWaitLimit = 1 << 20;                   // try_wait polls before a wait gives up
constexpr unsigned long long kWaitNs = 200000000ull;  // or 0.2 s of global time, whichever comes first

__device__ __forceinline__ unsigned sm_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(sm_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase `parity` of a barrier; false once max_polls polls or
// max_ns of global time found it incomplete (the caller records the error).
__device__ __forceinline__ bool mbar_wait_for(unsigned long long* bar, unsigned parity, int max_polls,
                                              unsigned long long max_ns) {
  // the common case (the plane has landed) reads no timer: a %globaltimer
  // read is a long-latency special-register access on every plane's path
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int it = 0; it < max_polls; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63) == 63 && global_ns() - t0 > max_ns) break;
  }
  return false;
}
// The tile loader's wait: kWaitLimit polls or kWaitNs.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  return mbar_wait_for(bar, parity, kWaitLimit, kWaitNs);
}

// Self-test of the bounded wait: one thread arms a barrier for 8 bytes that
// no copy will deliver and waits with the loader's wait code and a time limit
// of limit_ns.  When the wait gives up (the expected outcome) the thread
// delivers the 8 bytes itself (complete_tx), so the barrier's phase completes
// before the CTA exits; nothing is in flight at any time.
__global__ void wait_selftest_kernel(unsigned long long limit_ns, int* __restrict__ gave_up,
                                     unsigned long long* __restrict__ waited_ns) {
  __shared__ unsigned long long bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar);
  const unsigned b = sm_addr(&bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(8u) : "memory");
  const unsigned long long t0 = global_ns();
  const bool ok = mbar_wait_for(&bar, 0, 1 << 22, limit_ns);
  *waited_ns = global_ns() - t0;
  if (!ok) asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(8u) : "memory");
  *gave_up = ok ? 0 : 1;
}
// Fill ring slot s with plane k (clamped into the box) of u, v, w: x from slot
// i0-2 (tensor x = slot + 7: 8 (32 bx + 6) bytes, 16-byte aligned), y from
// row j0-1.  Positions past the field read zeros or row padding; only inactive
// positions use them.
__device__ __forceinline__ void tma_plane(PredSmem& S, const CUtensorMap* mu, const CUtensorMap* mv,
                                          const CUtensorMap* mw, int nz, int i0, int j0, int k, int s) {
  const int kk = clampi(k, 0, nz + 1);
  const int x = i0 - 2 + 7, y = j0 - 1;
  const unsigned b = sm_addr(&S.bar[s]);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the slot's last readers are done (barrier)
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(kTileBytes) : "memory");
  const CUtensorMap* maps[3] = {mu, mv, mw};
  double* dst[3] = {&S.u[s][0][0], &S.v[s][0][0], &S.w[s][0][0]};
#pragma unroll
  for (int f = 0; f < 3; ++f)
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(sm_addr(dst[f])), "l"(reinterpret_cast<unsigned long long>(maps[f])), "r"(x), "r"(y), "r"(kk), "r"(b)
        : "memory");
}


// Start copying plane k (clamped into the box) of u, v, w into ring slot s
// (cp.async; the caller commits the group).  Each smem row is 18 16-byte
// copies of slots i0-2 .. i0+33: index 7 + i0 - 2 = 32 bx + 6 (plus whole
// rows and planes of 8-double multiples) keeps every source 16-byte aligned.
// Rows and planes are clamped into the box; past x = nx + 1 the copies read
// row padding (or the next row, or the field's tail padding), which only
// positions without an output use.
__device__ __forceinline__ void issue_plane(PredSmem& S, const Layout& L, const double* __restrict__ u,
                                            const double* __restrict__ v, const double* __restrict__ w, int i0,
                                            int j0, int k, int s) {
  constexpr int NV = (TX + 4) / 2;
  const int kk = clampi(k, 0, L.nz + 1);
  const int nthr = blockDim.x * blockDim.y;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int e = tid; e < NV * SYH; e += nthr) {
    const int xv = e % NV, yy = e / NV;
    const int gj = clampi(j0 - 1 + yy, 0, L.ny + 1);
    const long long g = L.at(i0 - 2 + 2 * xv, gj, kk);
    cp_async16(&S.u[s][yy][2 * xv], u + g);
    cp_async16(&S.v[s][yy][2 * xv], v + g);
    cp_async16(&S.w[s][yy][2 * xv], w + g);
  }
}

// Products owned by position (a, b) = smem (x = xa, y = yb) at plane k, using
// ring slots s0 (plane k) and s1 (plane k+1).  Results go to product index
// (py, px) = (yb, xa) where xa/yb are smem coordinates of the position.
__device__ __forceinline__ void products(PredSmem& S, const FOne& c, int xa, int yb, int s0, int s1, int pb) {
  // SX[a] = u[a] + u[a+1]  (plane k, row b)
  const double sx = fadd(c, S.u[s0][yb][xa + 1], S.u[s0][yb][xa + 1 + 1]);
  // SY[b] = v[b] + v[b+1]
  const double sy = fadd(c, S.v[s0][yb][xa + 1], S.v[s0][yb + 1][xa + 1]);
  // SZ[k] = w[k] + w[k+1]
  const double sz = fadd(c, S.w[s0][yb][xa + 1], S.w[s1][yb][xa + 1]);
  // QXY at (x-face a+1, y-face b+1): (u[a+1,b] + u[a+1,b+1]) * (v[a,b+1] + v[a+1,b+1])
  const double q1 = fmul(c, fadd(c, S.u[s0][yb][xa + 1 + 1], S.u[s0][yb + 1][xa + 1 + 1]),
                         fadd(c, S.v[s0][yb + 1][xa + 1], S.v[s0][yb + 1][xa + 1 + 1]));
  // QXZ at (x-face a+1, cell b, z-face k+1): (u[a+1] at k, k+1) * (w[a], w[a+1] at k+1)
  const double q2 = fmul(c, fadd(c, S.u[s0][yb][xa + 1 + 1], S.u[s1][yb][xa + 1 + 1]),
                         fadd(c, S.w[s1][yb][xa + 1], S.w[s1][yb][xa + 1 + 1]));
  // QYZ at (cell a, y-face b+1, z-face k+1): (v[a,b+1] at k, k+1) * (w[a,b], w[a,b+1] at k+1)
  const double q3 = fmul(c, fadd(c, S.v[s0][yb + 1][xa + 1], S.v[s1][yb + 1][xa + 1]),
                         fadd(c, S.w[s1][yb][xa + 1], S.w[s1][yb + 1][xa + 1]));
  S.sx2[yb][xa] = fmul(c, sx, sx);
  S.sy2[yb][xa] = fmul(c, sy, sy);
  S.sz2[pb][yb][xa] = fmul(c, sz, sz);
  S.qxy[yb][xa] = q1;
  S.qxz[pb][yb][xa] = q2;
  S.qyz[pb][yb][xa] = q3;
}

// Products for z-face k only (the warm-up plane): SZ at cell k-1 (planes
// k-1, k) and QXZ/QYZ at z-face k.  s0 = plane k-1, s1 = plane k.
__device__ __forceinline__ void products_zface(PredSmem& S, const FOne& c, int xa, int yb, int s0, int s1, int pb) {
  const double sz = fadd(c, S.w[s0][yb][xa + 1], S.w[s1][yb][xa + 1]);
  const double q2 = fmul(c, fadd(c, S.u[s0][yb][xa + 1 + 1], S.u[s1][yb][xa + 1 + 1]),
                         fadd(c, S.w[s1][yb][xa + 1], S.w[s1][yb][xa + 1 + 1]));
  const double q3 = fmul(c, fadd(c, S.v[s0][yb + 1][xa + 1], S.v[s1][yb + 1][xa + 1]),
                         fadd(c, S.w[s1][yb][xa + 1], S.w[s1][yb + 1][xa + 1]));
  S.sz2[pb][yb][xa] = fmul(c, sz, sz);
  S.qxz[pb][yb][xa] = q2;
  S.qyz[pb][yb][xa] = q3;
}

}  // namespace

// MODE: 0 predictor, 1 conv only (writes conv into us/vs/ws), 2 diffusion only.
// One tile (bx, by) of TX x TY faces marching over the z-chunk bz.
// TMA: planes arrive by the tile loader (maps mu, mv, mw of a.u, a.v, a.w)
// instead of per-element cp.async.
template <int SCHEME, bool FIRST, bool DPF, int MODE, bool TMA = false>
__device__ __forceinline__ void predict_body(const PredictArgs& a, PredSmem& S, int bx, int by, int bz,
                                             const CUtensorMap* mu = nullptr, const CUtensorMap* mv = nullptr,
                                             const CUtensorMap* mw = nullptr) {
  const Layout L = a.L;
  const FOne c{a.one, a.mzero};
  const int lane = threadIdx.x;
  const int wy = threadIdx.y;  // 0..TY
  const int i0 = 1 + TX * bx;
  const int j0 = 1 + TY * by;
  const int kc = a.kc > 0 ? a.kc : KC;
  const int k0 = 1 + a.koff + kc * bz;
  const int k1 = min(k0 + kc, a.kend > 0 ? a.kend : L.nz + 1);
  // smem coordinates of this thread's position: x = i0-1+lane+1 -> xa = lane+1; y = j0-1+wy -> yb = wy
  const int xa = lane + 1;
  const int yb = wy;

  // Warm-up: planes k0-1 and k0 (one copy group) and k0+1 (a second one);
  // products at z-face k0 once the first group has landed.
  const bool producer = threadIdx.x == 0 && threadIdx.y == 0;
  unsigned phase = 0;  // tile loader: bit s is the parity of slot s's next phase
  bool ok = true;      // false once a wait gave up (recorded in a.err); every issued plane
                       // is still waited for (bounded), so none is in flight at exit
  auto wait_slot = [&](int sl) {
    const bool r = mbar_wait(&S.bar[sl], (phase >> sl) & 1u);
    ok = ok && r;
    phase ^= 1u << sl;
  };
  if (TMA) {
    if (producer) {
      for (int sl = 0; sl < RING; ++sl) mbar_init(&S.bar[sl]);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (producer) {
      tma_plane(S, mu, mv, mw, L.nz, i0, j0, k0 - 1, (k0 - 1) & 3);
      tma_plane(S, mu, mv, mw, L.nz, i0, j0, k0, k0 & 3);
      tma_plane(S, mu, mv, mw, L.nz, i0, j0, k0 + 1, (k0 + 1) & 3);
    }
    wait_slot((k0 - 1) & 3);
    wait_slot(k0 & 3);
  } else {
    issue_plane(S, L, a.u, a.v, a.w, i0, j0, k0 - 1, (k0 - 1) & 3);
    issue_plane(S, L, a.u, a.v, a.w, i0, j0, k0, k0 & 3);
    cp_async_commit();
    issue_plane(S, L, a.u, a.v, a.w, i0, j0, k0 + 1, (k0 + 1) & 3);
    cp_async_commit();
    cp_async_wait<1>();
  }
  __syncthreads();
  if (MODE != 2) {
    products_zface(S, c, xa, yb, (k0 - 1) & 3, k0 & 3, (k0 - 1) & 1);
    // low x-halo position of every row, by warp 0 (one partially active pass)
    if (wy == 0 && lane <= TY) products_zface(S, c, 0, lane, (k0 - 1) & 3, k0 & 3, (k0 - 1) & 1);
  }

  const int i = i0 + lane;
  const int j = j0 - 1 + wy;
  const int nx = L.nx, ny = L.ny;
  const bool in_xy = (wy >= 1) && (i <= nx) && (j <= ny);
  const bool act_u = in_xy && (i >= a.ulo);
  const bool act_v = in_xy && (j >= a.vlo);

  double hu = 0.0, hv = 0.0, hw = 0.0;  // tile loader: the AB2 history of this cell at plane k
  if (TMA && MODE == 0 && SCHEME != 0 && !FIRST && in_xy && k0 < k1) {
    const long long gh = L.at(i, j, k0);
    hu = __ldg(a.hx + gh);
    hv = __ldg(a.hy + gh);
    hw = __ldg(a.hz + gh);
  }
  for (int k = k0; k < k1; ++k) {
    const int s0 = k & 3, s1 = (k + 1) & 3, sm = (k + 3) & 3;  // planes k, k+1, k-1
    const int pb = k & 1, pbm = (k - 1) & 1;
    // With the tile loader, this cell's AB2 history is read one plane
    // ahead, so that its latency overlaps a whole iteration (each cell's
    // history is read and then rewritten by its own thread only); read where
    // it is used, it left the tile-loader kernel at 3.3 ms against 2.1.  The
    // cp.async loader reads it at the combine (its copies already fill that time).
    const double pu = hu, pv = hv, pw = hw;
    if (TMA && MODE == 0 && SCHEME != 0 && !FIRST && in_xy && k + 1 < k1) {
      const long long gh = L.at(i, j, k + 1);  // the next plane's, one iteration ahead
      hu = __ldg(a.hx + gh);
      hv = __ldg(a.hy + gh);
      hw = __ldg(a.hz + gh);
    }
    // plane k+1 has landed and every thread is done with plane k-2, whose
    // slot receives plane k+2 while this plane is computed
    if (TMA) wait_slot((k + 1) & 3);
    else cp_async_wait<0>();
    __syncthreads();
    if (TMA) {
      if (producer) tma_plane(S, mu, mv, mw, L.nz, i0, j0, k + 2, (k + 2) & 3);
    } else {
      issue_plane(S, L, a.u, a.v, a.w, i0, j0, k + 2, (k + 2) & 3);
      cp_async_commit();
    }
    if (MODE != 2) {
      products(S, c, xa, yb, s0, s1, pb);
      if (wy == 0 && lane <= TY) products(S, c, 0, lane, s0, s1, pb);
    }
    __syncthreads();
    const bool act_w = (k >= a.wlo);
    if (in_xy) {
      const long long g = L.at(i, j, k);
      // ---- x-component at x-face i ----
      if (act_u) {
        const double uc = S.u[s0][yb][xa + 1];
        const double sWE = fadd(c, S.u[s0][yb][xa - 1 + 1], S.u[s0][yb][xa + 1 + 1]);
        const double sSN = fadd(c, S.u[s0][yb - 1][xa + 1], S.u[s0][yb + 1][xa + 1]);
        const double sBT = fadd(c, S.u[sm][yb][xa + 1], S.u[s1][yb][xa + 1]);
        double C = 0.0;
        if (MODE != 2) {
          const double dX = fsub(c, S.sx2[yb][xa], S.sx2[yb][xa - 1]);
          const double dY = fsub(c, S.qxy[yb][xa - 1], S.qxy[yb - 1][xa - 1]);
          const double dZ = fsub(c, S.qxz[pb][yb][xa - 1], S.qxz[pbm][yb][xa - 1]);
          C = fmul(c, dX, a.cx);
          C = fma(dY, a.cy, C);
          C = fma(dZ, a.cz, C);  // C = -conv_x
        }
        double out;
        if (MODE == 1) {
          out = -C;
        } else if (MODE == 2) {
          out = fma(a.ix2, sWE, fma(a.iy2, sSN, fma(a.iz2, sBT, fmul(c, a.lap0, uc))));
        } else {
          out = predictor_combine<SCHEME, FIRST>(a, c, uc, sWE, sSN, sBT, C, TMA ? pu : a.hx[g], a.hx, g);
          if (DPF) out = fma(a.gpx, fsub(c, __ldg(a.p + g), __ldg(a.p + g - 1)), out);
        }
        a.us[g] = out;
      }
      // ---- y-component at y-face j ----
      if (act_v) {
        const double vc = S.v[s0][yb][xa + 1];
        const double sWE = fadd(c, S.v[s0][yb][xa - 1 + 1], S.v[s0][yb][xa + 1 + 1]);
        const double sSN = fadd(c, S.v[s0][yb - 1][xa + 1], S.v[s0][yb + 1][xa + 1]);
        const double sBT = fadd(c, S.v[sm][yb][xa + 1], S.v[s1][yb][xa + 1]);
        double C = 0.0;
        if (MODE != 2) {
          const double dX = fsub(c, S.qxy[yb - 1][xa], S.qxy[yb - 1][xa - 1]);
          const double dY = fsub(c, S.sy2[yb][xa], S.sy2[yb - 1][xa]);
          const double dZ = fsub(c, S.qyz[pb][yb - 1][xa], S.qyz[pbm][yb - 1][xa]);
          C = fmul(c, dX, a.cx);
          C = fma(dY, a.cy, C);
          C = fma(dZ, a.cz, C);
        }
        double out;
        if (MODE == 1) {
          out = -C;
        } else if (MODE == 2) {
          out = fma(a.ix2, sWE, fma(a.iy2, sSN, fma(a.iz2, sBT, fmul(c, a.lap0, vc))));
        } else {
          out = predictor_combine<SCHEME, FIRST>(a, c, vc, sWE, sSN, sBT, C, TMA ? pv : a.hy[g], a.hy, g);
          if (DPF) out = fma(a.gpy, fsub(c, __ldg(a.p + g), __ldg(a.p + g - L.sy)), out);
        }
        a.vs[g] = out;
      }
      // ---- z-component at z-face k ----
      if (act_w) {
        const double wc = S.w[s0][yb][xa + 1];
        const double sWE = fadd(c, S.w[s0][yb][xa - 1 + 1], S.w[s0][yb][xa + 1 + 1]);
        const double sSN = fadd(c, S.w[s0][yb - 1][xa + 1], S.w[s0][yb + 1][xa + 1]);
        const double sBT = fadd(c, S.w[sm][yb][xa + 1], S.w[s1][yb][xa + 1]);
        double C = 0.0;
        if (MODE != 2) {
          const double dX = fsub(c, S.qxz[pbm][yb][xa], S.qxz[pbm][yb][xa - 1]);
          const double dY = fsub(c, S.qyz[pbm][yb][xa], S.qyz[pbm][yb - 1][xa]);
          const double dZ = fsub(c, S.sz2[pb][yb][xa], S.sz2[pbm][yb][xa]);
          C = fmul(c, dX, a.cx);
          C = fma(dY, a.cy, C);
          C = fma(dZ, a.cz, C);
        }
        double out;
        if (MODE == 1) {
          out = -C;
        } else if (MODE == 2) {
          out = fma(a.ix2, sWE, fma(a.iy2, sSN, fma(a.iz2, sBT, fmul(c, a.lap0, wc))));
        } else {
          out = predictor_combine<SCHEME, FIRST>(a, c, wc, sWE, sSN, sBT, C, TMA ? pw : a.hz[g], a.hz, g);
          if (DPF) out = fma(a.gpz, fsub(c, __ldg(a.p + g), __ldg(a.p + g - L.sz)), out);
        }
        a.ws[g] = out;
      }
    }
  }
  if (TMA) {
    // the last plane issued (k1 + 1) is still in flight: drain it (bounded);
    // a wait that gave up marks the step invalid
    wait_slot((k1 + 1) & 3);
    if (!ok && a.err) atomicExch(a.err, 1);
  } else {
    cp_async_wait<0>();  // nothing left in flight when the tile is done
  }
}

template <int SCHEME, bool FIRST, bool DPF, int MODE>
__global__ void __launch_bounds__(TX*(TY + 1)) predict_kernel(PredictArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  predict_body<SCHEME, FIRST, DPF, MODE>(a, *reinterpret_cast<PredSmem*>(smem_raw), blockIdx.x, blockIdx.y,
                                         blockIdx.z);
}

// The same with the tile loader: the maps of a.u, a.v, a.w as kernel
// parameters, the ring slots 128-byte aligned in dynamic shared memory.
template <int SCHEME, bool FIRST, bool DPF>
__global__ void __launch_bounds__(TX*(TY + 1)) predict_tma_kernel(PredictArgs a, const __grid_constant__ CUtensorMap mu,
                                                                  const __grid_constant__ CUtensorMap mv,
                                                                  const __grid_constant__ CUtensorMap mw) {
  extern __shared__ __align__(16) unsigned char smem_tma[];  // base rounded up to 128 B below
  unsigned char* p = smem_tma + ((128u - (sm_addr(smem_tma) & 127u)) & 127u);
  predict_body<SCHEME, FIRST, DPF, 0, true>(a, *reinterpret_cast<PredSmem*>(p), blockIdx.x, blockIdx.y, blockIdx.z,
                                            &mu, &mv, &mw);
}

// Batched: persistent CTAs walk the work items (subdomain, tile) of a batch.
template <int SCHEME, bool FIRST, bool DPF>
__global__ void __launch_bounds__(TX*(TY + 1), 2) predict_batch_kernel(const PredictArgs* __restrict__ tab,
                                                                       const BatchItem* __restrict__ items,
                                                                       int n_items) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    // the subdomain's arguments in registers: a reference into shared memory
    // would be reloaded after every barrier of the plane loop
    const PredictArgs a = tab[w.sub];
    predict_body<SCHEME, FIRST, DPF, 0>(a, *reinterpret_cast<PredSmem*>(smem_raw), w.bx, w.by, w.bz);
    __syncthreads();
  }
}

size_t predict_smem_bytes() { return sizeof(PredSmem); }

// The tile loader serves a launch whose u, v, w are the mapped fields.
static bool tma_serves(const PredTma* t, const PredictArgs& a) {
  return t && t->ready && a.u == t->pu && a.v == t->pv && a.w == t->pw;
}

template <int SCHEME, bool FIRST, bool DPF, int MODE>
static cudaError_t launch_grid(const PredictArgs& b, dim3 grid, cudaStream_t st, const PredTma* tma) {
  const dim3 block(TX, TY + 1);
  if constexpr (MODE == 0) {
    if (tma_serves(tma, b)) {
      auto kern = predict_tma_kernel<SCHEME, FIRST, DPF>;
      const size_t sm = sizeof(PredSmem) + 128;
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return e;
      kern<<<grid, block, sm, st>>>(b, tma->u, tma->v, tma->w);
      return cudaGetLastError();
    }
  }
  auto kern = predict_kernel<SCHEME, FIRST, DPF, MODE>;
  const size_t sm = sizeof(PredSmem);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  kern<<<grid, block, sm, st>>>(b);
  return cudaGetLastError();
}

template <int SCHEME, bool FIRST, bool DPF, int MODE>
static cudaError_t launch_t(const PredictArgs& a, cudaStream_t st, const PredTma* tma) {
  PredictArgs b = a;
  b.kc = b.koff = b.kend = 0;
  const dim3 grid((a.L.nx + TX - 1) / TX, (a.L.ny + TY - 1) / TY, (a.L.nz + KC - 1) / KC);
  return launch_grid<SCHEME, FIRST, DPF, MODE>(b, grid, st, tma);
}

int predict_chunk_planes() { return KC; }

cudaError_t launch_wait_selftest(unsigned long long limit_ns, int* gave_up, unsigned long long* waited_ns,
                                 cudaStream_t st) {
  wait_selftest_kernel<<<1, 32, 0, st>>>(limit_ns, gave_up, waited_ns);
  return cudaGetLastError();
}

template <int SCHEME, bool FIRST, bool DPF>
static cudaError_t launch_planes_t(PredictArgs b, cudaStream_t st, int p0, int p1, int kc, const PredTma* tma) {
  b.kc = kc;
  b.koff = p0 - 1;
  b.kend = p1;
  const dim3 grid((b.L.nx + TX - 1) / TX, (b.L.ny + TY - 1) / TY, (p1 - p0 + kc - 1) / kc);
  return launch_grid<SCHEME, FIRST, DPF, 0>(b, grid, st, tma);
}

cudaError_t launch_predict_planes(PredictArgs a, int scheme, bool first, bool dpf, int p0, int p1, int kc,
                                  cudaStream_t st, const PredTma* tma) {
  if (p0 < 1 || p1 > a.L.nz + 1 || p0 > p1 || kc < 1) return cudaErrorInvalidValue;
  if (p0 == p1) return cudaSuccess;
#define NS_PRED_PCASE(S, F, D) \
  if (scheme == S && first == F && dpf == D) return launch_planes_t<S, F, D>(a, st, p0, p1, kc, tma);
  NS_PRED_PCASE(0, false, false) NS_PRED_PCASE(0, false, true) NS_PRED_PCASE(0, true, false) NS_PRED_PCASE(0, true, true)
  NS_PRED_PCASE(1, false, false) NS_PRED_PCASE(1, false, true) NS_PRED_PCASE(1, true, false) NS_PRED_PCASE(1, true, true)
  NS_PRED_PCASE(2, false, false) NS_PRED_PCASE(2, false, true) NS_PRED_PCASE(2, true, false) NS_PRED_PCASE(2, true, true)
#undef NS_PRED_PCASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_predict(const PredictArgs& a, int scheme, bool first, bool dpf, int mode, cudaStream_t st,
                           const PredTma* tma) {
  if (mode == 1) return launch_t<0, false, false, 1>(a, st, nullptr);
  if (mode == 2) return launch_t<0, false, false, 2>(a, st, nullptr);
#define NS_PRED_CASE(S, F, D) \
  if (scheme == S && first == F && dpf == D) return launch_t<S, F, D, 0>(a, st, tma);
  NS_PRED_CASE(0, false, false) NS_PRED_CASE(0, false, true) NS_PRED_CASE(0, true, false) NS_PRED_CASE(0, true, true)
  NS_PRED_CASE(1, false, false) NS_PRED_CASE(1, false, true) NS_PRED_CASE(1, true, false) NS_PRED_CASE(1, true, true)
  NS_PRED_CASE(2, false, false) NS_PRED_CASE(2, false, true) NS_PRED_CASE(2, true, false) NS_PRED_CASE(2, true, true)
#undef NS_PRED_CASE
  return cudaErrorInvalidValue;
}

bool make_pred_tma(PredTma& t, const Layout& L, const double* u, const double* v, const double* w) {
  t = PredTma{};
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return false;
  auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  // element (x, y, z) of the tensor is slot (x - 7, y, z): index 7 + slot + sy*y + sz*z
  const cuuint64_t dims[3] = {(cuuint64_t)L.px, (cuuint64_t)(L.ny + 2), (cuuint64_t)(L.nz + 2)};
  const cuuint64_t strides[2] = {(cuuint64_t)L.sy * sizeof(double), (cuuint64_t)L.sz * sizeof(double)};
  const cuuint32_t box[3] = {(cuuint32_t)SXW, (cuuint32_t)SYH, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const double* f[3] = {u, v, w};
  CUtensorMap* m[3] = {&t.u, &t.v, &t.w};
  for (int i = 0; i < 3; ++i)
    if (encode(m[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(f[i]), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  t.pu = u;
  t.pv = v;
  t.pw = w;
  t.ready = 1;
  return true;
}

void predict_tiles(const Layout& L, int& gx, int& gy, int& gz) {
  gx = (L.nx + TX - 1) / TX;
  gy = (L.ny + TY - 1) / TY;
  gz = (L.nz + KC - 1) / KC;
}

template <int SCHEME, bool FIRST, bool DPF>
static cudaError_t launch_bt(const PredictArgs* tab, const BatchItem* items, int n_items, int grid, cudaStream_t st) {
  auto kern = predict_batch_kernel<SCHEME, FIRST, DPF>;
  const size_t sm = sizeof(PredSmem);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  if (grid <= 0) {
    int per_sm = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TX * (TY + 1), sm);
    grid = std::max(1, per_sm) * nsm;
  }
  grid = std::min(grid, n_items);
  if (grid <= 0) return cudaSuccess;
  kern<<<grid, dim3(TX, TY + 1), sm, st>>>(tab, items, n_items);
  return cudaGetLastError();
}

cudaError_t launch_predict_batch(const PredictArgs* tab, const BatchItem* items, int n_items, int scheme, bool first,
                                 bool dpf, int grid, cudaStream_t st) {
#define NS_PRED_CASE(S, F, D) \
  if (scheme == S && first == F && dpf == D) return launch_bt<S, F, D>(tab, items, n_items, grid, st);
  NS_PRED_CASE(0, false, false) NS_PRED_CASE(0, false, true) NS_PRED_CASE(0, true, false) NS_PRED_CASE(0, true, true)
  NS_PRED_CASE(1, false, false) NS_PRED_CASE(1, false, true) NS_PRED_CASE(1, true, false) NS_PRED_CASE(1, true, true)
  NS_PRED_CASE(2, false, false) NS_PRED_CASE(2, false, true) NS_PRED_CASE(2, true, false) NS_PRED_CASE(2, true, true)
#undef NS_PRED_CASE
  return cudaErrorInvalidValue;
}

}  // namespace ns
