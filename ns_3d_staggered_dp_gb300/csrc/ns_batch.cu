// Batched re-simulation of many sub-blocks of a parent run
// (re_simulation_sub_tstep_interBC_combine.f90:415-811 for every subdomain
// at once, the generalisation of the single 32^3 sub-block of
// big_periodic_3D.f90:20-25,664-712 to many boxes of uneven size).
//
// Every subdomain is an all-wall box (velocity bc 2 or 4, pressure bc 2, 3
// or 4, dp_flag = 1, no gauge shift) whose boundary values come from the
// parent's u* and dp.  A step of all subdomains is a fixed sequence of
// stages; each stage is ONE persistent kernel whose CTAs walk a work queue
// of (subdomain, tile) items, so boxes of 16^3 and 64^3 share the GPU
// instead of running one small grid after another:
//   interp   faces + mean dp of the step from the parent snapshots (spline)
//   predict  fused convection/diffusion/AB2 predictor (ns_predict.cu)
//   vel_bc   x, y, z passes of vel_bc_staggered (ns_bc.cu)
//   x fwd    divergence + modify_rhs + dense x transform (ns_dct.cu)
//   y fwd    dense y transform
//   z solve  tridiagonal line solve along z
//   y inv, x inv
//   pr_bc    x, y, z passes of pr_bc_staggered
//   correct  projection (ns_correct.cu)
//   hist     AB2 history save/restore around the sub-steps (:602-612)
// The stage sequence of a (sub-)step is captured once in a CUDA graph and
// replayed.  Mode 1 launches the same kernels once per subdomain (the
// per-subdomain loop) for comparison; both modes give the same bits.
//
// Time interpolation (sub_tstep_BC_combined_interpolation.m:53-64): the
// faces of a step at time t are sum_q w_q * snapshot_q over the 6 snapshot
// knots around t, w the not-a-knot cubic spline weights (interp1 'spline').
// get_velpr_bc is linear in (u*, dp), so interpolating the faces equals
// extracting faces from the interpolated u*, dp the reference reads.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ns_internal.cuh"
#include "ns_kernels.cuh"
#include "ns_session.cuh"

using namespace ns;

namespace {

// Stage kernels (index into ns_batch_config.grid).
enum Stage {
  ST_INTERP = 0, ST_PREDICT, ST_VBC_X, ST_VBC_Y, ST_VBC_Z, ST_XF, ST_YF, ST_TRI, ST_YI, ST_XI,
  ST_PBC_X, ST_PBC_Y, ST_PBC_Z, ST_CORRECT, ST_HIST, ST_COUNT
};
const char* kStageName[ST_COUNT] = {"interp", "predict", "vel_bc_x", "vel_bc_y", "vel_bc_z", "dense_x_fwd",
                                    "dense_y_fwd", "tri_z_solve", "dense_y_inv", "dense_x_inv", "pr_bc_x",
                                    "pr_bc_y", "pr_bc_z", "correct", "hist"};
constexpr int kChunk = 256;  // elements per item of the elementwise stages

__host__ __device__ inline int plane_n1(const Layout& L, int a) { return a == 0 ? L.ny + 2 : L.nx + 2; }
__host__ __device__ inline int plane_n2(const Layout& L, int a) { return a == 2 ? L.ny + 2 : L.nz + 2; }

// Per-subdomain arguments of the interpolation / capture / copy kernels.
struct SubGeo {
  Layout L;
  int x0, y0, z0;       // 1-based parent origin
  double* face;         // current faces (24 planes, [axis][field][side] order)
  long long face_n;     // doubles of the 24 planes
  long long snap_off;   // offset of this subdomain's planes inside a snapshot slot
  double* mean;         // current mean dp (device scalar)
  double* fld[7];       // u, v, w, p, hx, hy, hz
  double* save[3];      // saved AB2 history
};

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// faces(t) = sum_q w_q * snapshot[slot_q] (and the mean dp alike).
__global__ void __launch_bounds__(kChunk) interp_kernel(const SubGeo* __restrict__ geo, const BatchItem* __restrict__ items,
                                                        int n_items, const double* __restrict__ snaps,
                                                        long long slot_stride, const double* __restrict__ snap_mean,
                                                        int nsub, const int* __restrict__ slots,
                                                        const double* __restrict__ wts) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const SubGeo& g = geo[w.sub];
    const int* sl = slots + 6 * w.sub;
    const double* wq = wts + 6 * w.sub;
    const long long e = (long long)w.bx * kChunk + threadIdx.x;
    if (e < g.face_n) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < 6; ++q) acc = fma(wq[q], snaps[sl[q] * slot_stride + g.snap_off + e], acc);
      g.face[e] = acc;
    }
    if (w.bx == 0 && threadIdx.x == 0) {
      double m = 0.0;
#pragma unroll
      for (int q = 0; q < 6; ++q) m = fma(wq[q], snap_mean[(long long)sl[q] * nsub + w.sub], m);
      *g.mean = m;
    }
  }
}

// Faces of every subdomain from the parent's fields (get_velpr_bc,
// NS_functions.f90:414-510; get_pr_bc :514-562).  pu/pv/pw are the parent's
// u* (using_Ustar) or u, pdp its dp (dp_flag = 1) or p; pprev, when not null,
// is the previous p whose dt*diff(pprev)/h the u branch adds with dp_flag = 0
// (:434-437).  Element e of a subdomain's face buffer is decoded to (axis a,
// field f, side, slot s1, s2 of the plane); the reference face array index is
// the slot minus the field's slot offset on that axis.  Every value is formed
// with the reference's operations in its order (no contraction into FMAs), so
// the faces equal get_velpr_bc of the same arrays bit for bit.
// With AB2-CN the buffer continues with the per-sweep planes: sweep a's
// faces of u, v, w on axis a from the parent's u* after that sweep
// (sw.f[a][field]), as big_periodic_3D.f90:433-489 records them.
struct SweepSrc {
  const double* f[3][3];
};
__global__ void __launch_bounds__(kChunk) capture_kernel(const SubGeo* __restrict__ geo,
                                                         const BatchItem* __restrict__ items, int n_items, Layout Lp,
                                                         const double* __restrict__ pus, const double* __restrict__ pvs,
                                                         const double* __restrict__ pws, const double* __restrict__ pdp,
                                                         const double* __restrict__ pprev, double dt,
                                                         double* __restrict__ slot_base, int bc, int pbc, double dx,
                                                         double dy, double dz, const double* __restrict__ gauge,
                                                         SweepSrc sw) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const SubGeo& g = geo[w.sub];
    long long e = (long long)w.bx * kChunk + threadIdx.x;
    if (e >= g.face_n) continue;
    double* out = slot_base + g.snap_off + e;
    const Layout& L = g.L;
    int a = 0, f = 0, side = 0;
    bool sweep = false;
    {
      long long r = e;
      bool found = false;
      for (int aa = 0; aa < 3 && !found; ++aa) {
        const long long ps = (long long)plane_n1(L, aa) * plane_n2(L, aa);
        for (int q = 0; q < 8; ++q) {
          if (r < ps) { a = aa; f = q / 2; side = q % 2; found = true; break; }
          r -= ps;
        }
      }
      for (int aa = 0; aa < 3 && !found; ++aa) {  // the per-sweep planes
        const long long ps = (long long)plane_n1(L, aa) * plane_n2(L, aa);
        for (int q = 0; q < 6; ++q) {
          if (r < ps) { a = aa; f = q / 2; side = q % 2; found = true; sweep = true; break; }
          r -= ps;
        }
      }
      e = r;
    }
    const unsigned n1 = (unsigned)plane_n1(L, a);
    const int s2 = (int)((unsigned)e / n1), s1 = (int)((unsigned)e - (unsigned)s2 * n1);  // e < one face plane
    const int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
    const int n3[3] = {L.nx, L.ny, L.nz};
    // reference (0-based) indices along a1, a2
    const int r1 = s1 - (f == a1 ? 1 : 0), r2 = s2 - (f == a2 ? 1 : 0);
    const int ext1 = (f == a1) ? n3[a1] + 1 : n3[a1] + 2, ext2 = (f == a2) ? n3[a2] + 1 : n3[a2] + 2;
    if (r1 < 0 || r1 >= ext1 || r2 < 0 || r2 >= ext2) {
      *out = 0.0;
      continue;
    }
    // indices along a and the combination (0 single, 1 mean of two, 2 difference over h)
    const int na = n3[a];
    int i0, i1 = 0, op;
    if (f == a) {                      // normal velocity component: the wall face itself
      i0 = side ? na : 0; op = 0;
    } else {
      const int code = (f == 3) ? pbc : bc;
      if (f == 3 && code == 3) {       // one-sided gradient (NS_functions.f90:534-536)
        i0 = side ? na + 1 : 1; i1 = side ? na : 0; op = 2;
      } else if (code == 2) {          // value on the wall: mean of ghost and first cell
        i0 = side ? na + 1 : 0; i1 = side ? na : 1; op = 1;
      } else {                         // value at the ghost
        i0 = side ? na + 1 : 0; op = 0;
      }
    }
    const double* F = sweep ? sw.f[a][f] : (f == 0 ? pus : (f == 1 ? pvs : (f == 2 ? pws : pdp)));
    const int x0[3] = {g.x0, g.y0, g.z0};
    // parent slot along axis b of the 0-based sub-array index i: x0 + i - (face axis ? 0 : 1)
    int ia[3], ib[3];
    ia[a] = i0; ib[a] = i1;
    ia[a1] = ib[a1] = r1;
    ia[a2] = ib[a2] = r2;
    int sa[3], sb[3];
    for (int b = 0; b < 3; ++b) {
      const int off = (f == b) ? 0 : 1;
      sa[b] = x0[b] + ia[b] - off;
      sb[b] = x0[b] + ib[b] - off;
    }
    // the recorded dp is the gauge-shifted one, dp - dp(1,1,1) (big_periodic_3D.f90:562)
    const double g0 = (f == 3 && gauge) ? *gauge : 0.0;
    // u_bc_corr = u_bc + diff(p_previous)/h*dt on the velocity fields (u branch, dp_flag = 0):
    // diff(p) at the face slot s of field f is p[s] - p[s - e_f] in the slot layout
    const bool corr = pprev && f < 3 && !sweep;
    const double hf = f == 0 ? dx : (f == 1 ? dy : dz);
    const long long ef = f == 0 ? 1 : (f == 1 ? Lp.sy : Lp.sz);
    auto val = [&](const int* s) {
      const long long q = Lp.at(s[0], s[1], s[2]);
      if (corr) return __dadd_rn(F[q], __dmul_rn(__ddiv_rn(__dsub_rn(pprev[q], pprev[q - ef]), hf), dt));
      return f == 3 && gauge ? __dsub_rn(F[q], g0) : F[q];
    };
    const double v0 = val(sa);
    double v;
    if (op == 0) {
      v = v0;
    } else {
      const double v1 = val(sb);
      const double h = a == 0 ? dx : (a == 1 ? dy : dz);
      v = (op == 1) ? __ddiv_rn(__dadd_rn(v0, v1), 2.0) : __ddiv_rn(__dsub_rn(v0, v1), h);
    }
    *out = v;
  }
}

// Mean of the parent's dp over each subdomain's interior cells (one CTA per
// subdomain, fixed summation order).
__global__ void __launch_bounds__(256) capture_mean_kernel(const SubGeo* __restrict__ geo, int nsub, Layout Lp,
                                                           const double* __restrict__ pdp, double* __restrict__ out,
                                                           const double* __restrict__ gauge) {
  __shared__ double red[256];
  const double g0 = gauge ? *gauge : 0.0;
  for (int s = blockIdx.x; s < nsub; s += gridDim.x) {
    const SubGeo& g = geo[s];
    const long long n = (long long)g.L.nx * g.L.ny * g.L.nz;
    double acc = 0.0;
    for (long long t = threadIdx.x; t < n; t += 256) {
      const int i = (int)(t % g.L.nx), j = (int)((t / g.L.nx) % g.L.ny), k = (int)(t / ((long long)g.L.nx * g.L.ny));
      // sub cell slot (i+1, j+1, k+1) -> parent slot x0 - 1 + slot
      acc += pdp[Lp.at(g.x0 + i, g.y0 + j, g.z0 + k)] - g0;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = red[0] / (double)n;
    __syncthreads();
  }
}

// Sub-block gather of u, v, w, p and the AB2 history from the parent
// (u_sub = u(idx_xu, idx_yu, idx_zu), big_periodic_3D.f90:665-669): sub slot
// s maps to parent slot x0 - 1 + s on every axis and field.
__global__ void __launch_bounds__(kChunk) gather_kernel(const SubGeo* __restrict__ geo, const BatchItem* __restrict__ items,
                                                        int n_items, Layout Lp, const double* __restrict__ pf0,
                                                        const double* __restrict__ pf1, const double* __restrict__ pf2,
                                                        const double* __restrict__ pf3, const double* __restrict__ pf4,
                                                        const double* __restrict__ pf5, const double* __restrict__ pf6) {
  const double* pf[7] = {pf0, pf1, pf2, pf3, pf4, pf5, pf6};
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const SubGeo& g = geo[w.sub];
    const Layout& L = g.L;
    const long long tot = (long long)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    const long long e = (long long)w.bx * kChunk + threadIdx.x;
    if (e >= tot) continue;
    const int i = (int)(e % (L.nx + 2)), j = (int)((e / (L.nx + 2)) % (L.ny + 2));
    const int k = (int)(e / ((long long)(L.nx + 2) * (L.ny + 2)));
    const long long gs = L.at(i, j, k);
    const long long gp = Lp.at(g.x0 - 1 + i, g.y0 - 1 + j, g.z0 - 1 + k);
#pragma unroll
    for (int f = 0; f < 7; ++f) g.fld[f][gs] = pf[f] ? pf[f][gp] : 0.0;
  }
}

// AB2 history save (op 1) / restore (op 2) of the subdomains listed in items.
__global__ void __launch_bounds__(kChunk) hist_kernel(const SubGeo* __restrict__ geo, const BatchItem* __restrict__ items,
                                                      int n_items) {
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];  // bz = op
    const SubGeo& g = geo[w.sub];
    const long long e = (long long)w.bx * kChunk + threadIdx.x;
    if (e >= g.L.fsize) continue;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (w.bz == 1) g.save[f][e] = g.fld[4 + f][e];
      else g.fld[4 + f][e] = g.save[f][e];
    }
  }
}

int persistent_grid(int want, int n_items) {
  int g = want > 0 ? want : 8 * 152;
  return std::max(1, std::min(g, n_items));
}

// ---------------------------------------------------------------------------
// Not-a-knot cubic spline on 6 knots: weights of the data values at t.
// Unknowns: second derivatives M0..M5; rows 1-4 slope continuity, rows 0
// and 5 third-derivative continuity at knots 1 and 4 (not-a-knot).
// ---------------------------------------------------------------------------
bool spline6_weights(const double* x, double t, double* w) {
  double h[5];
  for (int i = 0; i < 5; ++i) {
    h[i] = x[i + 1] - x[i];
    if (!(h[i] > 0)) return false;
  }
  // A M = B y  (B maps the data to the right-hand side)
  double A[6][6] = {}, B[6][6] = {};
  A[0][0] = -1.0 / h[0]; A[0][1] = 1.0 / h[0] + 1.0 / h[1]; A[0][2] = -1.0 / h[1];
  for (int i = 1; i <= 4; ++i) {
    A[i][i - 1] = h[i - 1];
    A[i][i] = 2.0 * (h[i - 1] + h[i]);
    A[i][i + 1] = h[i];
    B[i][i + 1] += 6.0 / h[i];
    B[i][i] -= 6.0 / h[i] + 6.0 / h[i - 1];
    B[i][i - 1] += 6.0 / h[i - 1];
  }
  A[5][3] = -1.0 / h[3]; A[5][4] = 1.0 / h[3] + 1.0 / h[4]; A[5][5] = -1.0 / h[4];
  // Solve A C = B (C = d M / d y) by Gaussian elimination with partial pivoting.
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
    if (A[piv][c] == 0.0) return false;
    if (piv != c)
      for (int k = 0; k < 6; ++k) { std::swap(A[c][k], A[piv][k]); std::swap(B[c][k], B[piv][k]); }
    for (int r = c + 1; r < 6; ++r) {
      const double m = A[r][c] / A[c][c];
      if (m == 0.0) continue;
      for (int k = 0; k < 6; ++k) { A[r][k] -= m * A[c][k]; B[r][k] -= m * B[c][k]; }
    }
  }
  double C[6][6];
  for (int r = 5; r >= 0; --r)
    for (int k = 0; k < 6; ++k) {
      double s = B[r][k];
      for (int q = r + 1; q < 6; ++q) s -= A[r][q] * C[q][k];
      C[r][k] = s / A[r][r];
    }
  // interval [x_i, x_i+1] containing t (clamped to the window)
  int i = 0;
  while (i < 4 && t > x[i + 1]) ++i;
  const double hi = h[i], a = x[i + 1] - t, b = t - x[i];
  for (int q = 0; q < 6; ++q) {
    const double yi = (q == i) ? 1.0 : 0.0, yj = (q == i + 1) ? 1.0 : 0.0;
    w[q] = C[i][q] * a * a * a / (6.0 * hi) + C[i + 1][q] * b * b * b / (6.0 * hi) + (yi / hi - C[i][q] * hi / 6.0) * a +
           (yj / hi - C[i + 1][q] * hi / 6.0) * b;
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// The batch
// ---------------------------------------------------------------------------
struct ns_batch {
  ns_batch_config cfg;
  int n = 0;
  std::vector<ns_subdomain> desc;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t cap_stream = nullptr;
  std::string err;
  // device memory
  double* arena = nullptr;       // fields of all subdomains
  size_t arena_n = 0;
  double* tables = nullptr;      // dense matrices and eigenvalues per size class
  double* adi_tab = nullptr;     // AB2-CN: line-system factors per (axis, size, normal/tangential)
  double2* tri_tab = nullptr;    // z-solve multipliers of every subdomain (one per spectrum entry)
  double* snaps = nullptr;       // n_slots x (all faces)
  double* snap_mean = nullptr;   // n_slots x n
  long long slot_stride = 0;
  std::vector<double> snap_t;
  std::vector<char> snap_ok;
  unsigned char* dev_args = nullptr;  // argument tables and work items
  int* dev_slots = nullptr;           // [stage slot][n][6]
  double* dev_wts = nullptr;
  int* host_slots = nullptr;          // pinned
  double* host_wts = nullptr;
  int max_r = 1;
  // per subdomain (host copies)
  std::vector<Layout> L;
  std::vector<SubGeo> geo;
  std::vector<SpecPlan> plan;
  // device tables
  SubGeo* d_geo = nullptr;
  PredictArgs* d_pred[2] = {nullptr, nullptr};   // [0] dt0/r, [1] dt0
  BatchSpecArgs* d_spec[2] = {nullptr, nullptr};
  CorrectArgs* d_corr[2] = {nullptr, nullptr};
  BatchBcArgs* d_bc = nullptr;
  BatchAdiArgs* d_adi = nullptr;  // AB2-CN only
  // work items: per active set (0 regular, s >= 1 sub-step s of the first
  // interval), per stage: offset, count, and per-subdomain ranges
  BatchItem* d_items = nullptr;
  // cnt_dense: the leading items of a spectral stage that take the dense
  // kernel (the rest take the FFT-based one); cnt for every other stage
  struct Range { long long off = 0; int cnt = 0; int cnt_dense = 0; };
  std::vector<std::vector<Range>> rng;                  // [set][stage]
  std::vector<std::vector<std::vector<Range>>> sub_rng; // [set][stage][sub]
  // the divergence items of the x forward stage (subdomains with an FFT-based
  // x), and those of their boundary cells' pressure-BC terms
  std::vector<Range> div_rng, bc_rng;                   // [set]
  std::vector<std::vector<Range>> sub_div_rng, sub_bc_rng;  // [set][sub]
  std::vector<std::vector<int>> active;                 // [set] -> subdomains
  size_t spec_smem[5] = {0, 0, 0, 0, 0};
  size_t spec_smem_dct[4] = {0, 0, 0, 0};
  // gather / capture items (all subdomains)
  Range gather_rng, capture_rng;
  // state
  int intervals_done = 0;
  long long launches = 0;
  std::map<int, cudaGraphExec_t> graphs;  // key: set * 2 + first
  std::map<int, long long> graph_count;
  cudaEvent_t copy_done = nullptr;
  // u branch with dp_flag = 0: the parent's p at the previous capture
  double* p_prev = nullptr;
  long long p_prev_n = 0;
};

namespace {

int bfail(ns_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}
#define NB_CUDA(b, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return bfail((b), NS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// A subdomain's face buffer: the 24 planes of get_velpr_bc ([axis][field
// 0..3][side]), then with AB2-CN the 18 per-sweep planes ([sweep axis][field
// 0..2][side], each over the other two axes).
long long face_doubles(const Layout& L, bool cn = false) {
  long long t = 0;
  for (int a = 0; a < 3; ++a) t += (cn ? 14LL : 8LL) * plane_n1(L, a) * plane_n2(L, a);
  return t;
}
long long sweep_face_off(const Layout& L, int a, int f, int side) {
  long long o = face_doubles(L);
  for (int q = 0; q < a; ++q) o += 6LL * plane_n1(L, q) * plane_n2(L, q);
  return o + (long long)(2 * f + side) * plane_n1(L, a) * plane_n2(L, a);
}

// Launch the kernel(s) of one stage for active set `set` (one launch, or one
// per subdomain in the loop mode).
cudaError_t launch_stage_kernel(ns_batch* b, int set, int stage, bool first, cudaStream_t st) {
  const ns_batch_config& c = b->cfg;
  const int v = set == 0 ? 1 : 0;
  const bool loop = c.mode == 1;
  const std::vector<int>& act = b->active[set];
  const int* slots = b->dev_slots + (size_t)set * b->n * 6;
  const double* wts = b->dev_wts + (size_t)set * b->n * 6;
  const int nparts = loop ? (int)act.size() : 1;
  const int pass_of[5] = {0, 2, 4, 3, 1};  // x fwd, y fwd, z solve, y inv, x inv
  for (int k = 0; k < nparts; ++k) {
    const ns_batch::Range& r = loop ? b->sub_rng[set][stage][act[k]] : b->rng[set][stage];
    const BatchItem* p = b->d_items + r.off;
    const int cnt = r.cnt;
    if (cnt <= 0) continue;
    const int want = c.grid[stage];
    const int grid = persistent_grid(want, cnt);
    cudaError_t e = cudaSuccess;
    switch (stage) {
      case ST_INTERP:
        interp_kernel<<<grid, kChunk, 0, st>>>(b->d_geo, p, cnt, b->snaps, b->slot_stride, b->snap_mean, b->n, slots,
                                               wts);
        e = cudaGetLastError();
        break;
      case ST_PREDICT:
        e = launch_predict_batch(b->d_pred[v], p, cnt, c.scheme, first, c.dp_flag != 0, want > 0 ? grid : 0, st);
        break;
      case ST_HIST:
        hist_kernel<<<grid, kChunk, 0, st>>>(b->d_geo, p, cnt);
        e = cudaGetLastError();
        break;
      case ST_VBC_X: case ST_VBC_Y: case ST_VBC_Z:  // AB2-CN: the ADI sweeps take these slots
        if (c.scheme == NS_AB2_CN) e = launch_adi_batch(stage - ST_VBC_X, b->d_adi, p, cnt, grid, st);
        else e = launch_bc_batch(stage - ST_VBC_X, false, b->d_bc, p, cnt, grid, st);
        break;
      case ST_PBC_X: case ST_PBC_Y: case ST_PBC_Z:
        e = launch_bc_batch(stage - ST_PBC_X, true, b->d_bc, p, cnt, grid, st);
        break;
      case ST_XF: case ST_YF: case ST_TRI: case ST_YI: case ST_XI: {
        const int pass = pass_of[stage - ST_XF];
        const int nd = r.cnt_dense, nf = cnt - r.cnt_dense;
        if (stage == ST_XF) {
          const ns_batch::Range& dr = loop ? b->sub_div_rng[set][act[k]] : b->div_rng[set];
          if (dr.cnt > 0) {
            e = launch_spec_batch_div(b->d_spec[v], b->d_items + dr.off, dr.cnt, 0, st);
            if (e != cudaSuccess) return e;
            ++b->launches;
          }
          const ns_batch::Range& br = loop ? b->sub_bc_rng[set][act[k]] : b->bc_rng[set];
          if (br.cnt > 0) {
            e = launch_spec_batch_bc(b->d_spec[v], b->d_items + br.off, br.cnt, 0, st);
            if (e != cudaSuccess) return e;
            ++b->launches;
          }
        }
        if (nd > 0)
          e = launch_spec_batch(pass, false, b->d_spec[v], p, nd, b->spec_smem[pass],
                                want > 0 ? persistent_grid(want, nd) : 0, st);
        if (e == cudaSuccess && nf > 0) {
          if (nd > 0) ++b->launches;
          e = launch_spec_batch(pass, true, b->d_spec[v], p + nd, nf, b->spec_smem_dct[pass],
                                want > 0 ? persistent_grid(want, nf) : 0, st);
        }
        break;
      }
      case ST_CORRECT:
        e = launch_correct_batch(b->d_corr[v], p, cnt, grid, st);
        break;
      default:
        break;
    }
    if (e != cudaSuccess) return e;
    ++b->launches;
  }
  return cudaSuccess;
}

const int kStageOrder[] = {ST_INTERP, ST_PREDICT, ST_HIST,  ST_VBC_X, ST_VBC_Y, ST_VBC_Z, ST_XF,      ST_YF,
                           ST_TRI,    ST_YI,      ST_XI,    ST_PBC_X, ST_PBC_Y, ST_PBC_Z, ST_CORRECT};

// Enqueue one (sub-)step of the subdomains of active set `set`.
int enqueue_stage(ns_batch* b, int set, bool first, cudaStream_t st) {
  for (int stage : kStageOrder) {
    if (stage == ST_HIST && set == 0) continue;
    cudaError_t e = launch_stage_kernel(b, set, stage, first, st);
    if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string(kStageName[stage]) + ": " + cudaGetErrorString(e));
  }
  return NS_OK;
}

// Run one stage sequence, through a cached graph when enabled.
int run_stage(ns_batch* b, int set, bool first) {
  if (!b->cfg.use_graph) return enqueue_stage(b, set, first, b->stream);
  const int key = set * 2 + (first ? 1 : 0);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    const long long l0 = b->launches;
    NB_CUDA(b, cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    int s = enqueue_stage(b, set, first, b->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    if (s) { if (g) cudaGraphDestroy(g); return s; }
    if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    it = b->graphs.emplace(key, ex).first;
    b->graph_count[key] = b->launches - l0;  // kernels per replay
    b->launches = l0;
  }
  NB_CUDA(b, cudaGraphLaunch(it->second, b->stream));
  b->launches += b->graph_count[key];
  return NS_OK;
}

}  // namespace

namespace {

size_t align32(size_t n) { return (n + 31) & ~size_t(31); }

int field_ext(const Layout& L, int field, int axis) {
  const int n = axis == 0 ? L.nx : (axis == 1 ? L.ny : L.nz);
  return field == axis ? n + 1 : n + 2;
}
// Host array of a subdomain field (reference shape) <-> padded device field.
cudaError_t box_copy(const Layout& L, double* dev, double* host, int field, bool to_dev, cudaStream_t st) {
  const int ex = field_ext(L, field, 0), ey = field_ext(L, field, 1), ez = field_ext(L, field, 2);
  cudaMemcpy3DParms prm{};
  cudaPitchedPtr hp = make_cudaPitchedPtr((void*)host, ex * sizeof(double), ex, ey);
  cudaPitchedPtr dpp = make_cudaPitchedPtr((void*)(dev + L.off), L.px * sizeof(double), L.px, L.ny + 2);
  const cudaPos pos = make_cudaPos((field == 0 ? 1 : 0) * sizeof(double), field == 1 ? 1 : 0, field == 2 ? 1 : 0);
  if (to_dev) { prm.srcPtr = hp; prm.dstPtr = dpp; prm.dstPos = pos; prm.kind = cudaMemcpyHostToDevice; }
  else { prm.srcPtr = dpp; prm.srcPos = pos; prm.dstPtr = hp; prm.kind = cudaMemcpyDeviceToHost; }
  prm.extent = make_cudaExtent(ex * sizeof(double), ey, ez);
  return cudaMemcpy3DAsync(&prm, st);
}

// Window of 6 knots around t and the spline weights (exact at a knot).
int window_weights(const std::vector<std::pair<double, int>>& knots, double t, double tol, int* slots, double* w) {
  const int nk = (int)knots.size();
  int K = -1;
  for (int i = 0; i < nk; ++i)
    if (knots[i].first <= t + tol) K = i;
  if (K < 0) return NS_ERR_ARG;
  if (std::fabs(t - knots[K].first) <= tol) {  // at a knot the spline returns the data
    const int s = std::max(0, std::min(K - 2, nk - 6));
    for (int q = 0; q < 6; ++q) {
      const int kk = std::min(nk - 1, s + q);
      slots[q] = knots[kk].second;
      w[q] = 0.0;
    }
    for (int q = 0; q < 6; ++q)
      if (s + q == K) w[q] = 1.0;
    if (nk < 6) {  // fewer than 6 snapshots: pad with the knot itself
      for (int q = 0; q < 6; ++q) { slots[q] = knots[K].second; w[q] = q == 0 ? 1.0 : 0.0; }
    }
    return NS_OK;
  }
  const int s = K - 2;
  if (s < 0 || s + 5 >= nk) return NS_ERR_ARG;
  double x[6];
  for (int q = 0; q < 6; ++q) { x[q] = knots[s + q].first; slots[q] = knots[s + q].second; }
  return spline6_weights(x, t, w) ? NS_OK : NS_ERR_ARG;
}

}  // namespace

extern "C" {

void ns_batch_config_default(ns_batch_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->scheme = NS_AB2;
  c->bc = 2;
  c->pbc = 3;
  c->restart = 0;
  c->n_slots = 16;
  c->mode = 0;
  c->use_graph = 1;
  c->using_ustar = 1;
  c->dp_flag = 1;
}

const char* ns_batch_last_error(const ns_batch* b) { return b ? b->err.c_str() : "null batch"; }

int ns_batch_destroy(ns_batch* b) {
  if (!b) return NS_ERR_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  if (b->arena) cudaFree(b->arena);
  if (b->tables) cudaFree(b->tables);
  if (b->adi_tab) cudaFree(b->adi_tab);
  if (b->tri_tab) cudaFree(b->tri_tab);
  if (b->snaps) cudaFree(b->snaps);
  if (b->snap_mean) cudaFree(b->snap_mean);
  if (b->p_prev) cudaFree(b->p_prev);
  if (b->dev_args) cudaFree(b->dev_args);
  if (b->dev_slots) cudaFree(b->dev_slots);
  if (b->dev_wts) cudaFree(b->dev_wts);
  if (b->host_slots) cudaFreeHost(b->host_slots);
  if (b->host_wts) cudaFreeHost(b->host_wts);
  if (b->copy_done) cudaEventDestroy(b->copy_done);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  delete b;
  return NS_OK;
}

// The tables of an FFT-based DCT line of N points as (re, im) pairs: the
// N-point twiddles exp(-2 pi i m / N), m < N, the forward post-twiddles
// exp(-i pi k / (2N)) / 2, k <= N, and the inverse pre-twiddles
// exp(i pi k / (2N)) / N, k < N; computed in long double.
static void append_dct_tables(int N, std::vector<double>& tab) {
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int m = 0; m < N; ++m) {
    const long double th = 2.0L * pi * (long double)m / (long double)N;
    tab.push_back((double)cosl(th));
    tab.push_back((double)(-sinl(th)));
  }
  for (int k = 0; k <= N; ++k) {
    const long double th = pi * (long double)k / (2.0L * N);
    tab.push_back((double)(cosl(th) / 2.0L));
    tab.push_back((double)(-sinl(th) / 2.0L));
  }
  for (int k = 0; k < N; ++k) {
    const long double th = pi * (long double)k / (2.0L * N);
    tab.push_back((double)(cosl(th) / N));
    tab.push_back((double)(sinl(th) / N));
  }
}

int ns_batch_create(const ns_batch_config* cfg, const ns_subdomain* subs, int n, ns_batch** out) {
  if (!cfg || !subs || n <= 0 || !out) return NS_ERR_ARG;
  *out = nullptr;
  const ns_batch_config& c = *cfg;
  std::string msg;
  if (c.scheme != NS_EULER && c.scheme != NS_AB2 && c.scheme != NS_AB2_CN) msg = "batched scheme must be Euler, AB2 or AB2-CN";
  else if (c.scheme == NS_AB2_CN && !c.using_ustar)
    msg = "AB2-CN re-simulation takes the parent's u* faces of every sweep (using_ustar = 1)";
  else if (c.bc != 2 && c.bc != 4) msg = "batched velocity bc must be 2 or 4";
  else if (c.pbc < 2 || c.pbc > 4) msg = "batched pressure bc must be 2, 3 or 4";
  else if (c.n_slots < 1) msg = "n_slots must be >= 1";
  else if ((c.using_ustar != 0 && c.using_ustar != 1) || (c.dp_flag != 0 && c.dp_flag != 1))
    msg = "using_ustar and dp_flag are 0 or 1";
  else if (!(c.dt0 > 0) || !(c.nu >= 0) || !(c.dx > 0) || !(c.dy > 0) || !(c.dz > 0)) msg = "nu, dt0, dx, dy, dz";
  for (int i = 0; i < n && msg.empty(); ++i) {
    const ns_subdomain& d = subs[i];
    if (d.nx < 4 || d.ny < 4 || d.nz < 4 || d.nx % 2 || d.nx > 1024 || d.ny > 128 || d.nz > 256)
      msg = "subdomain sizes: nx even <= 1024, ny <= 128, nz <= 256, all >= 4";
    else if (d.sub_tstep < 1 || (d.sub_tstep > 1 && c.scheme != NS_AB2))
      msg = "sub_tstep >= 1 (> 1 only with AB2, re_simulation_sub_tstep_interBC_combine.f90:356-359)";
    else if (d.x0 < 1 || d.y0 < 1 || d.z0 < 1) msg = "subdomain origins are 1-based";
    else if (!c.using_ustar && d.sub_tstep != 1)
      msg = "sub_tstep > 1 needs u* boundary values (re_simulation_sub_tstep_interBC_combine.f90:360-363)";
  }
  if (!msg.empty()) {
    std::fprintf(stderr, "ns_batch_create: %s\n", msg.c_str());
    return NS_ERR_ARG;
  }
  ns_batch* b = new ns_batch();
  b->cfg = c;
  b->n = n;
  b->desc.assign(subs, subs + n);
  auto bail = [&](int code) {
    std::fprintf(stderr, "ns_batch_create: %s\n", b->err.c_str());
    ns_batch_destroy(b);
    return code;
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(NS_ERR_CUDA);
  b->own_stream = true;
  if (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(NS_ERR_CUDA);
  if (cudaEventCreateWithFlags(&b->copy_done, cudaEventDisableTiming) != cudaSuccess) return bail(NS_ERR_CUDA);
  for (int i = 0; i < n; ++i) b->max_r = std::max(b->max_r, subs[i].sub_tstep);

  // ---- field arena ----
  b->L.resize(n);
  b->geo.resize(n);
  b->plan.resize(n);
  std::vector<size_t> base(n);
  size_t tot = 0;
  for (int i = 0; i < n; ++i) {
    const ns_subdomain& d = subs[i];
    b->L[i] = make_layout(d.nx, d.ny, d.nz);
    base[i] = tot;
    const size_t fs = align32(b->L[i].fsize);
    tot += 14 * fs;                                                  // 11 fields + saved history
    tot += align32((size_t)(d.nx / 2) * d.ny * d.nz * 2);           // packed spectrum
    tot += align32((size_t)face_doubles(b->L[i], c.scheme == NS_AB2_CN));  // current faces
    tot += 32;                                                       // mean dp
  }
  b->arena_n = tot;
  if (cudaMalloc(&b->arena, tot * sizeof(double)) != cudaSuccess) { b->err = "arena"; return bail(NS_ERR_NOMEM); }
  if (cudaMemsetAsync(b->arena, 0, tot * sizeof(double), b->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  long long snap_tot = 0;
  for (int i = 0; i < n; ++i) {
    const Layout& L = b->L[i];
    const size_t fs = align32(L.fsize);
    double* p = b->arena + base[i];
    SubGeo& g = b->geo[i];
    g.L = L;
    g.x0 = subs[i].x0; g.y0 = subs[i].y0; g.z0 = subs[i].z0;
    // fields 0-6: u v w p hx hy hz; 7-10: u* v* w* dp; 11-13: saved history; then the spectrum
    for (int f = 0; f < 7; ++f) g.fld[f] = p + f * fs;
    for (int f = 0; f < 3; ++f) g.save[f] = p + (11 + f) * fs;
    double* face = p + 14 * fs + align32((size_t)(L.nx / 2) * L.ny * L.nz * 2);
    g.face = face;
    g.face_n = face_doubles(L, c.scheme == NS_AB2_CN);
    g.mean = face + align32((size_t)g.face_n);
    g.snap_off = snap_tot;
    snap_tot += (long long)align32((size_t)g.face_n);
  }
  b->slot_stride = snap_tot;
  if (cudaMalloc(&b->snaps, (size_t)c.n_slots * snap_tot * sizeof(double)) != cudaSuccess) {
    b->err = "snapshots";
    return bail(NS_ERR_NOMEM);
  }
  if (cudaMalloc(&b->snap_mean, (size_t)c.n_slots * n * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  cudaMemsetAsync(b->snaps, 0, (size_t)c.n_slots * snap_tot * sizeof(double), b->stream);
  cudaMemsetAsync(b->snap_mean, 0, (size_t)c.n_slots * n * sizeof(double), b->stream);
  b->snap_t.assign(c.n_slots, 0.0);
  b->snap_ok.assign(c.n_slots, 0);

  // ---- size-class tables: dense x (transposed) and y pairs, x and y eigenvalues ----
  std::vector<double> tab;
  std::map<int, size_t> xF, xG, yF, yG, ex, ey;
  std::map<int, int> ysym, xsym;  // symmetry bits of the y and x pairs per size
  // FFT-based DCT tables of the axes of 24, 32, 48 and 64 points (pressure
  // codes 2 and 3; NS_DENSE_X / NS_DENSE_Y keep the dense products): the
  // N-point twiddles exp(-2 pi i m / N), m < N, then exp(-i pi k / (2N)) / 2,
  // k <= N, then exp(i pi k / (2N)) / N, k < N, as (re, im) pairs.
  std::map<int, size_t> dtab;
  const bool dct_code = c.pbc == 2 || c.pbc == 3;
  auto dct_size = [](int m) { return m == 24 || m == 32 || m == 48 || m == 64; };
  auto add_dct = [&](int N) {
    if (dtab.count(N)) return;
    dtab[N] = tab.size();
    append_dct_tables(N, tab);
    tab.resize(align32(tab.size()));
  };
  const bool dct_x_on = dct_code && !std::getenv("NS_DENSE_X"), dct_y_on = dct_code && !std::getenv("NS_DENSE_Y");
  for (int i = 0; i < n; ++i) {
    if (dct_x_on && dct_size(subs[i].nx)) add_dct(subs[i].nx);
    if (dct_y_on && dct_size(subs[i].ny)) add_dct(subs[i].ny);
  }
  for (int i = 0; i < n; ++i) {
    const int nx = subs[i].nx, ny = subs[i].ny;
    if (!xF.count(nx)) {
      std::vector<double> F, G;
      dense_pair(nx, c.pbc, F, G);
      xsym[nx] = dense_symmetry(nx, F, G);
      std::vector<double> Ft((size_t)nx * nx), Gt((size_t)nx * nx);
      for (int r = 0; r < nx; ++r)
        for (int q = 0; q < nx; ++q) { Ft[(size_t)q * nx + r] = F[(size_t)r * nx + q]; Gt[(size_t)q * nx + r] = G[(size_t)r * nx + q]; }
      xF[nx] = tab.size(); tab.insert(tab.end(), Ft.begin(), Ft.end()); tab.resize(align32(tab.size()));
      xG[nx] = tab.size(); tab.insert(tab.end(), Gt.begin(), Gt.end()); tab.resize(align32(tab.size()));
      ex[nx] = tab.size();
      for (int m = 0; m < nx; ++m) tab.push_back(-4.0 * axis_eig(nx, c.pbc, m, c.dx));
      tab.resize(align32(tab.size()));
    }
    if (!yF.count(ny)) {
      std::vector<double> F, G;
      dense_pair(ny, c.pbc, F, G);
      ysym[ny] = dense_symmetry(ny, F, G);
      yF[ny] = tab.size(); tab.insert(tab.end(), F.begin(), F.end()); tab.resize(align32(tab.size()));
      yG[ny] = tab.size(); tab.insert(tab.end(), G.begin(), G.end()); tab.resize(align32(tab.size()));
      ey[ny] = tab.size();
      for (int m = 0; m < ny; ++m) tab.push_back(-4.0 * axis_eig(ny, c.pbc, m, c.dy));
      tab.resize(align32(tab.size()));
    }
  }
  if (cudaMalloc(&b->tables, tab.size() * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMemcpyAsync(b->tables, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream) !=
      cudaSuccess)
    return bail(NS_ERR_CUDA);

  // z-solve multiplier tables, laid out like each subdomain's spectrum
  std::vector<size_t> tri_off(n);
  {
    size_t t = 0;
    for (int i = 0; i < n; ++i) {
      tri_off[i] = t;
      t += align32((size_t)(subs[i].nx / 2) * subs[i].ny * subs[i].nz);
    }
    if (cudaMalloc(&b->tri_tab, std::max<size_t>(t, 1) * sizeof(double2)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  }

  // ---- per-subdomain plans and argument tables ----
  const double hs[3] = {c.dx, c.dy, c.dz};
  const int bc3[3] = {c.bc, c.bc, c.bc};
  // AB2-CN: the factors of mat_CN_tridiagonal (NS_functions.f90:1296-1342) per
  // (sweep axis, cells along it, normal / tangential), shared by the
  // subdomains of the same size; sub_tstep is 1, so every step uses dt0.
  const bool cn = c.scheme == NS_AB2_CN;
  std::map<long long, LineSys> line_sys;
  if (cn) {
    constexpr int pad = 8;
    std::vector<HostLineSys> hsys;
    std::vector<long long> keys;
    for (int i = 0; i < n; ++i) {
      const int n3[3] = {subs[i].nx, subs[i].ny, subs[i].nz};
      for (int a = 0; a < 3; ++a)
        for (int normal = 0; normal < 2; ++normal) {
          const long long key = ((long long)a * 4096 + n3[a]) * 2 + normal;
          if (line_sys.count(key)) continue;
          line_sys[key] = LineSys{};
          keys.push_back(key);
          hsys.push_back(build_cn_system(n3[a], c.bc, hs[a], c.dt0, c.nu, normal != 0, 0));
        }
    }
    size_t total = 0;
    for (const HostLineSys& S : hsys) total += 3 * (S.l.size() + 2 * pad);
    std::vector<double> host(std::max<size_t>(total, 1), 0.0);
    if (cudaMalloc(&b->adi_tab, host.size() * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
    size_t off = 0;
    for (size_t q = 0; q < hsys.size(); ++q) {
      const HostLineSys& S = hsys[q];
      LineSys& D = line_sys[keys[q]];
      const size_t m = S.l.size(), mp = m + 2 * pad;
      std::memcpy(&host[off + pad], S.l.data(), m * sizeof(double)); D.l = b->adi_tab + off; off += mp;
      std::memcpy(&host[off + pad], S.dinv.data(), m * sizeof(double)); D.dinv = b->adi_tab + off; off += mp;
      std::memcpy(&host[off + pad], S.cu.data(), m * sizeof(double)); D.cu = b->adi_tab + off; off += mp;
      D.z = nullptr; D.s0 = D.s1 = 0.0; D.zA = D.zB = 0;
      D.lo = S.lo; D.hi = S.hi; D.periodic = 0; D.n = S.n; D.pad = pad;
    }
    if (cudaMemcpyAsync(b->adi_tab, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream) !=
        cudaSuccess)
      return bail(NS_ERR_CUDA);
  }
  std::vector<BatchAdiArgs> adia(cn ? n : 0);
  std::vector<PredictArgs> pred[2];
  std::vector<BatchSpecArgs> spec[2];
  std::vector<CorrectArgs> corr[2];
  std::vector<BatchBcArgs> bca(n);
  for (int v = 0; v < 2; ++v) { pred[v].resize(n); spec[v].resize(n); corr[v].resize(n); }
  for (int i = 0; i < n; ++i) {
    const ns_subdomain& d = subs[i];
    const Layout& L = b->L[i];
    SubGeo& g = b->geo[i];
    const size_t fs = align32(L.fsize);
    double* p = b->arena + base[i];
    double* us = p + 7 * fs; double* vs = p + 8 * fs; double* ws = p + 9 * fs; double* dp = p + 10 * fs;
    double2* specp = reinterpret_cast<double2*>(p + 14 * fs);
    // face planes of this subdomain: [axis][field][side]
    FaceSet F{};
    {
      size_t off = 0;
      for (int a = 0; a < 3; ++a)
        for (int f = 0; f < 4; ++f)
          for (int s = 0; s < 2; ++s) {
            F.ax[a].f[f][s] = g.face + off;
            off += (size_t)plane_n1(L, a) * plane_n2(L, a);
          }
    }
    SpecPlan& S = b->plan[i];
    S = SpecPlan{};
    S.nx = d.nx; S.ny = d.ny; S.nz = d.nz; S.nxh = d.nx / 2 + 1; S.nxs = d.nx / 2;
    S.kind[0] = 1; S.kind[1] = 1; S.kind[2] = 2;
    S.fwd[0] = b->tables + xF[d.nx]; S.inv[0] = b->tables + xG[d.nx];
    S.fwd[1] = b->tables + yF[d.ny]; S.inv[1] = b->tables + yG[d.ny];
    S.sym[1] = ysym[d.ny];
    S.sym[0] = xsym[d.nx];
    S.eig_x = b->tables + ex[d.nx];
    S.eig_o = b->tables + ey[d.ny];
    if (dct_x_on && dct_size(d.nx)) {
      const double2* t2 = reinterpret_cast<const double2*>(b->tables + dtab[d.nx]);
      S.dct_x = c.pbc;
      S.dctx_tw = t2; S.dctx_wf = t2 + d.nx; S.dctx_wi = t2 + 2 * d.nx + 1;
    }
    if (dct_y_on && dct_size(d.ny)) {
      const double2* t2 = reinterpret_cast<const double2*>(b->tables + dtab[d.ny]);
      S.dct_y = c.pbc;
      S.dct_tw = t2; S.dct_wf = t2 + d.ny; S.dct_wi = t2 + 2 * d.ny + 1;
    }
    S.tri_h2 = c.dz * c.dz;
    S.tri_rs = c.dz * c.dz;
    S.tri_elo = S.tri_ehi = c.pbc == 2 ? -1.0 : (c.pbc == 3 ? 1.0 : 0.0);
    S.has_mean = c.pbc == 3 ? 1 : 0;
    S.mean_val = (double)d.nx * (double)d.ny;
    S.mean_dev = g.mean;
    if (launch_tri_twist_table(2, S, b->tri_tab + tri_off[i], b->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
    S.tri_m = b->tri_tab + tri_off[i];
    S.tri_tw = 1;
    for (int a = 0; a < 3; ++a) {
      const double hh = hs[a];
      if (c.pbc == 2) { S.mod_lo[a] = -2.0 / (hh * hh); S.mod_hi[a] = -2.0 / (hh * hh); }
      else if (c.pbc == 3) { S.mod_lo[a] = 1.0 / hh; S.mod_hi[a] = -1.0 / hh; }
      else { S.mod_lo[a] = -1.0 / (hh * hh); S.mod_hi[a] = -1.0 / (hh * hh); }
      S.face_lo[a] = F.ax[a].f[3][0];
      S.face_hi[a] = F.ax[a].f[3][1];
    }
    for (int v = 0; v < 2; ++v) {
      const double dt = v == 0 ? c.dt0 / d.sub_tstep : c.dt0;
      PredictArgs& a = pred[v][i];
      a = PredictArgs{};
      a.L = L;
      a.u = g.fld[0]; a.v = g.fld[1]; a.w = g.fld[2]; a.p = g.fld[3];
      a.us = us; a.vs = vs; a.ws = ws;
      a.hx = g.fld[4]; a.hy = g.fld[5]; a.hz = g.fld[6];
      set_predict_coeffs(a, bc3, c.dx, c.dy, c.dz, dt, c.nu);
      BatchSpecArgs& sa = spec[v][i];
      sa = BatchSpecArgs{};
      sa.S = S;
      sa.d.L = L; sa.d.us = us; sa.d.vs = vs; sa.d.ws = ws;
      sa.d.cdx = 1.0 / (c.dx * dt); sa.d.cdy = 1.0 / (c.dy * dt); sa.d.cdz = 1.0 / (c.dz * dt);
      sa.d.one = 1.0; sa.d.mzero = -0.0; sa.d.rhs = nullptr;
      sa.spec = specp; sa.dp = dp; sa.L = L;
      CorrectArgs& ca = corr[v][i];
      ca = CorrectArgs{};
      ca.L = L; ca.us = us; ca.vs = vs; ca.ws = ws; ca.dp = dp;
      ca.u = g.fld[0]; ca.v = g.fld[1]; ca.w = g.fld[2]; ca.p = g.fld[3];
      ca.gx = -dt / c.dx; ca.gy = -dt / c.dy; ca.gz = -dt / c.dz;
      ca.dp_flag = c.dp_flag; ca.gauge = 0;
      ca.per[0] = ca.per[1] = ca.per[2] = 0;
      ca.one = 1.0; ca.mzero = -0.0;
    }
    BatchBcArgs& ba = bca[i];
    ba = BatchBcArgs{};
    ba.L = L; ba.us = us; ba.vs = vs; ba.ws = ws; ba.dp = dp; ba.F = F;
    for (int a = 0; a < 3; ++a) { ba.bc[a] = c.bc; ba.pbc[a] = c.pbc; ba.h[a] = hs[a]; }
    if (cn) {
      BatchAdiArgs& aa = adia[i];
      aa = BatchAdiArgs{};
      aa.L = L;
      aa.f[0] = us; aa.f[1] = vs; aa.f[2] = ws;
      const int n3[3] = {d.nx, d.ny, d.nz};
      for (int a = 0; a < 3; ++a)
        for (int f = 0; f < 3; ++f) {
          aa.sys[a][f] = line_sys[((long long)a * 4096 + n3[a]) * 2 + (f == a ? 1 : 0)];
          aa.face_lo[a][f] = g.face + sweep_face_off(L, a, f, 0);
          aa.face_hi[a][f] = g.face + sweep_face_off(L, a, f, 1);
        }
    }
  }
  for (int pass = 0; pass < 5; ++pass)
    for (int i = 0; i < n; ++i) {
      size_t& sm = spec_pass_dct(pass, b->plan[i]) ? b->spec_smem_dct[pass] : b->spec_smem[pass];
      sm = std::max(sm, spec_pass_smem(pass, b->plan[i]));
    }

  // ---- work items ----
  auto chunks = [](long long e) { return (int)((e + kChunk - 1) / kChunk); };
  auto sub_items = [&](int i, int stage, int set) {
    std::vector<BatchItem> v;
    const Layout& L = b->L[i];
    auto add1 = [&](int cnt, int bz) { for (int q = 0; q < cnt; ++q) v.push_back(BatchItem{i, q, 0, bz}); };
    switch (stage) {
      case ST_INTERP: add1(chunks(b->geo[i].face_n), 0); break;
      case ST_PREDICT: {
        int gx, gy, gz;
        predict_tiles(L, gx, gy, gz);
        for (int z = 0; z < gz; ++z)
          for (int y = 0; y < gy; ++y)
            for (int x = 0; x < gx; ++x) v.push_back(BatchItem{i, x, y, z});
        break;
      }
      case ST_VBC_X: case ST_VBC_Y: case ST_VBC_Z:
        if (c.scheme == NS_AB2_CN) {  // the ADI sweep: 128-line chunks of each field
          const int nl = plane_count(L, stage - ST_VBC_X);
          for (int f = 0; f < 3; ++f)
            for (int q = 0; q < (nl + kAdiBatchLines - 1) / kAdiBatchLines; ++q) v.push_back(BatchItem{i, q, f, 0});
        } else {
          add1(chunks(plane_count(L, stage - ST_VBC_X)), 0);
        }
        break;
      case ST_PBC_X: case ST_PBC_Y: case ST_PBC_Z: add1(chunks(plane_count(L, stage - ST_PBC_X)), 0); break;
      case ST_XF: case ST_YF: case ST_TRI: case ST_YI: case ST_XI: {
        const int pass_of[5] = {0, 2, 4, 3, 1};
        int gx, gy;
        spec_pass_grid(pass_of[stage - ST_XF], b->plan[i], gx, gy);
        for (int y = 0; y < gy; ++y)
          for (int x = 0; x < gx; ++x) v.push_back(BatchItem{i, x, y, 0});
        break;
      }
      case ST_CORRECT: add1(chunks((long long)(L.nx + 2) * (L.ny + 2) * (L.nz + 2)), 0); break;
      case ST_HIST: {
        const int r = subs[i].sub_tstep;
        int op = 0;
        if (set >= 1 && r > 1) op = set == 1 ? 1 : (set == r ? 2 : 0);
        if (op) add1(chunks(L.fsize), op);
        break;
      }
    }
    return v;
  };
  std::vector<BatchItem> all;
  const int nsets = b->max_r + 1;
  b->active.assign(nsets, {});
  for (int set = 0; set < nsets; ++set)
    for (int i = 0; i < n; ++i)
      if (set == 0 || subs[i].sub_tstep >= set) b->active[set].push_back(i);
  b->rng.assign(nsets, std::vector<ns_batch::Range>(ST_COUNT));
  b->sub_rng.assign(nsets, std::vector<std::vector<ns_batch::Range>>(ST_COUNT, std::vector<ns_batch::Range>(n)));
  // A spectral stage lists the subdomains of its dense kernel first, then
  // those of its FFT-based kernel.
  auto stage_dct = [&](int st, int i) {
    const int pass_of[5] = {0, 2, 4, 3, 1};
    return st >= ST_XF && st <= ST_XI && spec_pass_dct(pass_of[st - ST_XF], b->plan[i]);
  };
  for (int set = 0; set < nsets; ++set)
    for (int st = 0; st < ST_COUNT; ++st) {
      b->rng[set][st].off = (long long)all.size();
      for (int group = 0; group < 2; ++group) {
        for (int i : b->active[set]) {
          const bool dct = stage_dct(st, i);
          if ((int)dct != group) continue;
          std::vector<BatchItem> v = sub_items(i, st, set);
          b->sub_rng[set][st][i].off = (long long)all.size();
          b->sub_rng[set][st][i].cnt = (int)v.size();
          b->sub_rng[set][st][i].cnt_dense = dct ? 0 : (int)v.size();
          all.insert(all.end(), v.begin(), v.end());
        }
        if (group == 0) b->rng[set][st].cnt_dense = (int)((long long)all.size() - b->rng[set][st].off);
      }
      b->rng[set][st].cnt = (int)((long long)all.size() - b->rng[set][st].off);
    }
  b->div_rng.assign(nsets, ns_batch::Range{});
  b->sub_div_rng.assign(nsets, std::vector<ns_batch::Range>(n));
  for (int set = 0; set < nsets; ++set) {
    b->div_rng[set].off = (long long)all.size();
    for (int i : b->active[set]) {
      if (!stage_dct(ST_XF, i)) continue;
      const Layout& L = b->L[i];
      const long long ne = (long long)L.nx * L.ny * L.nz;
      const int nq = (int)((ne + kDivChunk - 1) / kDivChunk);
      b->sub_div_rng[set][i].off = (long long)all.size();
      b->sub_div_rng[set][i].cnt = nq;
      for (int q = 0; q < nq; ++q) all.push_back(BatchItem{i, q, 0, 0});
    }
    b->div_rng[set].cnt = (int)((long long)all.size() - b->div_rng[set].off);
  }
  b->bc_rng.assign(nsets, ns_batch::Range{});
  b->sub_bc_rng.assign(nsets, std::vector<ns_batch::Range>(n));
  for (int set = 0; set < nsets; ++set) {
    b->bc_rng[set].off = (long long)all.size();
    for (int i : b->active[set]) {
      if (!stage_dct(ST_XF, i) || !b->plan[i].any_bc_term()) continue;
      const long long nbc = b->plan[i].bc_cells();
      const int nq = (int)((nbc + kDivChunk - 1) / kDivChunk);
      b->sub_bc_rng[set][i].off = (long long)all.size();
      b->sub_bc_rng[set][i].cnt = nq;
      for (int q = 0; q < nq; ++q) all.push_back(BatchItem{i, q, 0, 0});
    }
    b->bc_rng[set].cnt = (int)((long long)all.size() - b->bc_rng[set].off);
  }
  b->gather_rng.off = (long long)all.size();
  for (int i = 0; i < n; ++i) {
    std::vector<BatchItem> v = sub_items(i, ST_CORRECT, 0);
    all.insert(all.end(), v.begin(), v.end());
  }
  b->gather_rng.cnt = (int)((long long)all.size() - b->gather_rng.off);
  b->capture_rng.off = (long long)all.size();
  for (int i = 0; i < n; ++i) {
    std::vector<BatchItem> v = sub_items(i, ST_INTERP, 0);
    all.insert(all.end(), v.begin(), v.end());
  }
  b->capture_rng.cnt = (int)((long long)all.size() - b->capture_rng.off);

  // ---- one device buffer for the argument tables and the items ----
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t o = 0;
  const size_t o_geo = o; o = al(o + n * sizeof(SubGeo));
  const size_t o_pred = o; o = al(o + 2 * n * sizeof(PredictArgs));
  const size_t o_spec = o; o = al(o + 2 * n * sizeof(BatchSpecArgs));
  const size_t o_corr = o; o = al(o + 2 * n * sizeof(CorrectArgs));
  const size_t o_bc = o; o = al(o + n * sizeof(BatchBcArgs));
  const size_t o_adi = o; o = al(o + adia.size() * sizeof(BatchAdiArgs));
  const size_t o_items = o; o = al(o + all.size() * sizeof(BatchItem));
  std::vector<unsigned char> hbuf(o, 0);
  std::memcpy(hbuf.data() + o_geo, b->geo.data(), n * sizeof(SubGeo));
  for (int v = 0; v < 2; ++v) {
    std::memcpy(hbuf.data() + o_pred + v * n * sizeof(PredictArgs), pred[v].data(), n * sizeof(PredictArgs));
    std::memcpy(hbuf.data() + o_spec + v * n * sizeof(BatchSpecArgs), spec[v].data(), n * sizeof(BatchSpecArgs));
    std::memcpy(hbuf.data() + o_corr + v * n * sizeof(CorrectArgs), corr[v].data(), n * sizeof(CorrectArgs));
  }
  std::memcpy(hbuf.data() + o_bc, bca.data(), n * sizeof(BatchBcArgs));
  if (!adia.empty()) std::memcpy(hbuf.data() + o_adi, adia.data(), adia.size() * sizeof(BatchAdiArgs));
  std::memcpy(hbuf.data() + o_items, all.data(), all.size() * sizeof(BatchItem));
  if (cudaMalloc(&b->dev_args, o) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMemcpyAsync(b->dev_args, hbuf.data(), o, cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
    return bail(NS_ERR_CUDA);
  b->d_geo = reinterpret_cast<SubGeo*>(b->dev_args + o_geo);
  for (int v = 0; v < 2; ++v) {
    b->d_pred[v] = reinterpret_cast<PredictArgs*>(b->dev_args + o_pred) + v * n;
    b->d_spec[v] = reinterpret_cast<BatchSpecArgs*>(b->dev_args + o_spec) + v * n;
    b->d_corr[v] = reinterpret_cast<CorrectArgs*>(b->dev_args + o_corr) + v * n;
  }
  b->d_bc = reinterpret_cast<BatchBcArgs*>(b->dev_args + o_bc);
  b->d_adi = adia.empty() ? nullptr : reinterpret_cast<BatchAdiArgs*>(b->dev_args + o_adi);
  b->d_items = reinterpret_cast<BatchItem*>(b->dev_args + o_items);
  // interpolation weights: one region per active set
  const size_t nw = (size_t)nsets * n * 6;
  if (cudaMalloc(&b->dev_slots, nw * sizeof(int)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMalloc(&b->dev_wts, nw * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMallocHost(&b->host_slots, nw * sizeof(int)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  if (cudaMallocHost(&b->host_wts, nw * sizeof(double)) != cudaSuccess) return bail(NS_ERR_NOMEM);
  cudaMemsetAsync(b->dev_slots, 0, nw * sizeof(int), b->stream);
  cudaMemsetAsync(b->dev_wts, 0, nw * sizeof(double), b->stream);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bail(NS_ERR_CUDA);
  *out = b;
  return NS_OK;
}

int ns_batch_set_stream(ns_batch* b, void* stream) {
  if (!b) return NS_ERR_ARG;
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->own_stream = false;
  b->stream = static_cast<cudaStream_t>(stream);
  return NS_OK;
}

int ns_batch_get_config(const ns_batch* b, ns_batch_config* out) {
  if (!b || !out) return NS_ERR_ARG;
  *out = b->cfg;
  return NS_OK;
}

int ns_batch_init_from_parent(ns_batch* b, const ns_handle* parent) {
  if (!b || !parent) return NS_ERR_ARG;
  const Layout& Lp = parent->L;
  for (int i = 0; i < b->n; ++i) {
    const ns_subdomain& d = b->desc[i];
    if (d.x0 + d.nx > Lp.nx + 1 || d.y0 + d.ny > Lp.ny + 1 || d.z0 + d.nz > Lp.nz + 1)
      return bfail(b, NS_ERR_SHAPE, "subdomain " + std::to_string(i) + " does not fit inside the parent");
  }
  cudaEvent_t ev;
  NB_CUDA(b, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaEventRecord(ev, parent->stream);
  cudaStreamWaitEvent(b->stream, ev, 0);
  const ns_batch::Range& r = b->gather_rng;
  gather_kernel<<<persistent_grid(0, r.cnt), kChunk, 0, b->stream>>>(b->d_geo, b->d_items + r.off, r.cnt, Lp, parent->u,
                                                                      parent->v, parent->w, parent->p, parent->hx,
                                                                      parent->hy, parent->hz);
  ++b->launches;
  cudaError_t e = cudaGetLastError();
  cudaEventRecord(ev, b->stream);
  cudaStreamWaitEvent(parent->stream, ev, 0);
  cudaEventDestroy(ev);
  if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string("gather: ") + cudaGetErrorString(e));
  b->intervals_done = 0;
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  return NS_OK;
}

int ns_batch_set_state(ns_batch* b, int i, const double* u, const double* v, const double* w, const double* p,
                       const double* hx, const double* hy, const double* hz) {
  if (!b || i < 0 || i >= b->n || !u || !v || !w || !p) return NS_ERR_ARG;
  const SubGeo& g = b->geo[i];
  const double* src[7] = {u, v, w, p, hx, hy, hz};
  for (int f = 0; f < 7; ++f) {
    if (src[f]) NB_CUDA(b, box_copy(g.L, g.fld[f], const_cast<double*>(src[f]), f < 4 ? f : f - 4, true, b->stream));
    else NB_CUDA(b, cudaMemsetAsync(g.fld[f], 0, g.L.fsize * sizeof(double), b->stream));
  }
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  b->intervals_done = 0;
  return NS_OK;
}

int ns_batch_get_state(ns_batch* b, int i, double* u, double* v, double* w, double* p, double* hx, double* hy,
                       double* hz) {
  if (!b || i < 0 || i >= b->n) return NS_ERR_ARG;
  const SubGeo& g = b->geo[i];
  double* dst[7] = {u, v, w, p, hx, hy, hz};
  for (int f = 0; f < 7; ++f)
    if (dst[f]) NB_CUDA(b, box_copy(g.L, g.fld[f], dst[f], f < 4 ? f : f - 4, false, b->stream));
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  return NS_OK;
}

int ns_batch_capture(ns_batch* b, const ns_handle* parent, int slot, double t) {
  if (!b || !parent || slot < 0 || slot >= b->cfg.n_slots) return NS_ERR_ARG;
  const Layout& Lp = parent->L;
  for (int i = 0; i < b->n; ++i) {
    const ns_subdomain& d = b->desc[i];
    if (d.x0 + d.nx > Lp.nx + 1 || d.y0 + d.ny > Lp.ny + 1 || d.z0 + d.nz > Lp.nz + 1)
      return bfail(b, NS_ERR_SHAPE, "subdomain " + std::to_string(i) + " does not fit inside the parent");
  }
  const ns_batch_config& c = b->cfg;
  const bool cn = parent->cfg.scheme == NS_AB2_CN;
  const double* pus = c.using_ustar ? (cn ? parent->us2 : parent->us) : parent->u;
  const double* pvs = c.using_ustar ? (cn ? parent->vs2 : parent->vs) : parent->v;
  const double* pws = c.using_ustar ? (cn ? parent->ws2 : parent->ws) : parent->w;
  // pressure source: dp (gauge-shifted as the step shifts it) or p, which holds the shift already
  const double* psrc = c.dp_flag ? parent->dp : parent->p;
  const double* gauge = (c.dp_flag && parent->cfg.gauge) ? parent->dp + Lp.at(0, 0, 0) : nullptr;
  const bool corr = !c.using_ustar && !c.dp_flag;
  SweepSrc sw{};
  if (c.scheme == NS_AB2_CN) {  // u* after the x sweep (kept), after the y sweep (A), after the z sweep (B)
    if (!cn || !parent->us3)
      return bfail(b, NS_ERR_ARG, "an AB2-CN batch captures from an AB2-CN parent created with keep_sweeps = 1");
    const double* after[3][3] = {{parent->us3, parent->vs3, parent->ws3},
                                 {parent->us, parent->vs, parent->ws},
                                 {parent->us2, parent->vs2, parent->ws2}};
    for (int a = 0; a < 3; ++a)
      for (int f = 0; f < 3; ++f) sw.f[a][f] = after[a][f];
  }
  if (corr && b->p_prev_n != Lp.fsize) {  // first capture from this parent: p_prev = the current p
    if (b->p_prev) cudaFree(b->p_prev);
    b->p_prev = nullptr;
    b->p_prev_n = 0;
    NB_CUDA(b, cudaMalloc(&b->p_prev, (size_t)Lp.fsize * sizeof(double)));
    b->p_prev_n = Lp.fsize;
    NB_CUDA(b, cudaStreamSynchronize(parent->stream));
    NB_CUDA(b, cudaMemcpyAsync(b->p_prev, parent->p, (size_t)Lp.fsize * sizeof(double), cudaMemcpyDeviceToDevice,
                               b->stream));
  }
  cudaEvent_t ev;
  NB_CUDA(b, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaEventRecord(ev, parent->stream);
  cudaStreamWaitEvent(b->stream, ev, 0);
  const ns_batch::Range& r = b->capture_rng;
  capture_kernel<<<persistent_grid(0, r.cnt), kChunk, 0, b->stream>>>(
      b->d_geo, b->d_items + r.off, r.cnt, Lp, pus, pvs, pws, psrc, corr ? b->p_prev : nullptr, c.dt0,
      b->snaps + (size_t)slot * b->slot_stride, c.bc, c.pbc, c.dx, c.dy, c.dz, gauge, sw);
  capture_mean_kernel<<<std::min(b->n, 1024), 256, 0, b->stream>>>(b->d_geo, b->n, Lp, psrc,
                                                                   b->snap_mean + (size_t)slot * b->n, gauge);
  if (corr) {  // this capture's p is the next capture's p_previous
    cudaMemcpyAsync(b->p_prev, parent->p, (size_t)Lp.fsize * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
  }
  b->launches += 2;
  cudaError_t e = cudaGetLastError();
  cudaEventRecord(ev, b->stream);
  cudaStreamWaitEvent(parent->stream, ev, 0);  // the parent's next step waits for the capture
  cudaEventDestroy(ev);
  if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  b->snap_t[slot] = t;
  b->snap_ok[slot] = 1;
  return NS_OK;
}

int ns_batch_set_snapshot(ns_batch* b, int slot, double t, int i, const double* const faces[24], double mean_dp) {
  if (!b || !faces || slot < 0 || slot >= b->cfg.n_slots || i < 0 || i >= b->n) return NS_ERR_ARG;
  const SubGeo& g = b->geo[i];
  const Layout& L = g.L;
  std::vector<double> buf((size_t)g.face_n, 0.0);
  // plane offsets [axis][field][side]
  size_t off[3][4][2];
  {
    size_t o = 0;
    for (int a = 0; a < 3; ++a)
      for (int f = 0; f < 4; ++f)
        for (int s = 0; s < 2; ++s) { off[a][f][s] = o; o += (size_t)plane_n1(L, a) * plane_n2(L, a); }
  }
  // get_velpr_bc order: field-major (u, v, w, p), then axis (x, y, z), then side
  for (int k = 0; k < 24; ++k) {
    const double* src = faces[k];
    if (!src) continue;
    const int f = k / 6, a = (k % 6) / 2, s = k % 2;
    const int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
    const int e1 = field_ext(L, f == 3 ? 3 : f, a1), e2 = field_ext(L, f == 3 ? 3 : f, a2);
    const int o1 = f == a1 ? 1 : 0, o2 = f == a2 ? 1 : 0;
    const int n1 = plane_n1(L, a);
    double* plane = buf.data() + off[a][f][s];
    for (int q = 0; q < e2; ++q)
      for (int r = 0; r < e1; ++r) plane[(size_t)(r + o1) + (size_t)n1 * (q + o2)] = src[r + (size_t)e1 * q];
  }
  // the get_velpr_bc planes only: an AB2-CN batch's per-sweep planes are set apart
  NB_CUDA(b, cudaMemcpyAsync(b->snaps + (size_t)slot * b->slot_stride + g.snap_off, buf.data(),
                             (size_t)face_doubles(L) * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  NB_CUDA(b, cudaMemcpyAsync(b->snap_mean + (size_t)slot * b->n + i, &mean_dp, sizeof(double), cudaMemcpyHostToDevice,
                             b->stream));
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  b->snap_t[slot] = t;
  b->snap_ok[slot] = 1;
  return NS_OK;
}

int ns_batch_get_snapshot(ns_batch* b, int slot, int i, double* const faces[24], double* mean_dp) {
  if (!b || !faces || slot < 0 || slot >= b->cfg.n_slots || i < 0 || i >= b->n) return NS_ERR_ARG;
  if (!b->snap_ok[slot]) return bfail(b, NS_ERR_ARG, "snapshot slot " + std::to_string(slot) + " is empty");
  const SubGeo& g = b->geo[i];
  const Layout& L = g.L;
  std::vector<double> buf((size_t)g.face_n, 0.0);
  double m = 0.0;
  NB_CUDA(b, cudaMemcpyAsync(buf.data(), b->snaps + (size_t)slot * b->slot_stride + g.snap_off,
                             buf.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  NB_CUDA(b, cudaMemcpyAsync(&m, b->snap_mean + (size_t)slot * b->n + i, sizeof(double), cudaMemcpyDeviceToHost,
                             b->stream));
  NB_CUDA(b, cudaStreamSynchronize(b->stream));
  size_t off[3][4][2];
  {
    size_t o = 0;
    for (int a = 0; a < 3; ++a)
      for (int f = 0; f < 4; ++f)
        for (int s = 0; s < 2; ++s) { off[a][f][s] = o; o += (size_t)plane_n1(L, a) * plane_n2(L, a); }
  }
  for (int k = 0; k < 24; ++k) {
    double* dst = faces[k];
    if (!dst) continue;
    const int f = k / 6, a = (k % 6) / 2, s = k % 2;
    const int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
    const int e1 = field_ext(L, f, a1), e2 = field_ext(L, f, a2);
    const int o1 = f == a1 ? 1 : 0, o2 = f == a2 ? 1 : 0;
    const int n1 = plane_n1(L, a);
    const double* plane = buf.data() + off[a][f][s];
    for (int q = 0; q < e2; ++q)
      for (int r = 0; r < e1; ++r) dst[r + (size_t)e1 * q] = plane[(size_t)(r + o1) + (size_t)n1 * (q + o2)];
  }
  if (mean_dp) *mean_dp = m;
  return NS_OK;
}

// The per-sweep faces of an AB2-CN batch in the reference's order
// (bx_u_1s, bx_u_nxs, bx_v_1s, bx_v_nxs, bx_w_1s, bx_w_nxs, by_u_1s, ..., bz_w_nzs),
// each in the shape of the get_velpr_bc face of the same name.
static int sweep_faces_copy(ns_batch* b, int slot, int i, double* const* out, const double* const* in) {
  if (!b || slot < 0 || slot >= b->cfg.n_slots || i < 0 || i >= b->n) return NS_ERR_ARG;
  if (b->cfg.scheme != NS_AB2_CN) return bfail(b, NS_ERR_ARG, "per-sweep faces belong to an AB2-CN batch");
  const SubGeo& g = b->geo[i];
  const Layout& L = g.L;
  const long long off0 = face_doubles(L);
  std::vector<double> buf((size_t)(g.face_n - off0), 0.0);
  double* dev = b->snaps + (size_t)slot * b->slot_stride + g.snap_off + off0;
  if (out) {
    if (!b->snap_ok[slot]) return bfail(b, NS_ERR_ARG, "snapshot slot " + std::to_string(slot) + " is empty");
    NB_CUDA(b, cudaMemcpyAsync(buf.data(), dev, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    NB_CUDA(b, cudaStreamSynchronize(b->stream));
  }
  for (int k = 0; k < 18; ++k) {
    const int a = k / 6, f = (k % 6) / 2, s = k % 2;
    const int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
    const int e1 = field_ext(L, f, a1), e2 = field_ext(L, f, a2);
    const int o1 = f == a1 ? 1 : 0, o2 = f == a2 ? 1 : 0;
    const int n1 = plane_n1(L, a);
    double* plane = buf.data() + (sweep_face_off(L, a, f, s) - off0);
    for (int q = 0; q < e2; ++q)
      for (int r = 0; r < e1; ++r) {
        const size_t pi = (size_t)(r + o1) + (size_t)n1 * (q + o2), hi = r + (size_t)e1 * q;
        if (out && out[k]) out[k][hi] = plane[pi];
        if (in && in[k]) plane[pi] = in[k][hi];
      }
  }
  if (in) {
    NB_CUDA(b, cudaMemcpyAsync(dev, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    NB_CUDA(b, cudaStreamSynchronize(b->stream));
  }
  return NS_OK;
}

int ns_batch_set_sweep_faces(ns_batch* b, int slot, int i, const double* const faces[18]) {
  if (!faces) return NS_ERR_ARG;
  return sweep_faces_copy(b, slot, i, nullptr, faces);
}

int ns_batch_get_sweep_faces(ns_batch* b, int slot, int i, double* const faces[18]) {
  if (!faces) return NS_ERR_ARG;
  return sweep_faces_copy(b, slot, i, faces, nullptr);
}

int ns_batch_advance(ns_batch* b, double t0) {
  if (!b) return NS_ERR_ARG;
  const ns_batch_config& c = b->cfg;
  std::vector<std::pair<double, int>> knots;
  for (int s = 0; s < c.n_slots; ++s)
    if (b->snap_ok[s]) knots.emplace_back(b->snap_t[s], s);
  std::sort(knots.begin(), knots.end());
  if (knots.empty()) return bfail(b, NS_ERR_ARG, "no parent snapshot captured");
  const double tol = 1e-9 * c.dt0;
  // The pinned weight buffers are rewritten below: wait for the previous copies.
  NB_CUDA(b, cudaEventSynchronize(b->copy_done));
  const bool sub_interval = b->intervals_done == 0;
  const int nstages = sub_interval ? b->max_r : 1;
  for (int s = 1; s <= nstages; ++s) {
    const int set = sub_interval ? s : 0;
    int* hs = b->host_slots + (size_t)set * b->n * 6;
    double* hw = b->host_wts + (size_t)set * b->n * 6;
    for (int i : b->active[set]) {
      const double dt = set == 0 ? c.dt0 : c.dt0 / b->desc[i].sub_tstep;
      const double t = t0 + (set == 0 ? 1 : s) * dt;
      if (window_weights(knots, t, tol, hs + 6 * i, hw + 6 * i) != NS_OK)
        return bfail(b, NS_ERR_ARG, "no 6-snapshot window around t = " + std::to_string(t));
    }
    NB_CUDA(b, cudaMemcpyAsync(b->dev_slots + (size_t)set * b->n * 6, hs, (size_t)b->n * 6 * sizeof(int),
                               cudaMemcpyHostToDevice, b->stream));
    NB_CUDA(b, cudaMemcpyAsync(b->dev_wts + (size_t)set * b->n * 6, hw, (size_t)b->n * 6 * sizeof(double),
                               cudaMemcpyHostToDevice, b->stream));
    if (s == nstages) NB_CUDA(b, cudaEventRecord(b->copy_done, b->stream));
    const bool first = sub_interval && s == 1 && !c.restart;
    int st = run_stage(b, set, first);
    if (st) return st;
  }
  b->intervals_done++;
  return NS_OK;
}

int ns_batch_max_div(ns_batch* b, int i, double* out) {
  if (!b || i < 0 || i >= b->n || !out) return NS_ERR_ARG;
  const SubGeo& g = b->geo[i];
  unsigned long long* bits = nullptr;
  NB_CUDA(b, cudaMalloc(&bits, sizeof(unsigned long long)));
  cudaError_t e = launch_diag(g.L, g.fld[0], g.fld[1], g.fld[2], 1.0 / b->cfg.dx, 1.0 / b->cfg.dy, 1.0 / b->cfg.dz,
                              bits, b->stream);
  unsigned long long hb = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(bits);
  if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, cudaGetErrorString(e));
  std::memcpy(out, &hb, sizeof(double));
  return NS_OK;
}

int ns_batch_error_metrics(ns_batch* b, const ns_handle* parent, double* out) {
  if (!b || !parent || !out) return NS_ERR_ARG;
  const Layout& Lp = parent->L;
  std::vector<MetricBox> boxes(b->n);
  for (int i = 0; i < b->n; ++i) {
    const ns_subdomain& d = b->desc[i];
    if (d.x0 + d.nx > Lp.nx + 1 || d.y0 + d.ny > Lp.ny + 1 || d.z0 + d.nz > Lp.nz + 1)
      return bfail(b, NS_ERR_SHAPE, "subdomain " + std::to_string(i) + " does not fit inside the parent");
    MetricBox& B = boxes[i];
    B.La = b->geo[i].L;
    B.Lb = Lp;
    for (int f = 0; f < 4; ++f) B.a[f] = b->geo[i].fld[f];
    B.b[0] = parent->u; B.b[1] = parent->v; B.b[2] = parent->w; B.b[3] = parent->p;
    B.ox = d.x0 - 1; B.oy = d.y0 - 1; B.oz = d.z0 - 1;
    B.idx = 1.0 / b->cfg.dx; B.idy = 1.0 / b->cfg.dy;
  }
  cudaEvent_t ev;
  NB_CUDA(b, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaEventRecord(ev, parent->stream);
  cudaStreamWaitEvent(b->stream, ev, 0);
  MetricBox* dbox = nullptr;
  cudaError_t e = cudaMallocAsync(&dbox, sizeof(MetricBox) * b->n, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dbox, boxes.data(), sizeof(MetricBox) * b->n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = launch_metrics(dbox, boxes, out, b->stream);
  if (dbox) cudaFreeAsync(dbox, b->stream);
  cudaEventRecord(ev, b->stream);
  cudaStreamWaitEvent(parent->stream, ev, 0);
  cudaEventDestroy(ev);
  b->launches += 1;
  if (e != cudaSuccess) return bfail(b, NS_ERR_CUDA, std::string("metrics: ") + cudaGetErrorString(e));
  return NS_OK;
}

int ns_batch_profile(ns_batch* b, int reps, double* ms_per_stage) {
  if (!b || !ms_per_stage) return NS_ERR_ARG;
  if (reps < 1) reps = 3;
  // On a copy of the state, as the autotuner: the timed launches rewrite it.
  double* save = nullptr;
  NB_CUDA(b, cudaMalloc(&save, b->arena_n * sizeof(double)));
  NB_CUDA(b, cudaMemcpyAsync(save, b->arena, b->arena_n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int status = NS_OK;
  for (int q = 0; q < ST_COUNT; ++q) ms_per_stage[q] = 0.0;
  for (int stage : kStageOrder) {
    if (stage == ST_HIST) continue;
    if (launch_stage_kernel(b, 0, stage, false, b->stream) != cudaSuccess) { status = NS_ERR_CUDA; break; }
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < reps; ++r) launch_stage_kernel(b, 0, stage, false, b->stream);
    cudaEventRecord(e1, b->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) { status = NS_ERR_CUDA; break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms_per_stage[stage] = ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemcpyAsync(b->arena, save, b->arena_n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  cudaFree(save);
  if (status) return bfail(b, status, "profile launch failed");
  return NS_OK;
}

int ns_batch_autotune(ns_batch* b, int reps) {
  if (!b) return NS_ERR_ARG;
  if (reps < 1) reps = 3;
  // Work on a copy of the state: the timed launches rewrite it.
  double* save = nullptr;
  NB_CUDA(b, cudaMalloc(&save, b->arena_n * sizeof(double)));
  NB_CUDA(b, cudaMemcpyAsync(save, b->arena, b->arena_n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int cand[] = {0, nsm, 2 * nsm, 4 * nsm, 8 * nsm, 16 * nsm};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int mode = b->cfg.mode;
  b->cfg.mode = 0;
  int status = NS_OK;
  for (int stage : kStageOrder) {
    if (stage == ST_HIST) continue;
    float best_ms = 1e30f;
    int best = 0;
    for (int g : cand) {
      b->cfg.grid[stage] = g;
      if (launch_stage_kernel(b, 0, stage, false, b->stream) != cudaSuccess) { status = NS_ERR_CUDA; break; }  // warm
      cudaEventRecord(e0, b->stream);
      for (int r = 0; r < reps; ++r) launch_stage_kernel(b, 0, stage, false, b->stream);
      cudaEventRecord(e1, b->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) { status = NS_ERR_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) { best_ms = ms; best = g; }
    }
    if (status) break;
    b->cfg.grid[stage] = best;
  }
  b->cfg.mode = mode;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemcpyAsync(b->arena, save, b->arena_n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  cudaFree(save);
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  b->graph_count.clear();
  if (status) return bfail(b, status, "autotune launch failed");
  return NS_OK;
}

int ns_batch_launch_count(const ns_batch* b, long long* launches) {
  if (!b || !launches) return NS_ERR_ARG;
  *launches = b->launches;
  return NS_OK;
}

int ns_spline_weights(const double* knots, int n_knots, double t, int* first, double* w) {
  if (!knots || n_knots < 1 || !first || !w) return NS_ERR_ARG;
  std::vector<std::pair<double, int>> k;
  for (int i = 0; i < n_knots; ++i) k.emplace_back(knots[i], i);
  const double span = n_knots > 1 ? knots[n_knots - 1] - knots[0] : 1.0;
  int slots[6];
  const int s = window_weights(k, t, 1e-12 * span, slots, w);
  if (s) return s;
  *first = slots[0];
  return NS_OK;
}

}  // extern "C"
