// Kernel argument blocks and launchers of the FP64 staggered step.
#pragma once
#include <cuda.h>
#include <vector>

#include "ns_internal.cuh"

namespace ns {

// One work item of a batched launch: a subdomain and the block coordinates
// of one CTA's worth of work in that subdomain.  Persistent CTAs walk an
// array of items (item blockIdx.x, then + gridDim.x, ...).
struct BatchItem {
  int sub, bx, by, bz;
};

// Called after every kernel launch with the kernel's name (launch counting
// and per-kernel event timing in ns_api.cu).
struct Marker {
  void (*fn)(void*, const char*) = nullptr;
  void* ctx = nullptr;
  void operator()(const char* name) const {
    if (fn) fn(ctx, name);
  }
};

// ---------------------------------------------------------------------------
// Predictor (ns_predict.cu)
// ---------------------------------------------------------------------------
struct PredictArgs {
  Layout L;
  const double* u;
  const double* v;
  const double* w;
  const double* p;
  double* us;
  double* vs;
  double* ws;
  double* hx;  // AB2 history (rhs_?_previous), read and rewritten in place
  double* hy;
  double* hz;
  double one, mzero;
  int ulo, vlo, wlo;  // first active face along the component's own axis (1 periodic, 2 wall)
  double cx, cy, cz;  // -1/(4 dx) etc: C = -conv
  // AB2 / Euler: rhs = k0*u + kx*sWE + ky*sSN + kz*sBT + C
  double k0, kx, ky, kz;
  // AB2-CN: u* = c0*u + ca*sWE + cb*sSN + cc*sBT + cC*C + cP*prev
  double c0, ca, cb, cc, cC, cP;
  double dt, e1, e2;  // AB2: u* = u + e1*rhs + e2*prev
  double gpx, gpy, gpz;  // -dt/dx etc. (dp_flag)
  double ix2, iy2, iz2, lap0;  // diffusion-only mode
  // Plane ranges with their own chunk depth (0: the defaults): chunk bz holds
  // the planes 1 + koff + kc*bz .. up to kend (exclusive; 0: nz + 1).
  int kc, koff, kend;
  int* err;  // device word set to 1 when a bounded wait of the tile loader gave up (may be null)
};
// Tile-loader maps (TMA) of three fields of one layout for the session
// predictor (ns_predict.cu): 3D tensors (px, ny+2, nz+2) of doubles, boxes of
// 40 x 18 x 1.  Used when the predictor's u, v, w are the mapped fields.
struct PredTma {
  CUtensorMap u, v, w;
  const double* pu;
  const double* pv;
  const double* pw;
  int ready;
};
bool make_pred_tma(PredTma& t, const Layout& L, const double* u, const double* v, const double* w);

// Combine the stencil pieces into u* and rewrite the AB2 history at g.
template <int SCHEME, bool FIRST>
// prev is hist[g] (read by the caller ahead of time; unused for Euler and
// the first step).
__device__ __forceinline__ double predictor_combine(const PredictArgs& a, const FOne& c, double uc, double sWE,
                                                    double sSN, double sBT, double C, double prev,
                                                    double* __restrict__ hist, long long g) {
  if (SCHEME == 2) {  // AB2-CN explicit half (big_periodic_3D.f90:398-423)
    double t = fmul(c, a.c0, uc);
    t = fma(a.ca, sWE, t);
    t = fma(a.cb, sSN, t);
    t = fma(a.cc, sBT, t);
    t = fma(FIRST ? a.dt : a.cC, C, t);  // Euler start: rhs = nu/2 diff - conv (big_periodic_3D.f90:400-408)
    if (!FIRST) t = fma(a.cP, prev, t);
    hist[g] = C;  // rhs_?_previous = -conv
    return t;
  } else {
    double rhs = fma(a.k0, uc, C);
    rhs = fma(a.kz, sBT, rhs);
    rhs = fma(a.ky, sSN, rhs);
    rhs = fma(a.kx, sWE, rhs);  // nu*diff - conv
    double t;
    if (SCHEME == 1 && !FIRST) {  // AB2 (big_periodic_3D.f90:369-396)
      t = fma(a.e2, prev, uc);
      t = fma(a.e1, rhs, t);
    } else {  // Euler, or the Euler start of AB2
      t = fma(a.dt, rhs, uc);
    }
    hist[g] = (SCHEME == 0) ? 0.0 : rhs;
    return t;
  }
}

size_t predict_smem_bytes();
cudaError_t launch_predict(const PredictArgs& a, int scheme, bool first, bool dpf, int mode, cudaStream_t st,
                           const PredTma* tma = nullptr);
int predict_chunk_planes();
// The predictor on the cell planes [p0, p1) (1 <= p0 < p1 <= nz + 1) in
// chunks of kc planes per CTA: small chunks spread a short range over more
// CTAs (less latency, a little more work per plane).
cudaError_t launch_predict_planes(PredictArgs a, int scheme, bool first, bool dpf, int p0, int p1, int kc,
                                  cudaStream_t st, const PredTma* tma = nullptr);
// Predictor tiles of one box (work items of the batched launch).
void predict_tiles(const Layout& L, int& gx, int& gy, int& gz);
// Batched predictor over the items (grid <= 0: one wave of resident CTAs).
cudaError_t launch_predict_batch(const PredictArgs* tab, const BatchItem* items, int n_items, int scheme, bool first,
                                 bool dpf, int grid, cudaStream_t st);

// ---------------------------------------------------------------------------
// Boundary fills (ns_bc.cu)
// ---------------------------------------------------------------------------
// A face plane on the device: full (n2 x n3) plane of the box in internal
// slot order, for the two axes other than the face's axis.
struct FacePlanes {
  // [field 0..3 = u,v,w,p][side 0 = low, 1 = high] for one axis
  const double* f[4][2];
};
struct FaceSet {
  FacePlanes ax[3];
};

// vel_bc_staggered (NS_functions.f90:213-310), one axis pass.
cudaError_t launch_vel_bc(const Layout& L, double* us, double* vs, double* ws, const FaceSet& F, const int bc[3],
                          cudaStream_t st);
// Face slot 0 of each periodic axis's face field from face n (after a state load).
cudaError_t launch_extra_slots(const Layout& L, double* u, double* v, double* w, const int bc[3], cudaStream_t st);
// pr_bc_staggered (NS_functions.f90:1403-1464), the three axis passes.
cudaError_t launch_pr_bc(const Layout& L, double* dp, const FaceSet& F, const int pbc[3], double dx, double dy,
                         double dz, cudaStream_t st);
// The same fill in parts: the x and y passes over the planes z in [k0, k1),
// and (z_pass) the z pass, which writes both ghost planes from planes 1 and
// nz.  Filling every cell plane 1..nz by x/y parts and then running the z
// pass gives the bits of launch_pr_bc: its x and y passes over the ghost
// planes are overwritten by its z pass.
cudaError_t launch_pr_bc_planes(const Layout& L, double* dp, const FaceSet& F, const int pbc[3], double dx,
                                double dy, int k0, int k1, cudaStream_t st);
cudaError_t launch_pr_bc_z(const Layout& L, double* dp, const FaceSet& F, int pbc_z, double dz, cudaStream_t st);
// Elements of the face plane normal to an axis (ghosts included).
int plane_count(const Layout& L, int axis);
// Per-subdomain arguments of the batched fills.
struct BatchBcArgs {
  Layout L;
  double* us;
  double* vs;
  double* ws;
  double* dp;
  FaceSet F;
  int bc[3], pbc[3];
  double h[3];
};
// One axis pass of vel_bc_staggered (pr false) or pr_bc_staggered (pr true)
// over the items (sub, 256-element chunk bx of the plane).
cudaError_t launch_bc_batch(int axis, bool pr, const BatchBcArgs* tab, const BatchItem* items, int n_items, int grid,
                            cudaStream_t st);

// ---------------------------------------------------------------------------
// ADI (ns_adi.cu)
// ---------------------------------------------------------------------------
// Factors of one line system (same for every line of a sweep and field).
struct LineSys {
  const double* l;     // forward multipliers; index pad + e for unknown e, zero-padded
  const double* dinv;  // 1/pivot (zero in the padding)
  const double* cu;    // super-diagonal * dinv (zero in the padding)
  const double* z;     // Sherman-Morrison vector (periodic only), index e
  double s0, s1;       // correction weights of y[first] and y[last] (periodic only)
  int zA, zB;          // the correction is applied on [0, zA) and [zB, n_unk)
  int lo, hi;          // first/last unknown slot along the axis
  int periodic;        // 1: reduced cyclic system on slots 1..n + copies to slots 0, n+1
  int n;               // cells along the axis
  int pad;             // zero padding on each side of the factor tables
};
struct AdiArgs {
  Layout L;
  const double* src[3];  // u*, v*, w* before the sweep
  double* dst[3];        // after the sweep (another buffer: fixed ping-pong roles)
  LineSys sys[3];        // per field (normal or tangential system)
  const double* face_lo[3];  // BC row values per field (internal-slot planes), NULL -> 0
  const double* face_hi[3];
  int z0, z1;                // x and y sweeps: only the lines of z slots [z0, z1) (z1 = 0: all)
};
cudaError_t launch_adi(int axis, const AdiArgs& a, cudaStream_t st);
// The tile loader's bounded mbarrier wait on a barrier that no copy fills (ns_predict.cu).
cudaError_t launch_wait_selftest(unsigned long long limit_ns, int* gave_up, unsigned long long* waited_ns,
                                 cudaStream_t st);
// One subdomain of the batched AB2-CN sweeps (ns_batch.cu): u*, v*, w* swept
// in place (walls only), the nine line systems and the BC-row planes of each
// sweep (the parent's per-sweep faces, big_periodic_3D.f90:433-489).
struct BatchAdiArgs {
  Layout L;
  double* f[3];                 // u*, v*, w*
  LineSys sys[3][3];            // [axis][field]
  const double* face_lo[3][3];  // [axis][field]: plane (other two axes, ghosts included) of the low BC row
  const double* face_hi[3][3];
};
constexpr int kAdiBatchLines = 128;  // lines per work item (bx) of one field (by) of one subdomain
cudaError_t launch_adi_batch(int axis, const BatchAdiArgs* tab, const BatchItem* items, int n_items, int grid,
                             cudaStream_t st);

// ---------------------------------------------------------------------------
// Periodic FFT Poisson (ns_fft.cu)
// ---------------------------------------------------------------------------
// Plan of the spectral pressure solve: per axis an FFT (periodic) or a dense
// trigonometric transform pair (non-periodic, ns_dct.cu).
struct FftPlan {
  int nx, ny, nz, nxh;
  const double2* tw_x;   // twiddles for the nx/2-point complex FFT (x)
  const double2* tw_xr;  // r2c split twiddles: exp(-2 pi i k / nx), k < nx/2
  const double2* tw_y;
  const double2* tw_z;
  const double* inv_lam;  // scale/lambda per spectrum entry (FFT z solve), 0 at the mean mode
  int dp_unaligned;       // 1: dp slot pairs (2m+1, 2m+2) are not 16-byte aligned (scalar stores)
  int nxs;                // spectrum row length: nx/2+1 (periodic x) or nx/2 (packed wall x)
  int kind[3];            // 0: FFT axis, 1: dense transform axis, 2: tridiagonal solve axis (a wall)
  const double* fwd[3];   // dense forward matrices (x: F^T [n][k]; y, z: F [k][n])
  const double* inv[3];   // dense inverse matrices (x: G^T [k][n]; y, z: G [n][k])
  int sym[3];             // bit 0: F[k][N-1-n] = (-1)^k F[k][n]; bit 1: G[N-1-n][k] = (-1)^k G[n][k]
  // A dense y axis of power-of-two length 32..512 with pbc 2 or 3 transformed through an FFT
  // (Makhoul) instead of the dense products (session plans; ns_fft.cu dct_y_kernel):
  int dct_y;              // 0: dense products; 2 or 3: the pressure code of the FFT-based transform
  const double2* dct_tw;  // exp(-2 pi i m / ny), m < ny
  const double2* dct_wf;  // exp(-i pi k / (2 ny)) / 2, k = 0..ny (forward post-twiddle)
  const double2* dct_wi;  // exp(+i pi k / (2 ny)) / ny, k < ny (inverse pre-twiddle)
  // The same for a wall x axis (packed modes; two x lines per complex FFT):
  int dct_x;
  const double2* dctx_tw;  // exp(-2 pi i m / nx), m < nx
  const double2* dctx_wf;  // exp(-i pi k / (2 nx)) / 2, k = 0..nx
  const double2* dctx_wi;  // exp(+i pi k / (2 nx)) / nx, k < nx
  int has_mean;           // 1: the singular mode is set to mean_val (after the forward passes)
  double mean_val;        // FFT z solve: the singular entry; tridiagonal solve: the singular line's mean
  const double* mean_dev; // non-null: the line mean is mean_val * (*mean_dev) (a mean_dp set on the device)
  // Tridiagonal solve along the wall axis s, one line per (x mode, other-axis mode):
  // rows (p[j-1] - (2 - e_j - sigma h^2) p[j] + p[j+1]) = h^2 scale rhs[j].
  const double* eig_x;    // lambda of the x modes (nxs entries; 2 per entry when x is packed)
  const double* eig_o;    // lambda of the modes of the remaining axis
  double tri_h2;          // h_s^2
  double tri_rs;          // h_s^2 * scale of the unnormalised FFT passes
  double tri_elo, tri_ehi;  // end-row diagonal changes: pbc 2 -1, pbc 3 +1, pbc 4 0
  const double2* tri_m;   // the twisted factorisation's multipliers (re, im) of every line, laid out
                          // like the spectrum (launch_tri_twist_table)
  double* sing_cm;        // session solve from a table: global scratch (2 N TRI_T doubles) of the
                          // singular line's multipliers (the batch keeps them in shared memory)
  int tri_tw;             // 1: tri_m holds the twisted multipliers, solved two lanes per line
  // All-periodic boxes: the z stage as cyclic tridiagonal line solves (ns_cyclic.cu)
  // instead of z FFT * 1/lambda * z IFFT.  Tables per (kx, ky) mode, laid out like the
  // spectrum: T's multipliers, w = rs T^-1 e0, q = T^-1 u; per mode (1/c, SM denominator).
  int zcyc;
  const double* cyc_m;
  const double* cyc_w;
  const double* cyc_q;
  const double2* cyc_s;
  const double* cyc_v;    // the singular (0, 0) line's solution mean, as a functional of its data
  double cyc_rs;          // h_z^2 * scale * nz
  double cyc_h2;          // h_z^2
  double mod_lo[3], mod_hi[3];        // pr_bc_staggered_modify_rhs coefficients per axis
  const double* face_lo[3];           // pressure face planes per axis (internal slot order)
  const double* face_hi[3];

  // pr_bc_staggered_modify_rhs (NS_functions.f90:1345-1400) at interior cell (i, j, k).
  // Interior cells leave through one integer test: the boundary terms sit in
  // a call so that they are branched around, not predicated (a predicated-off
  // FP64 instruction still takes its FP64-pipe issue slot at every cell).
  __device__ __forceinline__ double bc_term(int i, int j, int k) const {
    if (i != 1 && i != nx && j != 1 && j != ny && k != 1 && k != nz) return 0.0;
    return bc_term_edge(i, j, k);
  }
  __device__ __noinline__ double bc_term_edge(int i, int j, int k) const {
    double t = 0.0;
    const int n[3] = {nx, ny, nz};
    const int idx[3] = {i, j, k};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (mod_lo[a] == 0.0 && mod_hi[a] == 0.0) continue;
      const int s1 = (a == 0) ? j : i;
      const int s2 = (a == 2) ? j : k;
      const int n1 = (a == 0) ? ny + 2 : nx + 2;
      const int pl = s1 + n1 * s2;
      if (idx[a] == 1 && face_lo[a]) t = fma(mod_lo[a], face_lo[a][pl], t);
      if (idx[a] == n[a] && face_hi[a]) t = fma(mod_hi[a], face_hi[a][pl], t);
    }
    return t;
  }
  // The boundary cells of the interior box, each once: the x faces (i = 1,
  // nx; every j, k), then the y faces (j = 1, ny; 1 < i < nx; every k), then
  // the z faces (k = 1, nz; 1 < i < nx, 1 < j < ny).  A pass over them adds
  // bc_term_edge to a divergence computed without it: (div + 0) + t is
  // div + t bit for bit (t starts at +0 and only gains products, so it is
  // never -0).
  __host__ __device__ long long bc_cells() const {
    return 2LL * ny * nz + 2LL * (nx - 2) * nz + 2LL * (nx - 2) * (ny - 2);
  }
  __device__ __forceinline__ void bc_cell(long long q, int& i, int& j, int& k) const {
    const long long fx = (long long)ny * nz, fy = (long long)(nx - 2) * nz;
    if (q < 2 * fx) {
      const long long r = q % fx;
      i = q < fx ? 1 : nx; j = 1 + (int)(r % ny); k = 1 + (int)(r / ny);
      return;
    }
    q -= 2 * fx;
    if (q < 2 * fy) {
      const long long r = q % fy;
      j = q < fy ? 1 : ny; i = 2 + (int)(r % (nx - 2)); k = 1 + (int)(r / (nx - 2));
      return;
    }
    q -= 2 * fy;
    const long long fz = (long long)(nx - 2) * (ny - 2), r = q % fz;
    k = q < fz ? 1 : nz; i = 2 + (int)(r % (nx - 2)); j = 2 + (int)(r / (nx - 2));
  }
  __host__ __device__ bool any_bc_term() const {
    return mod_lo[0] != 0.0 || mod_hi[0] != 0.0 || mod_lo[1] != 0.0 || mod_hi[1] != 0.0 || mod_lo[2] != 0.0 ||
           mod_hi[2] != 0.0;
  }
};
using SpecPlan = FftPlan;
// The FFT-based y transform of a packed-x plan with dct_y set (ns_fft.cu).
cudaError_t launch_dct_y(bool fwd, const FftPlan& P, double2* spec, cudaStream_t st);
struct DivArgs;
// The FFT-based x transforms of a plan with dct_x set (ns_fft.cu): divergence
// (+ pressure-BC terms), or d.rhs when given, -> packed modes, and packed
// modes -> dp slots 1..nx.
cudaError_t launch_dct_x_fwd(const FftPlan& P, const DivArgs& d, double2* spec, cudaStream_t st, const Marker& mk);
cudaError_t launch_dct_x_inv(const FftPlan& P, const double2* spec, double* dp, const Layout& L, cudaStream_t st);
struct DivArgs {
  Layout L;
  const double* us;
  const double* vs;
  const double* ws;
  double cdx, cdy, cdz;  // 1/(dx dt) etc.
  double one, mzero;
  const double* rhs;     // non-null: transform this right-hand side (cell slots) instead of div(u*)/dt
};
// Forward 3D FFT of the cell field d.rhs (all-periodic plan): spec = 2 x DFT.
cudaError_t launch_fft_forward3(const FftPlan& P, const DivArgs& d, double2* spec, cudaStream_t st,
                                const Marker& mk);
// The spectral solve (FFT and dense axes mixed), divergence to dp interior:
// launch_poisson_fwd (divergence, forward passes, line solve) followed by
// launch_poisson_inv over all planes.
cudaError_t launch_fft_poisson(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk);
cudaError_t launch_poisson_fwd(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk);
// True when both inverse passes are FFTs along x and y, which work plane by
// plane in z: launch_poisson_inv then accepts any cell-plane range [k0, k1).
bool poisson_inv_by_planes(const FftPlan& P);    // both inverse passes take z plane ranges
bool poisson_inv_x_by_planes(const FftPlan& P);  // the x inverse pass takes z plane ranges
cudaError_t launch_poisson_inv_mid(const FftPlan& P, const DivArgs& d, double2* spec, const Layout& L,
                                   cudaStream_t st, const Marker& mk, int k0, int k1);
cudaError_t launch_poisson_inv_x(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                                 cudaStream_t st, const Marker& mk, int k0, int k1);
cudaError_t launch_poisson_inv(const FftPlan& P, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                               cudaStream_t st, const Marker& mk, int k0, int k1);
// Symmetry bits of a dense transform pair of even size n (sym in FftPlan),
// checked entry by entry on the host (ns_dct.cu).
int dense_symmetry(int n, const std::vector<double>& F, const std::vector<double>& G);
// The cyclic z solve of an all-periodic plan (ns_cyclic.cu): the size of its
// tables, their construction (sets P.cyc_*; eig_x, eig_o, cyc_h2, cyc_rs set
// before), and the solve of every z line of the spectrum in place.
size_t cyc_table_doubles(const FftPlan& P);
cudaError_t launch_cyc_table(FftPlan& P, double* buf, cudaStream_t st);
cudaError_t launch_cyc_z_solve(const FftPlan& P, double2* spec, cudaStream_t st);
// Lanes per x line of the dense x passes: the next power of two at or above
// nx/2 (the mode pairs of a line), at most 32; a 128-thread CTA takes 128/G lines.
__host__ __device__ __forceinline__ int dense_x_group(int nx) {
  const int h = nx / 2 > 1 ? nx / 2 : 1;
  int g = 1;
  while (g < h && g < 32) g <<= 1;
  return g;
}
// The x inverse takes row pairs (n, H-1-n) when its matrix folds twice
// (sym bits 1 and 4 or 5), so its groups cover nx/4 lanes.
__host__ __device__ __forceinline__ int dense_x_inv_group(const int sym, const int nx) {
  const int lvi = (sym >> 4) & 3;
  return ((sym & 2) && (lvi == 1 || lvi == 2)) ? dense_x_group(nx / 2) : dense_x_group(nx);
}
// Dense passes (ns_dct.cu): x forward/inverse, y/z forward/inverse.
cudaError_t launch_dense_x(bool fwd, const SpecPlan& S, const DivArgs& d, double2* spec, double* dp, const Layout& L,
                           cudaStream_t st);
cudaError_t launch_dense_yz(int axis, bool fwd, const SpecPlan& S, double2* spec, cudaStream_t st);
// Tridiagonal solve of every spectrum line along axis 1 (y) or 2 (z) (ns_dct.cu).
cudaError_t launch_tri_solve(int axis, const SpecPlan& S, double2* spec, cudaStream_t st);
// The twisted factorisation's multipliers of every line along axis 1 or 2,
// laid out like the spectrum: top-down m_j above the middle row k = N/2,
// bottom-up n_j below it, the middle pivot at k (ns_dct.cu).
cudaError_t launch_tri_twist_table(int axis, const SpecPlan& S, double2* tab, cudaStream_t st);
// Batched spectral passes of all-wall boxes (x dense packed, y dense, z line solve).
struct BatchSpecArgs {
  SpecPlan S;
  DivArgs d;
  double2* spec;
  double* dp;
  Layout L;
};
// pass: 0 x forward (divergence + BC terms), 1 x inverse, 2 y forward, 3 y inverse, 4 z line solve.
// A subdomain takes the FFT-based kernel of passes 0-3 where spec_pass_dct
// says so (its plan's dct_x / dct_y), the dense kernel otherwise; the two
// kernels take separate item lists (their register needs differ).
bool spec_pass_dct(int pass, const SpecPlan& S);
void spec_pass_grid(int pass, const SpecPlan& S, int& gx, int& gy);
size_t spec_pass_smem(int pass, const SpecPlan& S);
cudaError_t launch_spec_batch(int pass, bool dct, const BatchSpecArgs* tab, const BatchItem* items, int n_items,
                              size_t smem, int grid, cudaStream_t st);
// The divergence rows (plus the pressure-BC terms) of the subdomains whose x
// forward pass is FFT-based, into their spectrum buffers as rows of nx
// doubles (row = (j-1) + ny (k-1)); item (sub, q) covers the elements
// [kDivChunk q, kDivChunk (q+1)).  The FFT-based x forward then transforms
// the rows in place.
constexpr int kDivChunk = 256;
cudaError_t launch_spec_batch_div(const BatchSpecArgs* tab, const BatchItem* items, int n_items, int grid,
                                  cudaStream_t st);
// Then the pressure-BC terms of their boundary cells (SpecPlan::bc_cell
// order; item (sub, q) covers cells [kDivChunk q, kDivChunk (q+1))).
cudaError_t launch_spec_batch_bc(const BatchSpecArgs* tab, const BatchItem* items, int n_items, int grid,
                                 cudaStream_t st);

// ---------------------------------------------------------------------------
// Correction (ns_correct.cu)
// ---------------------------------------------------------------------------
struct CorrectArgs {
  Layout L;
  const double* us;
  const double* vs;
  const double* ws;
  const double* dp;
  double* u;
  double* v;
  double* w;
  double* p;
  double gx, gy, gz;  // -dt/dx etc.
  int dp_flag;
  int gauge;
  int per[3];
  double one, mzero;
};
cudaError_t launch_correct(const CorrectArgs& a, cudaStream_t st);
// The correction of the slot planes z in [k0, k1) only (0 <= k0 <= k1 <= nz + 2).
cudaError_t launch_correct_planes(const CorrectArgs& a, int k0, int k1, cudaStream_t st);
// Batched correction over the items (sub, 256-element chunk bx of the box).
cudaError_t launch_correct_batch(const CorrectArgs* tab, const BatchItem* items, int n_items, int grid,
                                 cudaStream_t st);

// Re-simulation error metrics (ns_metrics.cu): one box compares fields a
// (layout La) with reference fields b (layout Lb) at slot offset (ox, oy, oz).
struct MetricBox {
  Layout La;
  Layout Lb;
  const double* a[4];  // u, v, w, p
  const double* b[4];
  int ox, oy, oz;
  double idx, idy;     // 1/dx, 1/dy (vorticity)
};
// Reduce the boxes (dev_boxes: device copy of host_boxes) and fill out[12 * box + q]:
// rms of the reference u, v, w, p, then err_vel(1..8).  Synchronises st.
cudaError_t launch_metrics(const MetricBox* dev_boxes, const std::vector<MetricBox>& host_boxes, double* out,
                           cudaStream_t st);

// max|div u| over the interior and probe value (diagnostic).
cudaError_t launch_diag(const Layout& L, const double* u, const double* v, const double* w, double idx, double idy,
                        double idz, unsigned long long* out_bits, cudaStream_t st);

}  // namespace ns
