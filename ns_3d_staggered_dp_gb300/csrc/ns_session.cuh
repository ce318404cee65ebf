// The session handle of libns_gpu.so (shared by the session tier, ns_api.cu,
// and the batched tier, ns_batch.cu, which reads a parent session's fields).
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "../../include/ns_gpu.h"
#include "ns_internal.cuh"
#include "ns_kernels.cuh"

namespace ns {
struct AdjState;  // discrete adjoint tier (ns_adjoint.cu)
}

struct ns_handle {
  ns_config cfg;
  ns::Layout L;
  cudaStream_t stream = nullptr;
  cudaStream_t cap_stream = nullptr;  // private stream for graph capture
  bool own_stream = false;
  double dx, dy, dz;
  // device fields
  double *u = nullptr, *v = nullptr, *w = nullptr, *p = nullptr;
  double *hx = nullptr, *hy = nullptr, *hz = nullptr;
  double *us = nullptr, *vs = nullptr, *ws = nullptr, *dp = nullptr;
  double *us2 = nullptr, *vs2 = nullptr, *ws2 = nullptr;  // ADI ping-pong buffers
  double *us3 = nullptr, *vs3 = nullptr, *ws3 = nullptr;  // x-sweep output (cfg.keep_sweeps only)
  double2* spec = nullptr;
  double* stage = nullptr;   // host<->device staging of one reference-shaped field
  double* stage2 = nullptr;  // second staging buffer (multi-field transfers)
  cudaStream_t xfer = nullptr;  // copy stream of the multi-field transfers
  cudaStream_t side = nullptr;  // second compute stream of ns_step_host (x and y sweeps of a slab), greatest priority
  cudaStream_t prio = nullptr;  // compute stream of ns_step_host, greatest priority
  cudaStream_t scat = nullptr;  // ns_step_host: scatter of each landed slab into the padded layout, greatest priority
  cudaEvent_t ev_full[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  cudaEvent_t ev_aux[2] = {nullptr, nullptr};  // ns_step_host: history final, step done
  double* stage_f[7] = {};                     // ns_step_host: one staging buffer per state field
  std::vector<cudaEvent_t> ev_slab;            // ns_step_host: one event per z-slab
  double* inv_lam = nullptr;
  double* cyc_buf = nullptr;  // tables of the cyclic z solve (all-periodic boxes)
  double2* tri_tab = nullptr;  // the wall-axis line solve's twisted multipliers (one per spectrum entry)
  double* sing_cm = nullptr;   // its singular line's scratch
  double2* tw = nullptr;  // twiddle tables (x, xr, y, z)
  ns::FftPlan plan{};
  // ADI factors
  double* adi_buf = nullptr;
  ns::LineSys sys[3][3];  // [axis][field]
  // faces: [set 0..3][axis][field 0..3][side] -> device planes
  double* face_buf = nullptr;
  std::vector<double> face_host;  // host staging of one face set (ns_set_faces)
  double* mean_dev = nullptr;     // mean_dp of the singular mode on the device (ns_set_mean_dp)
  ns::FaceSet faces[4]{};
  bool face_set_nonzero[4] = {false, false, false, false};
  unsigned long long* diag_bits = nullptr;
  int* dev_err = nullptr;  // set on the device when a bounded wait of the predictor's tile loader gave up
  ns::PredTma tma{};        // tile-loader maps of u, v, w (tma.ready = 0: the predictor loads tiles itself)
  // state
  bool first_pending = true;
  long long steps = 0;
  std::string err;
  // graphs
  cudaGraphExec_t graph = nullptr;
  bool eager_done = false;
  long long graph_launches = 0;
  // launch counting and per-kernel timing (ns_profile)
  long long launches = 0;
  bool profiling = false;
  std::vector<std::pair<std::string, cudaEvent_t>> prof_events;
  // phase trace of ns_step_host (environment variable NS_TRACE set at ns_create):
  // timed events on the compute and copy streams, printed to stderr per call
  bool trace = false;
  std::vector<cudaEvent_t> trace_pool;
  std::vector<std::string> trace_names;
  // adjoint tier: checkpoints, stored inputs and adjoint fields (owned by ns_adjoint.cu)
  ns::AdjState* adj = nullptr;
};

namespace ns {
// Session internals shared by ns_api.cu and ns_adjoint.cu.
int api_fail(ns_handle* h, int code, const std::string& msg);
cudaError_t api_h2d_field(ns_handle* h, double* dst, const double* src, int field);
cudaError_t api_d2h_field(ns_handle* h, double* dst, const double* src, int field);
void api_mark(ns_handle* h, const char* name, int nkernels);
Marker api_marker(ns_handle* h);
int api_build_line_tables(ns_handle* h, bool transposed, LineSys sys[3][3], double** buf);
void api_free_adjoint(ns_handle* h);
}  // namespace ns


namespace ns {
// Dense transform pair (forward F [k][n], inverse G [n][k]) of one wall axis
// of n cells with pressure code pb (ns_api.cu).
void dense_pair(int n, int pb, std::vector<double>& F, std::vector<double>& G);
// sin^2(..)/h^2 of mode m of one axis (pbc 1 FFT bin, else the trigonometric mode).
double axis_eig(int n, int pb, int m, double h);
// Predictor coefficients of a box with velocity codes bc (ns_api.cu).
void set_predict_coeffs(PredictArgs& a, const int bc[3], double dx, double dy, double dz, double dt, double nu);
// Host description of one tridiagonal line system of an ADI sweep: LU
// factors without pivoting (forward multipliers l, 1/pivot dinv,
// super-diagonal / pivot cu) and, periodic only, the Sherman-Morrison data.
struct HostLineSys {
  std::vector<double> l, dinv, cu, z;
  double s0 = 0, s1 = 0;
  int zA = 0, zB = 0, lo = 0, hi = 0, periodic = 0, n = 0;
};
// The CN system of one sweep axis (mat_CN / mat_CN_tridiagonal,
// NS_functions.f90:1245-1342) for n cells with velocity code bc; normal: the
// swept field is staggered along the axis (ns_api.cu).
HostLineSys build_cn_system(int n, int bc, double h, double dt, double nu, bool normal, int closure,
                            bool transposed = false);
}  // namespace ns
