// Internal definitions shared by the FP64 staggered-step kernels (sm_103a).
//
// Device layout.  Every field lives in one padded box of slots
// [0, nx+1] x [0, ny+2) x [0, nz+2) with x fastest:
//
//   element(i, j, k) = base + off + i + sy*j + sz*k,   sy = px, sz = px*(ny+2)
//
// The internal slot of a reference (Fortran, 1-based) index is the index
// itself along a staggered (face) axis and the index minus one along a cell
// axis.  So u(I,J,K) -> (I, J-1, K-1), v(I,J,K) -> (I-1, J, K-1),
// w(I,J,K) -> (I-1, J-1, K), p(I,J,K) -> (I-1, J-1, K-1).  With this map,
// slot m of every field is "cell m" or "the low face of cell m", the same
// stencil serves every field, and on a periodic axis every field obeys
// X[0] = X[n], X[n+1] = X[1].  Face fields own one extra slot (slot 0 along
// their face axis) that the reference arrays do not have; on a periodic axis
// it holds the copy of face n, elsewhere it is unused.
//
// off = 7 puts slot 1 of every row on a 64-byte boundary (px is a multiple
// of 8 doubles).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ns_gpu.h"

namespace ns {

struct Layout {
  int nx, ny, nz;
  int px;          // row pitch (doubles)
  long long sy, sz;
  long long off;
  long long fsize;  // doubles allocated per field
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return off + i + sy * (long long)j + sz * (long long)k;
  }
};

inline Layout make_layout(int nx, int ny, int nz) {
  Layout L;
  L.nx = nx; L.ny = ny; L.nz = nz;
  L.off = 7;
  L.px = ((nx + 2 + 7 + 7) / 8) * 8;
  L.sy = L.px;
  L.sz = (long long)L.px * (ny + 2);
  // the predictor's 16-byte tile copies read whole rows from slot -1 to
  // slot 32 bx + 33, up to 25 doubles past the last row of the last plane
  L.fsize = L.sz * (nz + 2) + 32;
  return L;
}

// FP64 arithmetic in FMA form.  On this part DADD and DMUL issue at about
// 0.84x the DFMA rate, so sums and products that the step can express as
// FMAs are written as FMAs with a runtime 1.0 / -0.0 operand (bitwise the
// same result as the plain add / multiply: a*1 and a*b + (-0) are exact
// transformations under round-to-nearest).
struct FOne {
  double one, mzero;
};
__device__ __forceinline__ double fadd(const FOne& c, double a, double b) { return fma(a, c.one, b); }
__device__ __forceinline__ double fsub(const FOne& c, double a, double b) { return fma(b, -c.one, a); }
__device__ __forceinline__ double fmul(const FOne& c, double a, double b) { return fma(a, b, c.mzero); }

// Asynchronous 8-byte global -> shared copies (cp.async, L1-allocating) and
// their commit groups.
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
// 16-byte copies (both addresses 16-byte aligned; through L2 only).
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Error word on the device (bit flags).
enum : unsigned { ERRW_NONFINITE = 1u, ERRW_BOUNDS = 2u, ERRW_TIMEOUT = 4u };

}  // namespace ns
