// Block-row SpMV of the DG variable-block storage (device code shared by the
// plain kernels and the serving engine's slot kernels).
#pragma once

#include "dword.cuh"

namespace gbfem {

// One 8-lane group per block row (32 block rows per CTA), launched per
// degree class so that the row block size NS is a compile-time constant:
// lane g accumulates rows g, g+8, ... (40 rows = 5 full slots for p = 3, 75 =
// 10 slots of which the last is 3/8 full for p = 4).  On GB300 the SpMV is
// bound by the FP64 pipe as much as by HBM (one FMA per 8-byte value against
// ~0.6 T FMA/s), so lanes must not idle: a warp per row would leave 24 of 64
// lane slots empty for NS = 40.
//
// The blocks of a row are consecutive and column-major with leading dimension
// NS, so the whole block row is one NS x nct column-major matrix starting at
// the row's first block; colx lists the dof index of each of its nct columns.
// One flat loop over the columns (instead of blocks, then columns) keeps the
// four groups of a warp in step when their neighbours differ in degree; the
// rows of a class are ordered by nct for the same reason.  With a
// preconditioner the group's rows go through shared memory into the product
// with the inverted diagonal block.  The arithmetic type VT is double, float
// (inner solves of iterative refinement) or dw (double words on the FP32
// pipes: the FP64 pipe bounds the double form at ~5 TB/s of values, below
// HBM; the double-word form is bound by HBM).
constexpr int DGS_LANES = 8;
constexpr int DGS_THREADS = 256;
constexpr int DGS_ROWS = DGS_THREADS / DGS_LANES;

__device__ __forceinline__ double dgs_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float dgs_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ dw dgs_fma(dw a, dw b, dw c) { return t_fma(a, b, c); }
// vector entries into the arithmetic type and results back to FP64
template <typename VT>
__device__ __forceinline__ VT dgs_in(double v) {
  return (VT)v;
}
template <>
__device__ __forceinline__ dw dgs_in<dw>(double v) {
  return dw_from_double(v);
}
__device__ __forceinline__ double dgs_out(double v) { return v; }
__device__ __forceinline__ double dgs_out(float v) { return (double)v; }
__device__ __forceinline__ double dgs_out(dw v) { return dw_to_double(v); }

// P: block class, 1..4 tensor-basis prisms of degree P (6, 18, 40, 75
// functions), 5..8 complete-basis tetrahedra of degree P - 4 (4, 10, 20, 35)
template <int P>
struct DgSpmvDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : P == 4 ? 75
                          : P == 5 ? 4 : P == 6 ? 10 : P == 7 ? 20 : 35;
};

// The body of the block SpMV for the block rows of one CTA (blockDim.x ==
// DGS_THREADS); sv: DGS_ROWS x NS values of shared memory.  VT is the type of
// the stored matrix and of the arithmetic (double, or float for the inner
// solves of iterative refinement); vectors are FP64 either way.
template <int P, typename VT = double>
__device__ __forceinline__ void dg_block_row_spmv(
    int mode, int count, const int *__restrict__ ent_el, const int *__restrict__ roff,
    const long long *__restrict__ row_val, const long long *__restrict__ cx_off, const int *__restrict__ colx,
    const VT *__restrict__ val, const long long *__restrict__ dinv_off, const VT *__restrict__ dinv,
    const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ out,
    VT (*sv)[DgSpmvDims<P>::NS]) {
  constexpr int NS = DgSpmvDims<P>::NS;
  constexpr int S = (NS + DGS_LANES - 1) / DGS_LANES;
  const int grp = threadIdx.x / DGS_LANES, g = threadIdx.x % DGS_LANES;
  const int idx = blockIdx.x * DGS_ROWS + grp;
  const bool active = idx < count;
  const int e = active ? ent_el[idx] : 0;
  const int r0 = roff[e];
  VT acc[S];
#pragma unroll
  for (int s = 0; s < S; s++) acc[s] = VT(0);
  if (active) {
    const VT *A = val + row_val[e] + g;
    const int *cx = colx + cx_off[e];
    const int nct = (int)(cx_off[e + 1] - cx_off[e]);
    int t = 0;
    for (; t + 2 <= nct; t += 2) {
      const VT x0 = dgs_in<VT>(x[cx[t]]), x1 = dgs_in<VT>(x[cx[t + 1]]);
      const VT *col0 = A + (size_t)t * NS, *col1 = col0 + NS;
#pragma unroll
      for (int s = 0; s < S; s++)
        if (g + DGS_LANES * s < NS) acc[s] = dgs_fma(col1[DGS_LANES * s], x1, dgs_fma(col0[DGS_LANES * s], x0, acc[s]));
    }
    if (t < nct) {
      const VT x0 = dgs_in<VT>(x[cx[t]]);
      const VT *col0 = A + (size_t)t * NS;
#pragma unroll
      for (int s = 0; s < S; s++)
        if (g + DGS_LANES * s < NS) acc[s] = dgs_fma(col0[DGS_LANES * s], x0, acc[s]);
    }
  }
  if (mode != 1) {
#pragma unroll
    for (int s = 0; s < S; s++) {
      const int i = g + DGS_LANES * s;
      acc[s] = (b && active && i < NS ? dgs_in<VT>(b[r0 + i]) : VT(0)) - acc[s];
    }
  }
  if (mode == 2) {
    if (active) {
#pragma unroll
      for (int s = 0; s < S; s++) {
        const int i = g + DGS_LANES * s;
        if (i < NS) out[r0 + i] = dgs_out(acc[s]);
      }
    }
    return;
  }
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int i = g + DGS_LANES * s;
    if (i < NS) sv[grp][i] = acc[s];
  }
  __syncwarp();
  if (!active) return;
  const VT *D = dinv + dinv_off[e] + g;
  VT o[S];
#pragma unroll
  for (int s = 0; s < S; s++) o[s] = VT(0);
  for (int j = 0; j < NS; j++) {
    const VT t = sv[grp][j];
    const VT *col = D + (size_t)j * NS;
#pragma unroll
    for (int s = 0; s < S; s++)
      if (g + DGS_LANES * s < NS) o[s] = dgs_fma(col[DGS_LANES * s], t, o[s]);
  }
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int i = g + DGS_LANES * s;
    if (i < NS) out[r0 + i] = dgs_out(o[s]);
  }
}

}  // namespace gbfem
