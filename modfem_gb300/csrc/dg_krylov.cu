// Variable-block CRS products and block Jacobi for the DG matrix, FP64.
//
// Storage (the device form of lad_block, lsd_mkb/lad_block/lah_block.h): block
// row e holds the dofs of element e (roff[e] .. roff[e+1]); its blocks
// bptr[e] .. bptr[e+1] have column elements bcol[k] (ascending, the diagonal
// included) and dense values at val + boff[k], column-major with the row
// block's size as leading dimension (Dia / Aux of las_block_intf.c:362-520).
//
// The block Jacobi preconditioner of the reference (lar_fill_preconditioner_
// block with Block_type 1: an LU factorisation of every diagonal block,
// las_block_intf.c:1224-1330, applied by forward/back substitution) is kept
// here as the explicit inverse of each diagonal block: applying it is then a
// dense block product fused into the SpMV.

#include "dg_tables.h"
#include "gbfem_internal.h"

namespace gbfem {

// Gauss-Jordan inversion with partial pivoting (largest magnitude, first
// index on ties), one CTA per diagonal block held in shared memory.
constexpr int DGI_THREADS = 256;

__global__ void __launch_bounds__(DGI_THREADS) dg_block_inverse_kernel(int nel, const int *__restrict__ roff,
                                                                        const long long *__restrict__ boff_diag,
                                                                        const double *__restrict__ val,
                                                                        const long long *__restrict__ dinv_off,
                                                                        double *__restrict__ dinv, int *err) {
  __shared__ double a[GB_DG_MAXNS * GB_DG_MAXNS];
  __shared__ double fcol[GB_DG_MAXNS];
  __shared__ int piv[GB_DG_MAXNS];
  __shared__ int s_r;
  const int e = blockIdx.x;
  if (e >= nel) return;
  const int n = roff[e + 1] - roff[e];
  if (n <= 0 || n > GB_DG_MAXNS) {
    if (threadIdx.x == 0) atomicExch(err, 4);
    return;
  }
  const double *src = val + boff_diag[e];
  for (int t = threadIdx.x; t < n * n; t += DGI_THREADS) a[t] = src[t];
  __syncthreads();
  for (int k = 0; k < n; k++) {
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = n;
      for (int i = k + (int)threadIdx.x; i < n; i += 32) {
        const double v = fabs(a[i + n * k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        s_r = best > 0.0 ? bi : -1;
        piv[k] = bi;
      }
    }
    __syncthreads();
    const int r = s_r;
    if (r < 0) {  // singular diagonal block (uniform across the CTA)
      if (threadIdx.x == 0) atomicExch(err, 3);
      return;
    }
    if (r != k)
      for (int j = threadIdx.x; j < n; j += DGI_THREADS) {
        const double t = a[k + n * j];
        a[k + n * j] = a[r + n * j];
        a[r + n * j] = t;
      }
    __syncthreads();
    const double pinv = 1.0 / a[k + n * k];
    for (int i = threadIdx.x; i < n; i += DGI_THREADS) fcol[i] = a[i + n * k];
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += DGI_THREADS) a[k + n * j] = j == k ? pinv : a[k + n * j] * pinv;
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += DGI_THREADS) {
      const int i = t % n, j = t / n;
      if (i == k) continue;
      a[t] = j == k ? -fcol[i] * pinv : fma(-fcol[i], a[k + n * j], a[t]);
    }
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = n - 1; k >= 0; k--) {
    const int r = piv[k];
    if (r != k)
      for (int i = threadIdx.x; i < n; i += DGI_THREADS) {
        const double t = a[i + n * k];
        a[i + n * k] = a[i + n * r];
        a[i + n * r] = t;
      }
    __syncthreads();
  }
  double *dst = dinv + dinv_off[e];
  for (int t = threadIdx.x; t < n * n; t += DGI_THREADS) dst[t] = a[t];
}

int launch_dg_block_inverse(cudaStream_t st, int nel, const int *roff, const long long *boff_diag,
                            const double *val, const long long *dinv_off, double *dinv, int *err) {
  if (nel <= 0) return 0;
  dg_block_inverse_kernel<<<nel, DGI_THREADS, 0, st>>>(nel, roff, boff_diag, val, dinv_off, dinv, err);
  GB_CUDA(cudaGetLastError());
  return 1;
}

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
// with the inverted diagonal block.
constexpr int DGS_LANES = 8;
constexpr int DGS_THREADS = 256;
constexpr int DGS_ROWS = DGS_THREADS / DGS_LANES;

template <int P>
__global__ void __launch_bounds__(DGS_THREADS) dg_block_spmv_kernel(
    int mode, int count, const int *__restrict__ ent_el, const int *__restrict__ roff,
    const long long *__restrict__ row_val, const long long *__restrict__ cx_off, const int *__restrict__ colx,
    const double *__restrict__ val, const long long *__restrict__ dinv_off, const double *__restrict__ dinv,
    const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ out) {
  constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  constexpr int S = (NS + DGS_LANES - 1) / DGS_LANES;
  __shared__ double sv[DGS_ROWS][NS];
  const int grp = threadIdx.x / DGS_LANES, g = threadIdx.x % DGS_LANES;
  const int idx = blockIdx.x * DGS_ROWS + grp;
  const bool active = idx < count;
  const int e = active ? ent_el[idx] : 0;
  const int r0 = roff[e];
  double acc[S];
#pragma unroll
  for (int s = 0; s < S; s++) acc[s] = 0.0;
  if (active) {
    const double *A = val + row_val[e] + g;
    const int *cx = colx + cx_off[e];
    const int nct = (int)(cx_off[e + 1] - cx_off[e]);
    int t = 0;
    for (; t + 2 <= nct; t += 2) {
      const double x0 = x[cx[t]], x1 = x[cx[t + 1]];
      const double *col0 = A + (size_t)t * NS, *col1 = col0 + NS;
#pragma unroll
      for (int s = 0; s < S; s++)
        if (g + DGS_LANES * s < NS) acc[s] = fma(col1[DGS_LANES * s], x1, fma(col0[DGS_LANES * s], x0, acc[s]));
    }
    if (t < nct) {
      const double x0 = x[cx[t]];
      const double *col0 = A + (size_t)t * NS;
#pragma unroll
      for (int s = 0; s < S; s++)
        if (g + DGS_LANES * s < NS) acc[s] = fma(col0[DGS_LANES * s], x0, acc[s]);
    }
  }
  if (mode != 1) {
#pragma unroll
    for (int s = 0; s < S; s++) {
      const int i = g + DGS_LANES * s;
      acc[s] = (b && active && i < NS ? b[r0 + i] : 0.0) - acc[s];
    }
  }
  if (mode == 2) {
    if (active) {
#pragma unroll
      for (int s = 0; s < S; s++) {
        const int i = g + DGS_LANES * s;
        if (i < NS) out[r0 + i] = acc[s];
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
  const double *D = dinv + dinv_off[e] + g;
  double o[S];
#pragma unroll
  for (int s = 0; s < S; s++) o[s] = 0.0;
  for (int j = 0; j < NS; j++) {
    const double t = sv[grp][j];
    const double *col = D + (size_t)j * NS;
#pragma unroll
    for (int s = 0; s < S; s++)
      if (g + DGS_LANES * s < NS) o[s] = fma(col[DGS_LANES * s], t, o[s]);
  }
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int i = g + DGS_LANES * s;
    if (i < NS) out[r0 + i] = o[s];
  }
}

int launch_dg_block_spmv(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                         const long long *row_val, const long long *cx_off, const int *colx, const double *val,
                         const long long *dinv_off, const double *dinv, const double *x, const double *b,
                         double *out) {
  if (count <= 0) return 0;
  GB_CHECK(mode >= 0 && mode <= 2, "bad block SpMV mode");
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
  GB_CHECK(mode == 2 || (dinv && dinv_off), "block SpMV needs the inverted diagonal blocks");
  const int grid = (count + DGS_ROWS - 1) / DGS_ROWS;
#define GB_DGS_LAUNCH(PP)                                                                                  \
  dg_block_spmv_kernel<PP><<<grid, DGS_THREADS, 0, st>>>(mode, count, ent_el, roff, row_val, cx_off, colx, \
                                                         val, dinv_off, dinv, x, b, out)
  switch (p) {
    case 1: GB_DGS_LAUNCH(1); break;
    case 2: GB_DGS_LAUNCH(2); break;
    case 3: GB_DGS_LAUNCH(3); break;
    default: GB_DGS_LAUNCH(4); break;
  }
#undef GB_DGS_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
