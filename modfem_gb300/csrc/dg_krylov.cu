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

#include "dg_spmv.cuh"
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

template <int P, typename VT>
__global__ void __launch_bounds__(DGS_THREADS) dg_block_spmv_kernel(
    int mode, int count, const int *__restrict__ ent_el, const int *__restrict__ roff,
    const long long *__restrict__ row_val, const long long *__restrict__ cx_off, const int *__restrict__ colx,
    const VT *__restrict__ val, const long long *__restrict__ dinv_off, const VT *__restrict__ dinv,
    const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ out) {
  __shared__ VT sv[DGS_ROWS][DgSpmvDims<P>::NS];
  dg_block_row_spmv<P, VT>(mode, count, ent_el, roff, row_val, cx_off, colx, val, dinv_off, dinv, x, b, out, sv);
}

// Residual out = b - A x with the products and sums carried in two FP64
// words per row (error-free transformations: the exact product error from an
// FMA, Knuth's TwoSum, the errors summed in a second word and added once at
// the end: the compensated dot product "Dot2" of Ogita, Rump and Oishi,
// SIAM J. Sci. Comput. 26, 2005).  The result is as accurate as if computed
// in twice the working precision, then rounded: iterative refinement driven
// by it reaches a forward error near FP64 rounding whatever the FP64 residual
// floor of a badly scaled system.  Same lane layout as dg_block_row_spmv.
template <int P>
__global__ void __launch_bounds__(DGS_THREADS) dg_block_residual_dd_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ roff, const long long *__restrict__ row_val,
    const long long *__restrict__ cx_off, const int *__restrict__ colx, const double *__restrict__ val,
    const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ out) {
  constexpr int NS = DgSpmvDims<P>::NS;
  constexpr int S = (NS + DGS_LANES - 1) / DGS_LANES;
  const int grp = threadIdx.x / DGS_LANES, g = threadIdx.x % DGS_LANES;
  const int idx = blockIdx.x * DGS_ROWS + grp;
  if (idx >= count) return;
  const int e = ent_el[idx];
  const int r0 = roff[e];
  double hi[S], lo[S];
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int i = g + DGS_LANES * s;
    hi[s] = b && i < NS ? b[r0 + i] : 0.0;
    lo[s] = 0.0;
  }
  const double *A = val + row_val[e] + g;
  const int *cx = colx + cx_off[e];
  const int nct = (int)(cx_off[e + 1] - cx_off[e]);
  for (int t = 0; t < nct; t++) {
    const double xv = -x[cx[t]];
    const double *col = A + (size_t)t * NS;
#pragma unroll
    for (int s = 0; s < S; s++) {
      if (g + DGS_LANES * s >= NS) continue;
      const double a = col[DGS_LANES * s];
      const double p = a * xv;
      const double ep = fma(a, xv, -p);  // exact: a xv = p + ep
      const double sum = hi[s] + p;      // TwoSum(hi, p)
      const double bb = sum - hi[s];
      const double es = (hi[s] - (sum - bb)) + (p - bb);
      hi[s] = sum;
      lo[s] += ep + es;
    }
  }
#pragma unroll
  for (int s = 0; s < S; s++) {
    const int i = g + DGS_LANES * s;
    if (i < NS) out[r0 + i] = hi[s] + lo[s];
  }
}

int launch_dg_block_residual_dd(cudaStream_t st, int p, int count, const int *ent_el, const int *roff,
                                const long long *row_val, const long long *cx_off, const int *colx,
                                const double *val, const double *x, const double *b, double *out) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= 2 * GB_DG_PMAX, "DG block class must be 1..8 (prisms 1..4, tetrahedra 5..8)");
  const int grid = (count + DGS_ROWS - 1) / DGS_ROWS;
#define GB_DGR_LAUNCH(PP)                                                                               \
  dg_block_residual_dd_kernel<PP><<<grid, DGS_THREADS, 0, st>>>(count, ent_el, roff, row_val, cx_off, colx, \
                                                                val, x, b, out)
  switch (p) {
    case 1: GB_DGR_LAUNCH(1); break;
    case 2: GB_DGR_LAUNCH(2); break;
    case 3: GB_DGR_LAUNCH(3); break;
    case 4: GB_DGR_LAUNCH(4); break;
    case 5: GB_DGR_LAUNCH(5); break;
    case 6: GB_DGR_LAUNCH(6); break;
    case 7: GB_DGR_LAUNCH(7); break;
    default: GB_DGR_LAUNCH(8); break;
  }
#undef GB_DGR_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

__global__ void to_float_kernel(long long n, const double *__restrict__ a, float *__restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void to_dw_kernel(long long n, const double *__restrict__ a, dw *__restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = dw_from_double(a[i]);
}

int launch_to_dw(cudaStream_t st, long long n, const double *a, void *b) {
  if (n <= 0) return 0;
  to_dw_kernel<<<152 * 8, 256, 0, st>>>(n, a, reinterpret_cast<dw *>(b));
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_to_float(cudaStream_t st, long long n, const double *a, float *b) {
  if (n <= 0) return 0;
  to_float_kernel<<<152 * 8, 256, 0, st>>>(n, a, b);
  GB_CUDA(cudaGetLastError());
  return 1;
}

template <typename VT>
static int launch_dg_block_spmv_t(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                                  const long long *row_val, const long long *cx_off, const int *colx, const VT *val,
                                  const long long *dinv_off, const VT *dinv, const double *x, const double *b,
                                  double *out) {
  if (count <= 0) return 0;
  GB_CHECK(mode >= 0 && mode <= 2, "bad block SpMV mode");
  GB_CHECK(p >= 1 && p <= 2 * GB_DG_PMAX, "DG block class must be 1..8 (prisms 1..4, tetrahedra 5..8)");
  GB_CHECK(mode == 2 || (dinv && dinv_off), "block SpMV needs the inverted diagonal blocks");
  const int grid = (count + DGS_ROWS - 1) / DGS_ROWS;
#define GB_DGS_LAUNCH(PP)                                                                                      \
  dg_block_spmv_kernel<PP, VT><<<grid, DGS_THREADS, 0, st>>>(mode, count, ent_el, roff, row_val, cx_off, colx, \
                                                             val, dinv_off, dinv, x, b, out)
  switch (p) {
    case 1: GB_DGS_LAUNCH(1); break;
    case 2: GB_DGS_LAUNCH(2); break;
    case 3: GB_DGS_LAUNCH(3); break;
    case 4: GB_DGS_LAUNCH(4); break;
    case 5: GB_DGS_LAUNCH(5); break;
    case 6: GB_DGS_LAUNCH(6); break;
    case 7: GB_DGS_LAUNCH(7); break;
    default: GB_DGS_LAUNCH(8); break;
  }
#undef GB_DGS_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_dg_block_spmv(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                         const long long *row_val, const long long *cx_off, const int *colx, const double *val,
                         const long long *dinv_off, const double *dinv, const double *x, const double *b,
                         double *out) {
  return launch_dg_block_spmv_t<double>(st, mode, p, count, ent_el, roff, row_val, cx_off, colx, val, dinv_off,
                                        dinv, x, b, out);
}

int launch_dg_block_spmv32(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                           const long long *row_val, const long long *cx_off, const int *colx, const float *val,
                           const long long *dinv_off, const float *dinv, const double *x, const double *b,
                           double *out) {
  return launch_dg_block_spmv_t<float>(st, mode, p, count, ent_el, roff, row_val, cx_off, colx, val, dinv_off,
                                       dinv, x, b, out);
}

int launch_dg_block_spmv_dw(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                           const long long *row_val, const long long *cx_off, const int *colx, const void *val,
                           const long long *dinv_off, const void *dinv, const double *x, const double *b,
                           double *out) {
  return launch_dg_block_spmv_t<dw>(st, mode, p, count, ent_el, roff, row_val, cx_off, colx,
                                    reinterpret_cast<const dw *>(val), dinv_off, reinterpret_cast<const dw *>(dinv),
                                    x, b, out);
}

}  // namespace gbfem
