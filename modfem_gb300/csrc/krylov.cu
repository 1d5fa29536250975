// CRS residual / SpMV and the BLAS-1 pieces of restarted GMRES, FP64.
//
// SpMV: a group of 4 lanes per row (ModFEM's prism matrices hold about 21
// entries per row), each lane striding through the row, values and column
// indices loaded once (read-only path), a shuffle reduction per group.  The
// kernel is HBM-bound (12 bytes per nonzero) with an FP64 FMA per nonzero;
// on GB300 the two limits are of the same order.
//
// Reductions are two-stage and deterministic (fixed block partition, fixed
// tree order), so GMRES is bit-reproducible run to run.

#include "gbfem_internal.h"

namespace gbfem {

constexpr int SPMV_LANES = 4;
constexpr int RED_THREADS = 256;

// v = (use_rhs ? b : 0) - A x        (mode 0)
// v = scale[r] * (A x)              (mode 1: Jacobi-preconditioned operator)
template <int MODE>
__global__ void __launch_bounds__(256) crs_spmv_kernel(int n, const int *__restrict__ row_ptr,
                                                       const int *__restrict__ col_ind,
                                                       const double *__restrict__ val,
                                                       const double *__restrict__ x,
                                                       const double *__restrict__ b,
                                                       const double *__restrict__ scale,
                                                       double *__restrict__ v) {
  const int lane = threadIdx.x & (SPMV_LANES - 1);
  const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / SPMV_LANES;
  const bool valid = r < n;  // no early exit: every lane takes part in the shuffles
  const int lo = valid ? __ldg(row_ptr + r) : 0, hi = valid ? __ldg(row_ptr + r + 1) : 0;
  double s = 0.0;
  for (int k = lo + lane; k < hi; k += SPMV_LANES) s = fma(__ldg(val + k), __ldg(x + __ldg(col_ind + k)), s);
#pragma unroll
  for (int o = SPMV_LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, SPMV_LANES);
  if (valid && lane == 0) {
    if (MODE == 0)
      v[r] = (b ? __ldg(b + r) : 0.0) - s;
    else
      v[r] = __ldg(scale + r) * s;
  }
}

// dinv[r] = 1 / a_rr (lar_fill_preconditioner_crs, las_crs_intf.c:707)
__global__ void jacobi_diag_kernel(int n, const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                                   const double *__restrict__ val, double *__restrict__ dinv) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 1.0;
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; k++)
    if (col_ind[k] == r) d = 1.0 / val[k];
  dinv[r] = d;
}

// partial[k*nb + blockIdx.x] = sum over this block's rows of A_k[i] * w[i],
// A_k = base + k*ld, for k = blockIdx.y.
__global__ void __launch_bounds__(RED_THREADS) multidot_stage1(int n, const double *__restrict__ base,
                                                               long long ld, const double *__restrict__ w,
                                                               double *__restrict__ partial) {
  const int k = blockIdx.y, nb = gridDim.x;
  const double *a = base + (size_t)k * ld;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += (long long)nb * RED_THREADS)
    s = fma(__ldg(a + i), __ldg(w + i), s);
  __shared__ double sh[RED_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[(size_t)k * nb + blockIdx.x] = s;
  }
}

// out[k] = sum_b partial[k*nb + b]; if sqrt_out, out[k] = sqrt(sum).
__global__ void __launch_bounds__(RED_THREADS) multidot_stage2(int nb, const double *__restrict__ partial,
                                                               double *__restrict__ out, int sqrt_out) {
  const int k = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += RED_THREADS) s += partial[(size_t)k * nb + b];
  __shared__ double sh[RED_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < RED_THREADS / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[k] = sqrt_out ? sqrt(s) : s;
  }
}

// y[i] += sign * sum_{k<m} c[k] * A_k[i]   (c on the device)
__global__ void __launch_bounds__(256) multiaxpy_kernel(int n, int m, const double *__restrict__ c, double sign,
                                                        const double *__restrict__ base, long long ld,
                                                        double *__restrict__ y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < m; k++) s = fma(__ldg(c + k), __ldg(base + (size_t)k * ld + i), s);
  y[i] = fma(sign, s, y[i]);
}

// y[i] = alpha[0]^(power) * y[i] with power -1: divide by alpha; used to normalise.
__global__ void scale_kernel(int n, const double *__restrict__ alpha, int invert, const double *__restrict__ x,
                             double *__restrict__ y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = *alpha;
  y[i] = invert ? x[i] / a : x[i] * a;
}

// v = dinv .* (b - A x)  fused: first residual then scale (two kernels for clarity)
__global__ void mul_kernel(int n, const double *__restrict__ a, double *__restrict__ y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] *= a[i];
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int launch_spmv(cudaStream_t st, int mode, int n, const int *row_ptr, const int *col_ind, const double *val,
                const double *x, const double *b, const double *scale, double *v) {
  if (n <= 0) return 0;
  const int T = 256;
  const unsigned nb = nblk((long long)n * SPMV_LANES, T);
  if (mode == 0)
    crs_spmv_kernel<0><<<nb, T, 0, st>>>(n, row_ptr, col_ind, val, x, b, scale, v);
  else
    crs_spmv_kernel<1><<<nb, T, 0, st>>>(n, row_ptr, col_ind, val, x, b, scale, v);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_jacobi_diag(cudaStream_t st, int n, const int *row_ptr, const int *col_ind, const double *val,
                       double *dinv) {
  jacobi_diag_kernel<<<nblk(n, 256), 256, 0, st>>>(n, row_ptr, col_ind, val, dinv);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int reduction_blocks(int n) {
  int nb = (int)nblk(n, RED_THREADS * 8);
  if (nb > 1216) nb = 1216;  // 8 x 152 SMs
  if (nb < 1) nb = 1;
  return nb;
}

// out[k] = <A_k, w>, k < m (sqrt if requested); partial must hold m*nb doubles.
int launch_multidot(cudaStream_t st, int n, int m, const double *base, long long ld, const double *w,
                    double *partial, double *out, int sqrt_out) {
  const int nb = reduction_blocks(n);
  dim3 g1(nb, m);
  multidot_stage1<<<g1, RED_THREADS, 0, st>>>(n, base, ld, w, partial);
  multidot_stage2<<<m, RED_THREADS, 0, st>>>(nb, partial, out, sqrt_out);
  GB_CUDA(cudaGetLastError());
  return 2;
}

int launch_multiaxpy(cudaStream_t st, int n, int m, const double *c, double sign, const double *base,
                     long long ld, double *y) {
  if (m <= 0) return 0;
  multiaxpy_kernel<<<nblk(n, 256), 256, 0, st>>>(n, m, c, sign, base, ld, y);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_scale(cudaStream_t st, int n, const double *alpha, int invert, const double *x, double *y) {
  scale_kernel<<<nblk(n, 256), 256, 0, st>>>(n, alpha, invert, x, y);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_mul(cudaStream_t st, int n, const double *a, double *y) {
  mul_kernel<<<nblk(n, 256), 256, 0, st>>>(n, a, y);
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem

// ---------------------------------------------------------------------------
// FP64 FMA throughput probe: 8 independent FMA chains per thread held in
// registers, enough blocks to fill every SM several times over.
// ---------------------------------------------------------------------------
namespace gbfem {

__global__ void fp64_fma_chains(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[blockIdx.x] = s;  // never true; keeps the chains live
}

int measure_fp64_peak(cudaStream_t st, int device, double *tflops) {
  int sms = 0;
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  double *out = nullptr;
  GB_CUDA(cudaMalloc(&out, (size_t)sms * 4 * sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 4, threads = 256, iters = 20000;
  fp64_fma_chains<<<blocks, threads, 0, st>>>(out, 200, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0, st);
    fp64_fma_chains<<<blocks, threads, 0, st>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  GB_CUDA(err);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return 0;
}

}  // namespace gbfem
