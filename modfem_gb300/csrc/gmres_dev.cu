// Device-resident restarted GMRES(m) with point Jacobi for the std CRS
// matrix (gbfem_solve).  Same algorithm, stopping rule and iteration count as
// lsr_mkb_core_gmres (lsd_mkb/lsd_mkb_core/lss_mkb_core.c:2317-2660): left
// preconditioning by 1 / a_ii (lar_fill_preconditioner_crs,
// lad_crs/las_crs_intf.c:707), classical Gram-Schmidt, Givens rotations,
// stopping on the preconditioned residual relative to the initial one with
// both tolerances floored at 1e-12 (lss_mkb_core.c:2377-2378).
//
// Nothing of an Arnoldi step goes through the host: the Hessenberg column,
// the rotations, the convergence test and the small triangular solve run on
// the device, and every kernel of a restart cycle (restart residual, m
// Arnoldi steps, update of x) reads a state word and returns at once when the
// cycle has already ended.  An Arnoldi step is three kernels: the SpMV, the
// Gram-Schmidt dot products (the last block of each column entry to finish
// sums its block partials) and the orthogonalisation, one row a thread (its
// last block to finish runs the step's logic: norm, Givens rotations, test).
// Krylov vectors after the first are stored unnormalised with a scale each
// (V_k = sc_k W_k), applied by their readers, so no normalisation pass runs;
// the cycle's triangular solve runs in the update of x.  "Last block" is an
// atomic count after a memory fence: nothing waits.  One cycle is captured
// as a CUDA graph (per context, matrix size and Krylov dimension) and
// replayed; the host reads the state once per cycle.
//
// The SpMV runs on a sliced-ELL copy of the CRS matrix (SELL-32 in natural
// row order: slice s = rows 32 s .. 32 s + 31, padded to the slice's longest
// row; ModFEM's prism matrices hold 6..21 entries per row, so padding adds
// about 1 %): a warp reads 32 consecutive values and 32 consecutive column
// indices per step (fully coalesced 256 B and 128 B lines) instead of the
// short scattered row segments of the CRS kernel; column indices take 16
// bits where they fit (see sell_base).  The values are either FP64
// or double words (float pairs h + l, the same 8 bytes): with double words
// the products run on the FP32 pipes and the kernel is bound by HBM alone
// (GB300's FP64 pipe, ~0.6 T FMA/s, is itself near the HBM rate for one FMA
// per 12 bytes).  The copy holds the rows of D^-1 A (the point-Jacobi
// scaling folded in once per solve), so the product reads no preconditioner.
// Row sums run in column order in one thread, as the reference's loop does.
// Reductions are two-stage over a fixed block partition and fixed tree
// order: the solve is bit-reproducible.

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "dword.cuh"
#include "gbfem_internal.h"

namespace gbfem {

constexpr int GM_T = 256;
constexpr int GM_MMAX = 256;  // largest Krylov dimension (gbfem_solve's check)
constexpr int GM_RSTAGE = 64;  // Krylov dimensions up to which the triangular solve runs on a shared copy of R
constexpr int SELL_C = 32;

// ---------------------------------------------------------------- SELL-32
// Column indices are stored relative to the lane's base row min(r, n - 1) in
// 16 bits when every |column - base| of the matrix fits (ModFEM's first-
// appearance dof order keeps a prism row's columns within about one mesh
// layer of the row: 10 bytes a value instead of 12), as absolute 32-bit
// indices otherwise.
__device__ __forceinline__ int sell_base(int r, int n) { return r < n ? r : n - 1; }

// width[s]: the slice's longest row; fits[s]: every column within 16 bits of its base
__global__ void sell_width_kernel(int n, int nslices, const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                                  int *__restrict__ width, int *__restrict__ fits) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int w = 0, ok = 1;
  for (int l = 0; l < SELL_C; l++) {
    const int r = s * SELL_C + l;
    if (r >= n) continue;
    w = max(w, row_ptr[r + 1] - row_ptr[r]);
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
      const int d = col_ind[k] - r;
      ok &= d >= -32768 && d <= 32767;
    }
  }
  width[s] = w;
  fits[s] = ok;
}

// columns of slice s: entry j of lane l at off[s] + 32 j + l; padding entries
// point at the lane's base row with value 0
template <typename CT>
__global__ void sell_cols_kernel(int n, int nslices, const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                                 const int *__restrict__ off, CT *__restrict__ col) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(t / SELL_C), l = (int)(t % SELL_C);
  if (s >= nslices) return;
  const int r = s * SELL_C + l, base = sell_base(r, n);
  const int w = (off[s + 1] - off[s]) / SELL_C;
  const int lo = r < n ? row_ptr[r] : 0, len = r < n ? row_ptr[r + 1] - lo : 0;
  for (int j = 0; j < w; j++) {
    const int c = j < len ? col_ind[lo + j] : base;
    col[off[s] + SELL_C * j + l] = sizeof(CT) == 2 ? (CT)(c - base) : (CT)c;
  }
}

// the values and columns stream through once per product: loaded with the
// evict-first hint (ld.global.cs) so that L2 keeps the gathered vector
__device__ __forceinline__ int sell_col(const int *p, int) { return __ldcs(p); }
__device__ __forceinline__ int sell_col(const short *p, int base) { return base + (int)__ldcs(p); }
__device__ __forceinline__ double sell_ld(const double *p) { return __ldcs(p); }
__device__ __forceinline__ float2 sell_ld(const float2 *p) { return __ldcs(p); }

template <typename VT>
__device__ __forceinline__ VT sell_value(double v);
template <>
__device__ __forceinline__ double sell_value<double>(double v) {
  return v;
}
template <>
__device__ __forceinline__ float2 sell_value<float2>(double v) {
  return dw_f2(v);
}

// the rows of the Jacobi-preconditioned matrix D^-1 A (dinv[r] a_rj): the
// preconditioner is folded into the copy, so the product reads no dinv
template <typename VT>
__global__ void sell_vals_kernel(int n, int nslices, const int *__restrict__ row_ptr, const double *__restrict__ val,
                                 const double *__restrict__ dinv, const int *__restrict__ off, VT *__restrict__ sv) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(t / SELL_C), l = (int)(t % SELL_C);
  if (s >= nslices) return;
  const int r = s * SELL_C + l;
  const int w = (off[s + 1] - off[s]) / SELL_C;
  const int lo = r < n ? row_ptr[r] : 0, len = r < n ? row_ptr[r + 1] - lo : 0;
  const double d = r < n ? dinv[r] : 0.0;
  for (int j = 0; j < w; j++) sv[off[s] + SELL_C * j + l] = sell_value<VT>(j < len ? d * val[lo + j] : 0.0);
}

// one row per thread, a warp per slice: acc = sum_j val * x[col], in column
// order; eight entries' loads are issued before their products
__device__ __forceinline__ void sell_acc(double &acc, double a, double x) { acc = fma(a, x, acc); }
__device__ __forceinline__ void sell_acc(dw &acc, float2 a, double x) { acc = t_fma(dw(a.x, a.y), dw_from_double(x), acc); }
__device__ __forceinline__ double sell_out(double acc) { return acc; }
__device__ __forceinline__ double sell_out(dw acc) { return dw_to_double(acc); }

// double-word form: values and the vector both as float pairs (the vector's
// pair copy is written where the Arnoldi vector is formed), products summed
// exactly (TwoProd) with their errors collected (DwAcc), two accumulators
// (even and odd entries) so that the TwoSum chains overlap
template <typename CT>
__device__ __forceinline__ double sell_row_dw(const float2 *__restrict__ v, const CT *__restrict__ col, int w,
                                              int base, const float2 *__restrict__ x) {
  constexpr int U = 8;
  DwAcc acc0 = {0.0f, 0.0f, 0.0f}, acc1 = {0.0f, 0.0f, 0.0f};
  int j = 0;
  for (; j + U <= w; j += U) {
    float2 a[U], xv[U];
#pragma unroll
    for (int u = 0; u < U; u++) a[u] = sell_ld(v + u * SELL_C);
#pragma unroll
    for (int u = 0; u < U; u++) xv[u] = __ldg(x + sell_col(col + u * SELL_C, base));
#pragma unroll
    for (int u = 0; u < U; u += 2) {
      dwacc_prod(acc0, a[u], xv[u]);
      dwacc_prod(acc1, a[u + 1], xv[u + 1]);
    }
    v += U * SELL_C;
    col += U * SELL_C;
  }
  for (; j < w; j++) {
    dwacc_prod(acc0, sell_ld(v), __ldg(x + sell_col(col, base)));
    v += SELL_C;
    col += SELL_C;
  }
  dwacc_fold(acc0);
  dwacc_fold(acc1);
  return dw_to_double(dw(acc0.h, acc0.l) + dw(acc1.h, acc1.l));
}

template <typename VT, typename CT>
__device__ __forceinline__ double sell_row(const VT *__restrict__ v, const CT *__restrict__ col, int w, int base,
                                           const double *__restrict__ x) {
  using AT = typename std::conditional<sizeof(VT) == 8 && std::is_same<VT, double>::value, double, dw>::type;
  constexpr int U = 8;  // entries whose loads are in flight together
  AT acc = AT(0.0);
  int j = 0;
  for (; j + U <= w; j += U) {
    VT a[U];
    double xv[U];
#pragma unroll
    for (int u = 0; u < U; u++) a[u] = sell_ld(v + u * SELL_C);
#pragma unroll
    for (int u = 0; u < U; u++) xv[u] = __ldg(x + sell_col(col + u * SELL_C, base));
#pragma unroll
    for (int u = 0; u < U; u++) sell_acc(acc, a[u], xv[u]);
    v += U * SELL_C;
    col += U * SELL_C;
  }
  for (; j < w; j++) {
    sell_acc(acc, sell_ld(v), __ldg(x + sell_col(col, base)));
    v += SELL_C;
    col += SELL_C;
  }
  return sell_out(acc);
}

// ---------------------------------------------------------------- state
enum { GM_RESTART = 0, GM_ARNOLDI = 1, GM_DONE = 2 };

struct GmState {
  int phase, j, it, done_cols, final_flag, m, max_iter, pad;
  double beta0, resid, beta, hn, tol_rel, tol_abs;
};

// device arrays of one solve
struct GmArgs {
  int n, nslices, nb;
  const int *row_ptr, *col_ind, *sell_off, *sell_col32;
  const short *sell_col16;  // one of the two column arrays is set
  const double *val, *sell_val64;
  const float2 *sell_valdw;
  const double *dinv, *b;
  double *x, *V, *tmp, *H, *cs, *sn, *s, *y, *hcol, *partial;
  double *sc;  // scale of each Krylov vector: V_k = sc_k W_k, W_k stored
  float2 *xdw;  // double-word copy of the current Arnoldi vector (double-word SpMV only)
  GmState *st;
  int ng;          // blocks of the row-parallel kernels
  double *npart;   // [ng] their norm partials
  unsigned *cnt;   // [m + 2] finished-block counts (dot products 0..m-1, orthogonalisation m + 1)
};

// sum of nb partials in a fixed order (one block of GM_T threads); valid in thread 0
__device__ double gm_block_total(const double *partial, int nb) {
  __shared__ double sh[GM_T];
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += GM_T) v += partial[b];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = GM_T / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  return sh[0];
}

__device__ __forceinline__ double gm_block_sum(double s) {
  __shared__ double sh[GM_T / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < GM_T / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;
}

// restart residual tmp = dinv (b - A x), FP64 (CRS rows, 4 lanes a row, or
// the FP64 SELL copy)
__global__ void __launch_bounds__(GM_T) gm_restart_residual(GmArgs a) {
  const GmState &S = *a.st;
  if (S.phase != GM_RESTART || S.final_flag) return;
  if (a.sell_val64) {
    const int s = blockIdx.x * (GM_T / 32) + threadIdx.x / 32, l = threadIdx.x & 31;
    if (s >= a.nslices) return;
    const int r = s * SELL_C + l, base = sell_base(r, a.n);
    const int o = a.sell_off[s], w = (a.sell_off[s + 1] - o) / SELL_C;
    const double acc = a.sell_col16 ? sell_row(a.sell_val64 + o + l, a.sell_col16 + o + l, w, base, a.x)
                                    : sell_row(a.sell_val64 + o + l, a.sell_col32 + o + l, w, base, a.x);
    if (r < a.n) a.tmp[r] = a.dinv[r] * a.b[r] - acc;  // the copy holds D^-1 A
    return;
  }
  const int lane = threadIdx.x & 3;
  const long long r = ((long long)blockIdx.x * GM_T + threadIdx.x) / 4;
  const bool valid = r < a.n;
  const int lo = valid ? a.row_ptr[r] : 0, hi = valid ? a.row_ptr[r + 1] : 0;
  double s = 0.0;
  for (int k = lo + lane; k < hi; k += 4) s = fma(__ldg(a.val + k), __ldg(a.x + __ldg(a.col_ind + k)), s);
  s += __shfl_down_sync(0xffffffffu, s, 2, 4);
  s += __shfl_down_sync(0xffffffffu, s, 1, 4);
  if (valid && lane == 0) a.tmp[r] = (a.b[r] - s) * a.dinv[r];
}

// partial[b] = sum over block b's entries of v^2 (v = tmp, or V[j+1])
template <int WHICH>
__global__ void __launch_bounds__(GM_T) gm_norm_partial(GmArgs a, int j) {
  const GmState &S = *a.st;
  if (WHICH == 0 ? (S.phase != GM_RESTART || S.final_flag) : (S.phase != GM_ARNOLDI || S.j != j)) return;
  const double *v = WHICH == 0 ? a.tmp : a.V + (size_t)(j + 1) * a.n;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * GM_T + threadIdx.x; i < a.n; i += (long long)gridDim.x * GM_T)
    s = fma(v[i], v[i], s);
  s = gm_block_sum(s);
  if (threadIdx.x == 0) a.partial[blockIdx.x] = s;
}

// the restart test (lss_mkb_core.c:2377-2400) and the start of a cycle
__global__ void __launch_bounds__(GM_T) gm_logic_restart(GmArgs a) {
  GmState &S = *a.st;
  if (S.phase != GM_RESTART) return;
  const double tot = gm_block_total(a.partial, a.nb);
  if (threadIdx.x != 0) return;
  S.done_cols = 0;
  if (S.final_flag) {
    S.phase = GM_DONE;
    return;
  }
  const double rn = sqrt(tot);
  if (S.beta0 < 0) S.beta0 = rn;
  S.resid = rn;
  if (rn < S.tol_abs || (S.beta0 > 0 && rn / S.beta0 < S.tol_rel) || S.it >= S.max_iter) {
    S.phase = GM_DONE;
    return;
  }
  a.s[0] = rn;
  for (int i = 1; i <= S.m; i++) a.s[i] = 0.0;
  a.sc[0] = 1.0;  // V_0 is stored normalised
  S.beta = rn;
  S.j = 0;
  S.phase = GM_ARNOLDI;
}

__global__ void __launch_bounds__(GM_T) gm_start_cycle(GmArgs a) {
  const GmState &S = *a.st;
  if (S.phase != GM_ARNOLDI || S.j != 0) return;
  const double inv = 1.0 / S.beta;
  for (long long i = (long long)blockIdx.x * GM_T + threadIdx.x; i < a.n; i += (long long)gridDim.x * GM_T) {
    const double v = a.tmp[i] * inv;
    a.V[i] = v;
    if (a.xdw) a.xdw[i] = dw_f2(v);
  }
}

// V[j+1] = dinv A V[j]
template <typename VT, typename CT>
__global__ void __launch_bounds__(GM_T) gm_arnoldi_spmv(GmArgs a, const VT *__restrict__ sv,
                                                        const CT *__restrict__ scol, int j) {
  const GmState &S = *a.st;
  if (S.phase != GM_ARNOLDI || S.j != j) return;
  const int s = blockIdx.x * (GM_T / 32) + threadIdx.x / 32, l = threadIdx.x & 31;
  if (s >= a.nslices) return;
  const int r = s * SELL_C + l;
  const int o = a.sell_off[s], w = (a.sell_off[s + 1] - o) / SELL_C;
  double acc;
  if constexpr (std::is_same<VT, float2>::value)
    acc = sell_row_dw(sv + o + l, scol + o + l, w, sell_base(r, a.n), a.xdw);
  else
    acc = sell_row(sv + o + l, scol + o + l, w, sell_base(r, a.n), a.V + (size_t)j * a.n);
  // the copy holds D^-1 A; W_j is stored unnormalised: V_j = sc_j W_j
  if (r < a.n) a.V[(size_t)(j + 1) * a.n + r] = a.sc[j] * acc;
}

// Gram-Schmidt dot products <W_k, w>, k = blockIdx.y <= j (w = W_{j+1}),
// block partials; the last block of each
// k to finish (an atomic count after a fence, no waiting) sums the partials
// in block order (one warp, lane-strided then a shuffle tree) and stores the
// column entry h_k = <V_k, w> = sc_k total.  Partials of other blocks are
// read through L2 (__ldcg).
__global__ void __launch_bounds__(GM_T) gm_dot_partial(GmArgs a, int j) {
  const GmState &S = *a.st;
  if (S.phase != GM_ARNOLDI || S.j != j) return;
  __shared__ bool last;
  const int k = blockIdx.y;
  const double *v = a.V + (size_t)k * a.n, *w = a.V + (size_t)(j + 1) * a.n;
  double s0 = 0.0;
  for (long long i = (long long)blockIdx.x * GM_T + threadIdx.x; i < a.n; i += (long long)gridDim.x * GM_T)
    s0 = fma(__ldg(v + i), __ldg(w + i), s0);
  const double s = gm_block_sum(s0);
  if (threadIdx.x == 0) {
    a.partial[(size_t)k * a.nb + blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(a.cnt + k, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  double t = 0.0;
  for (int b = threadIdx.x; b < a.nb; b += 32) t += __ldcg(a.partial + (size_t)k * a.nb + b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) {
    a.hcol[k] = a.sc[k] * t;
    a.cnt[k] = 0;  // for the next step
  }
}

// The step's logic, by the last block of gm_orthogonalize: |w| from the
// norm partials, the Hessenberg column j with the earlier rotations applied
// (column and rotations staged in shared memory: thread 0's chain of
// dependent operations then waits on no global memory), the new rotation,
// the residual estimate and the decision (next step, or end of the cycle).
__device__ void gm_step_logic(const GmArgs &a, int j, GmState &S) {
  __shared__ double col[GM_MMAX + 2], rc[GM_MMAX + 1], rs[GM_MMAX + 1];
  const int tid = threadIdx.x;
  double v = 0.0;
  for (int b = tid; b < a.ng; b += GM_T) v += __ldcg(a.npart + b);
  __shared__ double sh[GM_T];
  sh[tid] = v;
  for (int k = tid; k <= j; k += GM_T) col[k] = __ldcg(a.hcol + k);
  for (int k = tid; k < j; k += GM_T) {
    rc[k] = a.cs[k];
    rs[k] = a.sn[k];
  }
  __syncthreads();
  for (int o = GM_T / 2; o > 0; o >>= 1) {
    if (tid < o) sh[tid] += sh[tid + o];
    __syncthreads();
  }
  if (tid != 0) return;
  const int m = S.m, ld = m + 1;
  const double hn = sqrt(sh[0]);
  col[j + 1] = hn;
  for (int k = 0; k < j; k++) {
    const double x0 = col[k], x1 = col[k + 1];
    col[k] = rc[k] * x0 + rs[k] * x1;
    col[k + 1] = rc[k] * x1 - rs[k] * x0;
  }
  const double x0 = col[j], x1 = col[j + 1];
  const double rr = hypot(x0, x1), cj = x0 / rr, sj = x1 / rr;
  col[j] = rr;
  col[j + 1] = 0.0;
  double *H = a.H + (size_t)j * ld;
  for (int k = 0; k <= j + 1; k++) H[k] = col[k];
  a.cs[j] = cj;
  a.sn[j] = sj;
  const double s0 = a.s[j];
  a.s[j] = cj * s0;
  const double s1 = -sj * s0;
  a.s[j + 1] = s1;
  const int it = S.it + 1;
  const double resid = fabs(s1);
  S.it = it;
  S.resid = resid;
  S.hn = hn;
  a.sc[j + 1] = 1.0 / hn;
  const bool conv = resid < S.tol_abs || resid / S.beta0 < S.tol_rel;
  if (j == m - 1 || it >= S.max_iter || conv) {
    S.done_cols = j + 1;  // the triangular solve runs in gm_update_x
    S.final_flag = (conv || it >= S.max_iter) ? 1 : 0;
    S.phase = GM_RESTART;
  } else {
    S.j = j + 1;
  }
}

// w = W_{j+1} -= sum_k h_k sc_k W_k (one row a thread), the block partials
// of its squared norm and its double-word copy for the next SpMV; the last
// block to finish then runs the step's logic.
__global__ void __launch_bounds__(GM_T) gm_orthogonalize(GmArgs a, int j) {
  GmState &S = *a.st;
  if (S.phase != GM_ARNOLDI || S.j != j) return;
  __shared__ double coef[GM_MMAX + 1];
  __shared__ bool last;
  for (int k = threadIdx.x; k <= j; k += GM_T) coef[k] = a.hcol[k] * a.sc[k];
  __syncthreads();
  double *w = a.V + (size_t)(j + 1) * a.n;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * GM_T + threadIdx.x; i < a.n; i += (long long)gridDim.x * GM_T) {
    double acc = 0.0;
    for (int k = 0; k <= j; k++) acc = fma(coef[k], __ldg(a.V + (size_t)k * a.n + i), acc);
    const double wi = w[i] - acc;
    w[i] = wi;
    if (a.xdw) a.xdw[i] = dw_f2(wi);
    s = fma(wi, wi, s);
  }
  s = gm_block_sum(s);
  if (threadIdx.x == 0) {
    a.npart[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(a.cnt + S.m + 1, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x == 0) a.cnt[S.m + 1] = 0;  // for the next step
  gm_step_logic(a, j, S);
}

// At the end of a cycle: y from the triangular system R y = s (every block
// solves it, the same arithmetic in each: thread 0 on a shared-memory copy
// of R when the Krylov dimension is at most GM_RSTAGE, else on R in global
// memory), then x += sum_k y_k V_k, one row a thread.
__global__ void __launch_bounds__(GM_T) gm_update_x(GmArgs a) {
  const GmState &S = *a.st;
  if (S.phase != GM_RESTART || S.done_cols == 0) return;
  __shared__ double R[GM_RSTAGE * GM_RSTAGE], yc[GM_MMAX + 1];
  const int done = S.done_cols, ld = S.m + 1, tid = threadIdx.x;
  const bool staged = done <= GM_RSTAGE;
  if (staged)
    for (int t = tid; t < done * done; t += GM_T) R[t] = a.H[(size_t)(t / done) * ld + t % done];  // column t / done
  __syncthreads();
  if (tid == 0) {
    for (int k = done - 1; k >= 0; k--) {
      double v = a.s[k];
      if (staged)
        for (int i = k + 1; i < done; i++) v -= R[i * done + k] * yc[i];
      else
        for (int i = k + 1; i < done; i++) v -= a.H[k + (size_t)i * ld] * yc[i];
      yc[k] = v / (staged ? R[k * done + k] : a.H[k + (size_t)k * ld]);
    }
    for (int k = 0; k < done; k++) yc[k] *= a.sc[k];  // to the stored W_k
  }
  __syncthreads();
  for (long long i = (long long)blockIdx.x * GM_T + tid; i < a.n; i += (long long)gridDim.x * GM_T) {
    double acc = 0.0;
    for (int k = 0; k < done; k++) acc = fma(yc[k], __ldg(a.V + (size_t)k * a.n + i), acc);
    a.x[i] += acc;
  }
}

}  // namespace gbfem

using gbfem::DevBuf;
using gbfem::GmArgs;
using gbfem::GmState;

namespace {

unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// SELL-32 index arrays of the context's structure (once per structure)
int build_sell(gbfem_ctx c) {
  const int n = c->ndof, ns = (n + gbfem::SELL_C - 1) / gbfem::SELL_C;
  if (c->sell_ready && c->sell_n == n && c->sell_nnz == c->nnz) return 0;
  GB_TRY(c->sell_off.alloc((size_t)2 * ns + 1));
  gbfem::sell_width_kernel<<<nblk(ns, 256), 256, 0, c->stream>>>(n, ns, c->row_ptr.p, c->col_ind.p, c->sell_off.p,
                                                                 c->sell_off.p + ns);
  GB_CUDA(cudaGetLastError());
  std::vector<int> w(2 * (size_t)ns), off(ns + 1);
  GB_CUDA(cudaMemcpyAsync(w.data(), c->sell_off.p, 2 * (size_t)ns * sizeof(int), cudaMemcpyDeviceToHost,
                          c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  bool fits16 = true;
  for (int s = 0; s < ns; s++) fits16 = fits16 && w[ns + s];
  long long tot = 0;
  for (int s = 0; s < ns; s++) {
    off[s] = (int)tot;
    tot += (long long)gbfem::SELL_C * w[s];
  }
  GB_CHECK(tot < 2147483647LL, "matrix too large for the sliced-ELL copy");
  off[ns] = (int)tot;
  GB_CUDA(cudaMemcpyAsync(c->sell_off.p, off.data(), (size_t)(ns + 1) * sizeof(int), cudaMemcpyHostToDevice,
                          c->stream));
  const unsigned gc = nblk((long long)ns * gbfem::SELL_C, 256);
  if (fits16) {
    c->sell_col.release();
    GB_TRY(c->sell_col16.alloc((size_t)std::max<long long>(tot, 1)));
    gbfem::sell_cols_kernel<short><<<gc, 256, 0, c->stream>>>(n, ns, c->row_ptr.p, c->col_ind.p, c->sell_off.p,
                                                                c->sell_col16.p);
  } else {
    c->sell_col16.release();
    GB_TRY(c->sell_col.alloc((size_t)std::max<long long>(tot, 1)));
    gbfem::sell_cols_kernel<int><<<gc, 256, 0, c->stream>>>(n, ns, c->row_ptr.p, c->col_ind.p, c->sell_off.p,
                                                              c->sell_col.p);
  }
  GB_CUDA(cudaGetLastError());
  c->sell_cols16 = fits16;
  GB_CUDA(cudaStreamSynchronize(c->stream));  // off[] is a stack vector
  c->sell_total = tot;
  c->sell_n = n;
  c->sell_nnz = c->nnz;
  c->sell_ready = true;
  return 0;
}

// the values of the current matrix into the SELL copy (every solve)
int fill_sell_values(gbfem_ctx c) {
  const int n = c->ndof, ns = (n + gbfem::SELL_C - 1) / gbfem::SELL_C;
  const unsigned g = nblk((long long)ns * gbfem::SELL_C, 256);
  if (c->std_spmv_dword) {
    GB_TRY(c->sell_valdw.alloc((size_t)std::max<long long>(c->sell_total, 1)));
    gbfem::sell_vals_kernel<float2><<<g, 256, 0, c->stream>>>(n, ns, c->row_ptr.p, c->val.p, c->dinv.p,
                                                               c->sell_off.p, c->sell_valdw.p);
  } else {
    GB_TRY(c->sell_val.alloc((size_t)std::max<long long>(c->sell_total, 1)));
    gbfem::sell_vals_kernel<double><<<g, 256, 0, c->stream>>>(n, ns, c->row_ptr.p, c->val.p, c->dinv.p,
                                                               c->sell_off.p, c->sell_val.p);
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

// Captures one restart cycle: restart residual and test, m Arnoldi steps,
// update of x.  Events around the first step's SpMV time it in every replay.
int capture_cycle(gbfem_ctx c, const GmArgs &a, int m, bool dword, int *kernels) {
  cudaStream_t st = c->stream;
  const int ns = a.nslices;
  const unsigned gs = nblk(ns, gbfem::GM_T / 32);
  const unsigned gcrs = nblk((long long)a.n * 4, gbfem::GM_T);
  const unsigned gv = (unsigned)a.nb;
  int k = 0;
  cudaGraph_t graph = nullptr;
  GB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  gbfem::gm_restart_residual<<<a.sell_val64 ? gs : gcrs, gbfem::GM_T, 0, st>>>(a);
  gbfem::gm_norm_partial<0><<<gv, gbfem::GM_T, 0, st>>>(a, 0);
  gbfem::gm_logic_restart<<<1, gbfem::GM_T, 0, st>>>(a);
  gbfem::gm_start_cycle<<<gv, gbfem::GM_T, 0, st>>>(a);
  k += 4;
  for (int j = 0; j < m; j++) {
    if (j == 0) cudaEventRecordWithFlags(c->ev2, st, cudaEventRecordExternal);
    if (dword) {
      if (a.sell_col16)
        gbfem::gm_arnoldi_spmv<<<gs, gbfem::GM_T, 0, st>>>(a, a.sell_valdw, a.sell_col16, j);
      else
        gbfem::gm_arnoldi_spmv<<<gs, gbfem::GM_T, 0, st>>>(a, a.sell_valdw, a.sell_col32, j);
    } else {
      if (a.sell_col16)
        gbfem::gm_arnoldi_spmv<<<gs, gbfem::GM_T, 0, st>>>(a, a.sell_val64, a.sell_col16, j);
      else
        gbfem::gm_arnoldi_spmv<<<gs, gbfem::GM_T, 0, st>>>(a, a.sell_val64, a.sell_col32, j);
    }
    if (j == 0) cudaEventRecordWithFlags(c->ev3, st, cudaEventRecordExternal);
    gbfem::gm_dot_partial<<<dim3(gv, j + 1), gbfem::GM_T, 0, st>>>(a, j);
    gbfem::gm_orthogonalize<<<(unsigned)a.ng, gbfem::GM_T, 0, st>>>(a, j);
    k += 3;
  }
  gbfem::gm_update_x<<<(unsigned)a.ng, gbfem::GM_T, 0, st>>>(a);
  k += 1;
  const cudaError_t e1 = cudaGetLastError();
  const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
  GB_CUDA(e1);
  GB_CUDA(e2);
  if (c->gm_graph) cudaGraphExecDestroy(c->gm_graph);
  c->gm_graph = nullptr;
  const cudaError_t e3 = cudaGraphInstantiate(&c->gm_graph, graph, 0);
  cudaGraphDestroy(graph);
  GB_CUDA(e3);
  *kernels = k;
  return 0;
}

}  // namespace

namespace gbfem {

// gbfem_solve's body: see the file comment.
int gmres_device_std(gbfem_ctx c, int krylov, int max_iter, double tol_rel, int ini_zero, double *x,
                     double *res_out, double *res_rel_out) {
  const int n = c->ndof, m = krylov;
  cudaStream_t st = c->stream;
  GB_TRY(build_sell(c));
  GB_TRY(c->dinv.alloc(n));
  GB_TRY(launch_jacobi_diag(st, n, c->row_ptr.p, c->col_ind.p, c->val.p, c->dinv.p));
  GB_TRY(fill_sell_values(c));
  const int nb = reduction_blocks(n);
  GB_TRY(c->V.alloc((size_t)n * (m + 1)));
  GB_TRY(c->x.alloc(n));
  GB_TRY(c->tmp.alloc(n));
  GB_TRY(c->partial.alloc((size_t)nb * (m + 2)));
  // row-parallel grid: one row a thread up to 8 blocks per SM (1,216 on
  // GB300), beyond that a grid-stride loop (every block counts itself into
  // one atomic word at the end of the step)
  const int ng = (int)std::min<unsigned>(nblk(n, GM_T), 1216u);
  GB_TRY(c->gm_npart.alloc((size_t)ng));
  GB_TRY(c->gm_cnt.alloc((size_t)m + 2));
  GB_CUDA(cudaMemsetAsync(c->gm_cnt.p, 0, ((size_t)m + 2) * sizeof(unsigned), st));
  // H (m+1)^2, cs, sn, s (m+1 each), y (m), hcol (m+1), sc (m+1), state
  const size_t nsmall = (size_t)(m + 1) * (m + 1) + 3 * (size_t)(m + 1) + m + 2 * (size_t)(m + 1) + 16;
  GB_TRY(c->gm_small.alloc(nsmall));
  double *H = c->gm_small.p, *cs = H + (size_t)(m + 1) * (m + 1), *sn = cs + (m + 1), *s = sn + (m + 1),
         *y = s + (m + 1), *hcol = y + m, *scv = hcol + (m + 1);
  GmState *state = reinterpret_cast<GmState *>(scv + (m + 1));
  GmArgs a;
  memset(&a, 0, sizeof(a));  // padding too: the struct is compared bytewise below
  a.n = n;
  a.nslices = (n + SELL_C - 1) / SELL_C;
  a.nb = nb;
  a.row_ptr = c->row_ptr.p;
  a.col_ind = c->col_ind.p;
  a.sell_off = c->sell_off.p;
  a.sell_col32 = c->sell_cols16 ? nullptr : c->sell_col.p;
  a.sell_col16 = c->sell_cols16 ? c->sell_col16.p : nullptr;
  a.val = c->val.p;
  a.sell_val64 = c->std_spmv_dword ? nullptr : c->sell_val.p;
  a.sell_valdw = c->std_spmv_dword ? c->sell_valdw.p : nullptr;
  a.dinv = c->dinv.p;
  a.b = c->rhs.p;
  a.x = c->x.p;
  a.V = c->V.p;
  a.tmp = c->tmp.p;
  a.H = H;
  a.cs = cs;
  a.sn = sn;
  a.s = s;
  a.y = y;
  a.hcol = hcol;
  a.sc = scv;
  a.partial = c->partial.p;
  a.ng = ng;
  a.npart = c->gm_npart.p;
  a.cnt = c->gm_cnt.p;
  if (c->std_spmv_dword) {
    GB_TRY(c->gm_xdw.alloc(n));
    a.xdw = c->gm_xdw.p;
  }
  a.st = state;
  if (ini_zero)
    GB_CUDA(cudaMemsetAsync(c->x.p, 0, (size_t)n * sizeof(double), st));
  else
    GB_CUDA(cudaMemcpyAsync(c->x.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  GmState h{};
  h.phase = GM_RESTART;
  h.m = m;
  h.max_iter = max_iter;
  h.beta0 = -1.0;
  h.tol_abs = 1e-12;
  h.tol_rel = tol_rel < 1e-12 ? 1e-12 : tol_rel;
  GB_CUDA(cudaMemcpyAsync(state, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  // the graph bakes in every pointer and size: capture again when one changed
  static_assert(sizeof(GmArgs) <= sizeof(c->gm_key_args), "graph key too small");
  const bool same = c->gm_graph && c->gm_key_n == n && c->gm_key_m == m && c->gm_key_dw == c->std_spmv_dword &&
                    memcmp(c->gm_key_args, &a, sizeof(a)) == 0;
  int kernels_per_cycle = c->gm_kernels;
  if (!same) {
    GB_TRY(capture_cycle(c, a, m, c->std_spmv_dword, &kernels_per_cycle));
    c->gm_key_n = n;
    c->gm_key_m = m;
    c->gm_key_dw = c->std_spmv_dword;
    memcpy(c->gm_key_args, &a, sizeof(a));
    c->gm_kernels = kernels_per_cycle;
  }
  GmState *hs = nullptr;
  GB_CUDA(cudaMallocHost(&hs, sizeof(GmState)));
  float spmv_ms = 0.f;
  int spmv_n = 0, cycles = 0, it_prev = 0;
  cudaEventRecord(c->ev0, st);
  int rc = 0;
  for (;;) {
    if (cudaGraphLaunch(c->gm_graph, st) != cudaSuccess ||
        cudaMemcpyAsync(hs, state, sizeof(GmState), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("GMRES cycle launch failed");
      rc = -1;
      break;
    }
    cycles++;
    if (hs->it > it_prev) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, c->ev2, c->ev3) == cudaSuccess) {
        spmv_ms += ms;
        spmv_n++;
      }
    }
    it_prev = hs->it;
    if (hs->phase == GM_DONE || hs->final_flag) break;
  }
  cudaEventRecord(c->ev1, st);
  const GmState fin = *hs;
  cudaFreeHost(hs);
  GB_TRY(rc);
  GB_CUDA(cudaMemcpyAsync(x, c->x.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  cudaEventElapsedTime(&c->last_solve_ms, c->ev0, c->ev1);
  // one SpMV per iteration: the timed samples stand for all of them
  c->last_spmv_ms = spmv_n ? spmv_ms / spmv_n * fin.it : 0.f;
  c->last_spmv_count = fin.it;
  c->last_solve_kernels = 4 + cycles * kernels_per_cycle;
  if (res_out) *res_out = fin.resid;
  if (res_rel_out) *res_rel_out = fin.beta0 > 0 ? fin.resid / fin.beta0 : 0.0;
  return fin.it;
}

}  // namespace gbfem
