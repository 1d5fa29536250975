// DG prism volume integrals on the tensor cores (tcgen05, sm_103a) with
// FP64-equivalent results: split BF16 products.
//
// The element matrix of apr_num_int_el (apd_dg_prism/aps_dg_prism_intf.c:
// 1239-1728) is a fixed linear map of per-point geometry:
//   K_uw = sum_q sum_ab D_q[a][u] G_q[a][b] D_q[b][w]
//        = sum_k E[(u,w)][k] g_e[k],   k = (q, ab), ab in {00,01,02,11,12,22}
// with E (upper entries x 6 nq) constant per degree and g_e = the 6 entries
// of G_q = (w_q / |det J|) C^T A C at every point (FP64, as the FP64 kernel
// forms them).  For a batch of elements this is one GEMM K = E g.
//
// Precision (Ozaki-style splitting): E (per row) and g_e (per element) are
// scaled by powers of two into [-1, 1) and cut into SL = 10 truncation slices
// of 6 bits, each an integer in [-63, 63] held exactly in BF16:
//   E = rs_r sum_i es_i 2^{-6(i+1)},  g = cs_e sum_j gs_j 2^{-6(j+1)}.
// The products of slices are exact in the FP32 tensor accumulator: every
// partial sum is an integer below 10 * 288 * 63^2 < 2^24.  Pairs with the same
// i + j = d share an accumulator C_d (d = 0..9; pairs with i + j > 9 are
// dropped), and
//   K = rs_r cs_e sum_d C_d 2^{-6(d+2)}
// is recombined exactly in int64 (two 49-bit partial sums) and rounded once to
// FP64.  Measured on the oracle's elements: within 6e-15 of the FP64 element
// matrices in the energy scale used by the parity tests.
//
// Kernel: one CTA per 32 elements, 256 threads.
//  A. FP64: geometry per (element, point) -> G (registers), per-element max
//     exponent, integer slicing of g into SL BF16 slices in shared memory
//     (the tcgen05 canonical K-major layout), and the load vector.
//  B. tcgen05: for each 128-row tile of E, its slices stream from global
//     memory (pre-arranged in the canonical layout) through a 3-stage
//     shared-memory ring by bulk-async copies (TMA engine) with mbarrier
//     transaction counts; one thread issues tcgen05.mma (M 128, N 32, K 16,
//     BF16 x BF16 -> FP32) into SL TMEM accumulators (SL x 32 columns).
//  C. epilogue per tile: tcgen05.ld of the SL accumulators, int64
//     recombination, FP64 scaling, both symmetric positions of the diagonal
//     block written.
// Every wait has an iteration limit; on expiry the CTA records an error,
// drains the copies and MMAs it issued (also with a limit), frees its TMEM
// and returns.
//
// Second mode (TF32, FP32 accumulation): the same GEMM with each scaled
// operand cut into a TF32 high part and a TF32 remainder (hi + lo carries
// about 22 bits), the three products hi hi + hi lo + lo hi accumulated in one
// FP32 TMEM accumulator per element (kind::tf32, K 8 per instruction, 64
// elements per CTA).  Accuracy is that of FP32 accumulation (about 1e-6 of
// the entry scale), not FP64: it stands beside the split-BF16 form as the
// cheaper, approximate contraction.

#include <cuda_bf16.h>

#include <cstring>
#include <mutex>

#include "dg_tables.h"
#include "gbfem_internal.h"
#include "tc_ptx.cuh"

namespace gbfem {

constexpr int TC_M = 128;       // MMA M (rows of E per tile)
constexpr int TC_THREADS = 256;
constexpr int TC_BITS = 6;      // bits per slice (split-BF16 mode)

// MODE 0: split BF16 (exact slice products); MODE 1: TF32 hi/lo
template <int MODE>
struct TcMode {
  static constexpr int ESZ = MODE == 0 ? 2 : 4;        // operand bytes
  static constexpr int SL = MODE == 0 ? 10 : 2;        // slices per operand
  static constexpr int NE = MODE == 0 ? 32 : 64;       // elements per CTA (MMA N)
  static constexpr int KC = MODE == 0 ? 48 : 24;       // K per streamed chunk (96 bytes of a row)
  static constexpr int KSTEP = MODE == 0 ? 16 : 8;     // K per instruction (32 bytes)
  static constexpr int NACC = MODE == 0 ? SL : 1;      // TMEM accumulators
  static constexpr int TMEM_COLS = MODE == 0 ? 512 : 64;  // >= NACC * NE, power of two
  static constexpr uint32_t FMT = MODE == 0 ? 1u : 2u;  // operand format: BF16 / TF32
  static constexpr int STAGES = MODE == 0 ? 3 : 4;     // E chunks in flight
};

template <int P, int MODE>
struct TcDims {
  using Md = TcMode<MODE>;
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  static constexpr int NQ = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 48 : 80;
  static constexpr int NSYM = NS * (NS + 1) / 2;
  static constexpr int KDIM = 6 * NQ;
  static constexpr int KPAD = (KDIM + Md::KC - 1) / Md::KC * Md::KC;
  static constexpr int NKC = KPAD / Md::KC;
  static constexpr int MT = (NSYM + TC_M - 1) / TC_M;
  static constexpr int GSL_BYTES = Md::SL * Md::NE * KPAD * Md::ESZ;  // g slices
  static constexpr int CHUNK_BYTES = TC_M * Md::KC * Md::ESZ;        // one E chunk
  static constexpr int RING_BYTES = Md::STAGES * CHUNK_BYTES;
  static constexpr int SMEM = GSL_BYTES + RING_BYTES + 512;          // + scales, barriers
  // exactness of the FP32 accumulation in the split-BF16 mode: at most SL
  // slice pairs per accumulator, products of integers below 2^6
  static_assert(MODE != 0 || (long long)Md::SL * KPAD * 63 * 63 < (1LL << 24),
                "slice sums must stay exact in FP32");
  static_assert(SMEM <= 227 * 1024, "shared memory");
};

// ------------------------------------------------------------------ kernel
template <int P, int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1) dg_tc_volume_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, const double *__restrict__ QPtab,
    const double *__restrict__ PHItab, const uint8_t *__restrict__ Etc, const int *__restrict__ rowexp,
    const int2 *__restrict__ uw, const long long *__restrict__ boff, const int *__restrict__ roff,
    double *__restrict__ val, double *__restrict__ rhs, int *err) {
  using Dm = TcDims<P, MODE>;
  using Md = TcMode<MODE>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, KPAD = Dm::KPAD, NKC = Dm::NKC, MT = Dm::MT;
  constexpr int SL = Md::SL, NE = Md::NE, KC = Md::KC, ESZ = Md::ESZ;
  constexpr int SLICE_BYTES = NE * KPAD * ESZ;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *gsl = smem;                             // [SL][NE x KPAD] slices, canonical layout
  uint8_t *ring = smem + Dm::GSL_BYTES;            // [STAGES][TC_M x KC] E chunks
  int *sexp = (int *)(ring + Dm::RING_BYTES);      // per-element exponent
  uint64_t *bars = (uint64_t *)(sexp + NE);        // full[3], empty[3], acc
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * Md::STAGES + 1);
  int *abort_flag = (int *)(tmem_slot + 1);
  // phase-A staging inside the ring (unused until phase B)
  double *sxa = (double *)ring;                    // [NE][27]: 18 coordinates, 9 tensor entries
  double *svol = sxa + NE * 27;                    // [NE][NQ]: w |det|
  static_assert(8 * (NE * 27 + NE * NQ) <= Dm::RING_BYTES, "phase-A staging fits the ring");
  const int tid = threadIdx.x, warp = tid >> 5;
  const int e0 = blockIdx.x * NE;
  const int nel_here = min(NE, count - e0);

  // ---------------- phase A: geometry, slices of g, load vector ----------------
  for (int t = tid; t < NE * 27; t += TC_THREADS) {
    const int el = t / 27, c = t % 27;
    double v = 0.0;
    if (el < nel_here) {
      const int e = ent_el[e0 + el];
      if (c < 18) {
        v = xyz[3 * (size_t)el_nodes[6 * (size_t)e + c / 3] + c % 3];
      } else {
        const int r = c - 18;
        v = D_el ? D_el[9 * (size_t)e + r] : ((r % 4 == 0) ? (k_el ? k_el[e] : 1.0) : 0.0);
      }
    }
    sxa[t] = v;
  }
  if (tid < NE) sexp[tid] = -1100;
  if (tid == 0) {
    for (int i = 0; i < 2 * Md::STAGES + 1; i++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(bars + i)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                 "r"(Md::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  constexpr int ITEMS = (NE * NQ + TC_THREADS - 1) / TC_THREADS;
  double g[ITEMS][6];
#pragma unroll
  for (int t = 0; t < ITEMS; t++) {
    const int it = tid + t * TC_THREADS;
    const int el = it / NQ, q = it % NQ;
#pragma unroll
    for (int c = 0; c < 6; c++) g[t][c] = 0.0;
    if (it < NE * NQ && el < nel_here) {
      const double *X = sxa + el * 27, *A = X + 18;
      const double xi = QPtab[4 * q], eta = QPtab[4 * q + 1], zeta = QPtab[4 * q + 2], w = QPtab[4 * q + 3];
      const double lo = (1.0 - zeta) / 2.0, hi = (1.0 + zeta) / 2.0, l0 = 1.0 - xi - eta;
      const double dx[6] = {-lo, lo, 0.0, -hi, hi, 0.0};
      const double dy[6] = {-lo, 0.0, lo, -hi, 0.0, hi};
      const double dz[6] = {-0.5 * l0, -0.5 * xi, -0.5 * eta, 0.5 * l0, 0.5 * xi, 0.5 * eta};
      double j1[3] = {0, 0, 0}, j2[3] = {0, 0, 0}, j3[3] = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < 6; i++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
          j1[d] = fma(dx[i], X[3 * i + d], j1[d]);
          j2[d] = fma(dy[i], X[3 * i + d], j2[d]);
          j3[d] = fma(dz[i], X[3 * i + d], j3[d]);
        }
      double cb[3][3];
      cb[0][0] = j2[1] * j3[2] - j2[2] * j3[1]; cb[0][1] = j2[2] * j3[0] - j2[0] * j3[2]; cb[0][2] = j2[0] * j3[1] - j2[1] * j3[0];
      cb[1][0] = j3[1] * j1[2] - j3[2] * j1[1]; cb[1][1] = j3[2] * j1[0] - j3[0] * j1[2]; cb[1][2] = j3[0] * j1[1] - j3[1] * j1[0];
      cb[2][0] = j1[1] * j2[2] - j1[2] * j2[1]; cb[2][1] = j1[2] * j2[0] - j1[0] * j2[2]; cb[2][2] = j1[0] * j2[1] - j1[1] * j2[0];
      const double adet = fabs(fma(j1[0], cb[0][0], fma(j1[1], cb[0][1], j1[2] * cb[0][2])));
      const double s = w / adet;
      double Ac[3][3];
#pragma unroll
      for (int b = 0; b < 3; b++)
#pragma unroll
        for (int r = 0; r < 3; r++) Ac[b][r] = fma(A[3 * r], cb[b][0], fma(A[3 * r + 1], cb[b][1], A[3 * r + 2] * cb[b][2]));
      // G_ab = s c_a . (A c_b), packed 00 01 02 11 12 22
      const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int c = 0; c < 6; c++) {
        const int a = pa[c], b = pb[c];
        g[t][c] = s * fma(cb[a][0], Ac[b][0], fma(cb[a][1], Ac[b][1], cb[a][2] * Ac[b][2]));
      }
      svol[el * NQ + q] = w * adet;
      int em = -1100;
#pragma unroll
      for (int c = 0; c < 6; c++)
        if (g[t][c] != 0.0) em = max(em, tc_exp_above(g[t][c]));
      atomicMax(sexp + el, em);
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < ITEMS; t++) {
    const int it = tid + t * TC_THREADS;
    if (it >= NE * NQ) continue;
    const int el = it / NQ, q = it % NQ;
    const int E = sexp[el];
#pragma unroll
    for (int c = 0; c < 6; c++) {
      const double v = g[t][c];
      const int k = 6 * q + c;
      if constexpr (MODE == 0) {
        // y = |g| 2^-E in [0, 1) as a 60-bit fixed-point integer, 6 bits per slice
        const long long bits = __double_as_longlong(v);
        const int ex = (int)((bits >> 52) & 0x7FF);
        // |v| = m 2^(ex - 1075) with m the 53-bit mantissa; fixed = |v| 2^(60 - E)
        unsigned long long fixed = 0;
        if (ex != 0) {
          const unsigned long long m = (bits & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
          const int sh = ex - 1075 + 60 - E;  // left shift of m
          if (sh >= 0)
            fixed = sh < 11 ? m << sh : 0ULL;  // |v| < 2^E keeps m << sh below 2^60
          else if (sh > -64)
            fixed = m >> (-sh);
        }
        const bool neg = bits < 0;
#pragma unroll
        for (int i = 0; i < SL; i++) {
          int chunk = (int)((fixed >> (60 - TC_BITS * (i + 1))) & 63ULL);
          if (neg) chunk = -chunk;
          *(__nv_bfloat16 *)(gsl + i * SLICE_BYTES + tc_off(el, k, KPAD, ESZ)) = __int2bfloat16_rn(chunk);
        }
      } else {
        // y = g 2^-E in (-1, 1): TF32 high part and TF32 remainder
        const double y = v * tc_pow2(E < -1000 ? 0 : -E);  // E = -1100: no nonzero entry
        const float hi = tc_tf32((float)y);
        const float lo = tc_tf32((float)(y - (double)hi));
        *(float *)(gsl + tc_off(el, k, KPAD, ESZ)) = hi;
        *(float *)(gsl + SLICE_BYTES + tc_off(el, k, KPAD, ESZ)) = lo;
      }
    }
  }
  // zero the padding of K (k >= 6 NQ) in every slice (byte-wise: 0 in both formats)
  if constexpr (Dm::KDIM < KPAD)
    for (int t = tid; t < SL * NE * (KPAD - Dm::KDIM); t += TC_THREADS) {
      const int i = t / (NE * (KPAD - Dm::KDIM)), r = t % (NE * (KPAD - Dm::KDIM));
      const int el = r / (KPAD - Dm::KDIM), k = Dm::KDIM + r % (KPAD - Dm::KDIM);
      uint8_t *dst = gsl + i * SLICE_BYTES + tc_off(el, k, KPAD, ESZ);
#pragma unroll
      for (int b = 0; b < ESZ; b++) dst[b] = 0;
    }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  // load vector R_u = f sum_q phi_u(q) w |det|
  for (int t = tid; t < nel_here * NS; t += TC_THREADS) {
    const int el = t / NS, u = t % NS;
    double r = 0.0;
    for (int q = 0; q < NQ; q++) r = fma(PHItab[(size_t)q * NS + u], svol[el * NQ + q], r);
    rhs[roff[ent_el[e0 + el]] + u] = f * r;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();  // the ring is free for the E chunks
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // ---------------- phases B and C, one 128-row tile of E at a time ----------------
  const uint32_t idesc = (1u << 4) | (Md::FMT << 7) | (Md::FMT << 10) | ((uint32_t)(NE >> 3) << 17) |
                         ((uint32_t)(TC_M >> 4) << 24);
  const uint32_t full0 = tc_smem(bars), empty0 = tc_smem(bars + Md::STAGES), accb = tc_smem(bars + 2 * Md::STAGES);
  const int T = MT * SL * NKC;  // chunks, in (tile, slice i, k chunk) order
  auto chunk_src = [&](int t) { return Etc + (size_t)t * Dm::CHUNK_BYTES; };
  int issued = 0, mma_done = 0;  // chunks copied / consumed (thread 0)
  if (tid == 0)
    for (; issued < Md::STAGES && issued < T; issued++)
      tc_bulk_load(tc_smem(ring + issued * Dm::CHUNK_BYTES), chunk_src(issued), Dm::CHUNK_BYTES,
                   full0 + 8 * issued);
  for (int m = 0; m < MT; m++) {
    if (tid == 0) {
      for (int i = 0; i < SL && !*abort_flag; i++) {
        for (int kc = 0; kc < NKC; kc++) {
          const int t = mma_done, s = t % Md::STAGES;
          if (!tc_wait(full0 + 8 * s, (t / Md::STAGES) & 1)) {
            *abort_flag = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t abase = tc_smem(ring + s * Dm::CHUNK_BYTES);
          for (int j = 0; j < SL - i; j++) {
            const int d = MODE == 0 ? i + j : 0;  // accumulator
            const uint32_t bbase = tc_smem(gsl + j * SLICE_BYTES);
#pragma unroll
            for (int ks = 0; ks < KC / Md::KSTEP; ks++) {
              const uint64_t ad = tc_desc(abase + ks * 256, 128, (KC * ESZ / 16) * 128);
              const uint64_t bd =
                  tc_desc(bbase + ((kc * KC + Md::KSTEP * ks) * ESZ / 16) * 128, 128, (KPAD * ESZ / 16) * 128);
              const bool first = i == 0 && kc == 0 && ks == 0 && (MODE == 0 || j == 0);
              tc_mma<MODE>(tmem + d * NE, ad, bd, idesc, first ? 0u : 1u);
            }
          }
          tc_commit(empty0 + 8 * s);
          mma_done++;
          // refill the stage of the previous chunk (its MMAs are queued ahead
          // of this chunk's, so the tensor pipe keeps working meanwhile)
          if (t >= 1 && issued < T) {
            const int tp = t - 1, sp = tp % Md::STAGES;
            if (!tc_wait(empty0 + 8 * sp, (tp / Md::STAGES) & 1)) {
              *abort_flag = 1;
              break;
            }
            tc_bulk_load(tc_smem(ring + sp * Dm::CHUNK_BYTES), chunk_src(issued), Dm::CHUNK_BYTES, full0 + 8 * sp);
            issued++;
          }
        }
      }
      tc_commit(accb);  // also when aborting: drains every MMA issued so far
    }
    __syncthreads();
    const bool waited = tc_wait(accb, m & 1);
    if (__syncthreads_or(!waited || *abort_flag)) {
      if (tid == 0) {
        atomicExch(err, 5);
        // let the copies still in flight land before the CTA leaves
        for (int t = mma_done; t < issued; t++) tc_wait(full0 + 8 * (t % Md::STAGES), (t / Md::STAGES) & 1);
      }
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: warp -> TMEM lane quarter (rows) and element half (columns)
    const int lq = warp & 3, half = warp >> 2;
    const int r = m * TC_M + lq * 32 + (tid & 31);
    const bool row_ok = r < Dm::NSYM;
    const int2 pw = row_ok ? uw[r] : make_int2(0, 0);
    const int rexp = row_ok ? rowexp[r] : 0;
#pragma unroll
    for (int grp = 0; grp < NE / 16; grp++) {
      const int c0 = half * (NE / 2) + grp * 8;
      float C[Md::NACC][8];
#pragma unroll
      for (int d = 0; d < Md::NACC; d++)
        tc_ld8(tmem + ((uint32_t)(lq * 32) << 16) + d * NE + c0, C[d]);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int el = c0 + c;
        if (!row_ok || el >= nel_here) continue;
        const int sc = rexp + sexp[el];  // row and element scale exponents
        double v;
        if constexpr (MODE == 0) {
          // sum_d C_d 2^(-6(d+2)) = hi 2^-36 + lo 2^-66 with hi = C_0..C_4 and
          // lo = C_5..C_9 in base 64 (each below 2^49: exact in int64 and FP64)
          long long hi = 0, lo = 0;
#pragma unroll
          for (int d = 0; d < SL / 2; d++) hi = hi * 64 + (long long)__float2int_rn(C[d][c]);
#pragma unroll
          for (int d = SL / 2; d < SL; d++) lo = lo * 64 + (long long)__float2int_rn(C[d][c]);
          v = fma((double)lo, tc_pow2(sc - 66), (double)hi * tc_pow2(sc - 36));
        } else {
          v = (double)C[0][c] * tc_pow2(sc);
        }
        double *blk = val + boff[ent_el[e0 + el]];
        blk[pw.y + NS * pw.x] = v;
        if (pw.x != pw.y) blk[pw.x + NS * pw.y] = v;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Md::TMEM_COLS));
}

// ------------------------------------------------------------------ host side
struct TcTables {
  uint8_t *E = nullptr;   // slices in chunk order (tile, slice, k chunk), canonical layout
  int *rowexp = nullptr;  // row scale exponent: |E[r][k]| < 2^rowexp[r]
  int2 *uw = nullptr;     // packed upper entry -> (u, w)
  double *QP = nullptr, *PHI = nullptr;
};
static TcTables g_tc[64][2][GB_DG_PMAX + 1];
static bool g_tc_ready[64][2][GB_DG_PMAX + 1];
static std::mutex g_tc_mu;

template <int P, int MODE>
static int tc_build_tables(TcTables &T) {
  using Dm = TcDims<P, MODE>;
  using Md = TcMode<MODE>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, KPAD = Dm::KPAD, NKC = Dm::NKC, MT = Dm::MT;
  constexpr int SL = Md::SL, KC = Md::KC, ESZ = Md::ESZ;
  // reference derivative table D[q][a][u] and values PHI[q][u] of the monomial basis
  std::vector<double> D((size_t)NQ * 3 * NS), PHI((size_t)NQ * NS), QP((size_t)NQ * 4);
  for (int q = 0; q < NQ; q++) {
    const double *e = GB_DG_QP[P - 1][q];
    for (int k = 0; k < 4; k++) QP[q * 4 + k] = e[k];
    double px[8], py[8], pz[8];
    px[0] = py[0] = pz[0] = 1.0;
    for (int i = 1; i <= P; i++) {
      px[i] = px[i - 1] * e[0];
      py[i] = py[i - 1] * e[1];
      pz[i] = pz[i - 1] * e[2];
    }
    for (int u = 0; u < NS; u++) {
      const int a = GB_DG_EXP[P - 1][u][0], b = GB_DG_EXP[P - 1][u][1], c = GB_DG_EXP[P - 1][u][2];
      PHI[(size_t)q * NS + u] = px[a] * py[b] * pz[c];
      D[((size_t)q * 3 + 0) * NS + u] = a ? a * px[a - 1] * py[b] * pz[c] : 0.0;
      D[((size_t)q * 3 + 1) * NS + u] = b ? b * px[a] * py[b - 1] * pz[c] : 0.0;
      D[((size_t)q * 3 + 2) * NS + u] = c ? c * px[a] * py[b] * pz[c - 1] : 0.0;
    }
  }
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
  std::vector<int2> uw(MT * TC_M, make_int2(0, 0));
  std::vector<int> rexp(MT * TC_M, 0);
  std::vector<uint8_t> E((size_t)MT * SL * NKC * Dm::CHUNK_BYTES, 0);
  std::vector<double> row(KPAD);
  int r = 0;
  for (int u = 0; u < NS; u++)
    for (int w = u; w < NS; w++, r++) {
      uw[r] = make_int2(u, w);
      double mx = 0.0;
      for (int k = 0; k < KPAD; k++) {
        double v = 0.0;
        if (k < Dm::KDIM) {
          const int q = k / 6, c = k % 6, a = pa[c], b = pb[c];
          const double *Dq = D.data() + (size_t)q * 3 * NS;
          v = a == b ? Dq[a * NS + u] * Dq[a * NS + w] : Dq[a * NS + u] * Dq[b * NS + w] + Dq[b * NS + u] * Dq[a * NS + w];
        }
        row[k] = v;
        mx = std::max(mx, std::fabs(v));
      }
      int ex = 0;
      if (mx > 0) {
        std::frexp(mx, &ex);  // mx < 2^ex
      }
      rexp[r] = ex;
      const int m = r / TC_M, rr = r % TC_M;
      for (int k = 0; k < KPAD; k++) {
        const int kc = k / KC, kk = k % KC;
        auto at = [&](int i) {
          const size_t chunk = ((size_t)m * SL + i) * NKC + kc;
          return E.data() + chunk * Dm::CHUNK_BYTES + tc_off(rr, kk, KC, ESZ);
        };
        if (MODE == 0) {
          double y = std::fabs(row[k]) * std::ldexp(1.0, -ex);  // [0, 1)
          const bool neg = row[k] < 0;
          for (int i = 0; i < SL; i++) {
            y *= 64.0;
            const double t = std::floor(y);
            y -= t;
            const __nv_bfloat16 h = __float2bfloat16((float)(neg ? -t : t));
            memcpy(at(i), &h, 2);
          }
        } else {
          const double y = row[k] * std::ldexp(1.0, -ex);  // (-1, 1)
          const float hi = tc_tf32((float)y), lo = tc_tf32((float)(y - (double)hi));
          memcpy(at(0), &hi, 4);
          memcpy(at(1), &lo, 4);
        }
      }
    }
  GB_CUDA(cudaMalloc(&T.E, E.size()));
  GB_CUDA(cudaMalloc(&T.rowexp, rexp.size() * sizeof(int)));
  GB_CUDA(cudaMalloc(&T.uw, uw.size() * sizeof(int2)));
  GB_CUDA(cudaMalloc(&T.QP, QP.size() * sizeof(double)));
  GB_CUDA(cudaMalloc(&T.PHI, PHI.size() * sizeof(double)));
  GB_CUDA(cudaMemcpy(T.E, E.data(), E.size(), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(T.rowexp, rexp.data(), rexp.size() * sizeof(int), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(T.uw, uw.data(), uw.size() * sizeof(int2), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(T.QP, QP.data(), QP.size() * sizeof(double), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(T.PHI, PHI.data(), PHI.size() * sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

bool dg_tc_supported(int p) { return p >= 1 && p <= 3; }

template <int P, int MODE>
static int tc_launch(cudaStream_t st, const TcTables &T, int count, const int *ent_el, const int *el_nodes,
                     const double *xyz, const double *k_el, const double *D_el, double f, const long long *boff,
                     const int *roff, double *val, double *rhs, int *err) {
  const int smem = TcDims<P, MODE>::SMEM;
  const int grid = (count + TcMode<MODE>::NE - 1) / TcMode<MODE>::NE;
  GB_CUDA(cudaFuncSetAttribute(dg_tc_volume_kernel<P, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  dg_tc_volume_kernel<P, MODE><<<grid, TC_THREADS, smem, st>>>(count, ent_el, el_nodes, xyz, k_el, D_el, f, T.QP,
                                                              T.PHI, T.E, T.rowexp, T.uw, boff, roff, val, rhs, err);
  GB_CUDA(cudaGetLastError());
  return 1;
}

// mode 0: split BF16 (FP64-equivalent); mode 1: TF32 hi/lo (FP32 accuracy)
int launch_dg_tc_volume(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                        const double *xyz, const double *k_el, const double *D_el, double f, const long long *boff,
                        const int *roff, double *val, double *rhs, int *err, int mode) {
  if (count <= 0) return 0;
  GB_CHECK(dg_tc_supported(p), "tensor-core DG volume kernel covers p = 1..3");
  GB_CHECK(device >= 0 && device < 64, "device index out of range");
  GB_CHECK(mode == 0 || mode == 1, "tensor-core mode must be 0 (split BF16) or 1 (TF32)");
  {
    std::lock_guard<std::mutex> lk(g_tc_mu);
    if (!g_tc_ready[device][mode][p]) {
      TcTables &T = g_tc[device][mode][p];
      int r;
      if (mode == 0)
        r = p == 1 ? tc_build_tables<1, 0>(T) : p == 2 ? tc_build_tables<2, 0>(T) : tc_build_tables<3, 0>(T);
      else
        r = p == 1 ? tc_build_tables<1, 1>(T) : p == 2 ? tc_build_tables<2, 1>(T) : tc_build_tables<3, 1>(T);
      if (r < 0) return r;
      g_tc_ready[device][mode][p] = true;
    }
  }
  const TcTables &T = g_tc[device][mode][p];
#define GB_TC_ARGS T, count, ent_el, el_nodes, xyz, k_el, D_el, f, boff, roff, val, rhs, err
  if (mode == 0) {
    switch (p) {
      case 1: return tc_launch<1, 0>(st, GB_TC_ARGS);
      case 2: return tc_launch<2, 0>(st, GB_TC_ARGS);
      default: return tc_launch<3, 0>(st, GB_TC_ARGS);
    }
  }
  switch (p) {
    case 1: return tc_launch<1, 1>(st, GB_TC_ARGS);
    case 2: return tc_launch<2, 1>(st, GB_TC_ARGS);
    default: return tc_launch<3, 1>(st, GB_TC_ARGS);
  }
#undef GB_TC_ARGS
}

}  // namespace gbfem
