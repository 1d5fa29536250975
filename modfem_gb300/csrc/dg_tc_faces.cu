// DG prism face integrals on the tensor cores (tcgen05, sm_103a) with
// FP64-equivalent results: split BF16 products, one CTA per owner element.
//
// Reference: pdr_conv_diff_comp_fa_stiff_mat_app of the DG weak form
// (pds_conv_diff_weakform_dg.c:232-1140); the face algebra and the owner-row
// form are those of the FP64 face kernel (dg_face.cuh, dg_faces.cu): for every
// face of element e, e's rows of the face matrix are
//   K[i][j] = sum_q L_i(q) Phi_j(q) + M_i(q) Gam_j(q),
// i over e's functions, j over e's and the neighbour's.  With the points as K
// (k = 2q: Phi / L, k = 2q + 1: Gam / M) this is one GEMM per face:
//   D (M = 128 rows: j, e's functions then the neighbour's) x (N: i) =
//   A (j x 2nq) . B (i x 2nq)^T,
// D[j][i] = K[i][j].  A and B are formed in FP64 in shared memory, each row
// scaled by a power of two into (-1, 1) and cut into SL = 7 truncation slices
// of 8 bits (integers in [-255, 255], exact in BF16).  Slice pairs with
// i + j = d share FP32 TMEM accumulator d (pairs with i + j > 6 dropped);
// every partial sum is an integer below 7 * 32 * 255^2 < 2^24, so the
// accumulation is exact, and
//   D = 2^(ea_j + eb_i) sum_d C_d 2^(-8(d+2))
// is recombined in int64 and rounded once to FP64 on the integer pipe.
// The owner's diagonal-block share is summed over its faces in FP64 registers
// and added once to the block the volume kernel wrote; the off-diagonal block
// (e, neighbour) is written whole, as in the FP64 kernel (deterministic, no
// atomics).  Covers owners of degree <= 3 whose neighbours all have degree
// <= 3 (2 nq <= 32); the others keep the FP64 face kernel.
//
// First the geometry and monomial factors of all the element's faces at
// once (one thread per face, point and side: the long FP64 chains with their
// divisions and square roots run side by side).  Then per face: FP64 basis
// values, row exponents, slicing (all threads); 56 MMAs (M 128, N = NS
// rounded up to 16, K 16) issued by one thread into 7 accumulators; commit to
// an mbarrier; epilogue by all warps (tcgen05.ld: warp w reads TMEM lane
// quarter w % 4 = rows, column half w / 4).  Every wait has an iteration
// limit: on expiry the CTA records an error, lets its MMAs drain (again with
// a limit), frees its TMEM and returns.

#include "dg_face.cuh"
#include "gbfem_internal.h"
#include "tc_ptx.cuh"

namespace gbfem {

static __device__ const double tf_fq[GB_DG_PMAX][2][GB_DG_MAXNQF][3] = GB_DG_FQ_INIT;
static __device__ const unsigned char tf_exp[GB_DG_PMAX][GB_DG_MAXNS][3] = GB_DG_EXP_INIT;
static __device__ const int tf_ns[GB_DG_PMAX + 1] = GB_DG_NS_INIT;
static __device__ const int tf_nqf[GB_DG_PMAX + 1][2] = GB_DG_NQF_INIT;

constexpr int TF_SL = 7;          // slices per operand
constexpr int TF_BITS = 8;        // bits per slice (integers up to 255: exact in BF16)
constexpr int TF_KP = 32;         // K: 2 x (up to 16 face points)
constexpr int TF_NQ = 16;         // face points of the largest rule with max(p1, p2) <= 3
constexpr int TF_NF = 5;          // faces of a prism
constexpr int TF_M = 128;         // MMA M
constexpr int TF_THREADS = 256;
constexpr int TF_TMEM_COLS = 512;
constexpr int TF_GEO = 16;
constexpr int TF_FAC = 30;
static_assert((long long)TF_SL * TF_KP * 255 * 255 < (1LL << 24), "slice sums must stay exact in FP32");
static_assert(TF_NF * (2 * TF_NQ + 1) <= TF_THREADS, "one thread per (face, point, side) and per face");

template <int P>
struct TfDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : 40;
  static constexpr int NPAD = (NS + 15) / 16 * 16;  // MMA N
  static constexpr int ROWS = NS + 40;              // own + neighbour (degree <= 3) functions
  static constexpr int A_SLICE = TF_M * TF_KP * 2;  // bytes per A slice
  static constexpr int B_SLICE = NPAD * TF_KP * 2;
  static constexpr int OFF_B = TF_SL * A_SLICE;
  static constexpr int OFF_A64 = OFF_B + TF_SL * B_SLICE;
  static constexpr int OFF_B64 = OFF_A64 + ROWS * TF_KP * 8;
  static constexpr int OFF_MISC = OFF_B64 + NS * TF_KP * 8;
  // per face: sX [2][18], sA [2][9], sGeo [TF_NQ][TF_GEO], sFac [TF_NQ][2][TF_FAC], pen, spare
  static constexpr int FACE_DOUBLES = 36 + 18 + TF_NQ * TF_GEO + 2 * TF_NQ * TF_FAC + 2;
  static constexpr int OFF_HF = OFF_MISC + TF_NF * FACE_DOUBLES * 8;
  static constexpr int OFF_INT = (OFF_HF + TF_NF * (int)sizeof(DgHalfFace) + 15) / 16 * 16;  // ea, eb, bar, slot
  static constexpr int SMEM = OFF_INT + (128 + 64) * 4 + 64;
  static_assert(TF_SL * NPAD <= TF_TMEM_COLS, "accumulators fit the TMEM allocation");
  static_assert(SMEM <= 227 * 1024, "shared memory");
  static_assert(OFF_HF % 16 == 0 && OFF_INT % 16 == 0, "alignment");
};

// biased FP64 exponent field of x (0 for zero / subnormal)
__device__ __forceinline__ int tf_biased_exp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// row exponent e with |x| < 2^e for every x of the row, from the largest
// biased exponent (integer pipe only); 0 for a zero row
__device__ __forceinline__ int tf_row_exp(int emax) { return emax > 0 ? emax - 1022 : 0; }

// |v| 2^-e (|v| < 2^e) as a 56-bit fixed-point integer
__device__ __forceinline__ unsigned long long tf_fixed(double v, int e) {
  const long long bits = __double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0) return 0ULL;
  const unsigned long long m = (bits & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const int sh = ex - 1075 + 56 - e;  // m 2^sh < 2^56, so sh <= 3
  if (sh >= 0) return sh < 4 ? m << sh : 0ULL;
  return sh > -64 ? m >> (-sh) : 0ULL;
}

// x 2^sc as a double, rounded to nearest (ties away), on the integer pipe:
// normalise by the leading-zero count and assemble sign, exponent and
// mantissa (GB300 issues FP64 at 1/64 of the FP32 rate; this keeps the
// epilogue off that pipe).  Assumes the result is a normal number.
__device__ __forceinline__ double tf_i64_scaled(long long x, int sc) {
  if (x == 0) return 0.0;
  const unsigned long long sgn = x < 0 ? (1ULL << 63) : 0ULL;
  const unsigned long long a = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << lz;  // leading one at bit 63
  const unsigned long long bits =
      (sgn | ((unsigned long long)(63 - lz + sc + 1023) << 52) | ((n >> 11) & 0xFFFFFFFFFFFFFULL)) + ((n >> 10) & 1ULL);
  return __longlong_as_double((long long)bits);
}

// One side of one face point (the split of dg_face_point by side, same
// operations): the point in that side's local coordinates and v = J^-1 A^T n;
// also the area weight.  The normal comes from the first neighbour in both
// cases.
__device__ __forceinline__ void tf_face_side(int nfv, const double *fq, const double *X1, const unsigned char *loc1,
                                             int side1, const double *A1, const double *X2,
                                             const unsigned char *loc2, const double *A2, int sd, v3 &e, v3 &v,
                                             double &a) {
  double w[4];
  if (nfv == 3) {
    w[0] = 1.0 - fq[0] - fq[1];
    w[1] = fq[0];
    w[2] = fq[1];
    w[3] = 0.0;
  } else {
    const double u = (fq[0] + 1.0) / 2.0, vv = (fq[1] + 1.0) / 2.0;
    w[0] = (1.0 - u) * (1.0 - vv);
    w[1] = u * (1.0 - vv);
    w[2] = u * vv;
    w[3] = (1.0 - u) * vv;
  }
  v3 e1 = {0, 0, 0}, e2 = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (i >= nfv) break;
    e1 = v3_fma(w[i], prism_vertex_local(loc1[i]), e1);
    if (sd) e2 = v3_fma(w[i], prism_vertex_local(loc2[i]), e2);
  }
  v3 j1, j2, j3;
  prism_jacobian_columns(X1, e1, j1, j2, j3);
  const v3 ds = prism_side_vector(side1, j1, j2, j3);
  const double d = sqrt(v3_dot(ds, ds));
  const v3 n = v3_scale(1.0 / d, ds);
  a = d * fq[2];
  e = sd ? e2 : e1;
  v = sd ? dg_face_v(X2, e2, A2, n) : dg_face_v(X1, e1, A1, n);
}

template <int P>
__global__ void __launch_bounds__(TF_THREADS, 1) dg_tc_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double pen, double gval,
    const long long *__restrict__ boff_diag, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs, int *err) {
  using Dm = TfDims<P>;
  constexpr int NS = Dm::NS, NPAD = Dm::NPAD, FD = Dm::FACE_DOUBLES;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *asl = smem, *bsl = smem + Dm::OFF_B;
  double *A64 = (double *)(smem + Dm::OFF_A64);      // [ROWS][TF_KP]
  double *B64 = (double *)(smem + Dm::OFF_B64);      // [NS][TF_KP]
  double *sface = (double *)(smem + Dm::OFF_MISC);   // [TF_NF][FD]
  DgHalfFace *sHF = (DgHalfFace *)(smem + Dm::OFF_HF);
  int *ea = (int *)(smem + Dm::OFF_INT);             // A row exponents
  int *eb = ea + 128;                                // B row exponents
  uint64_t *bar = (uint64_t *)(eb + 64);
  uint32_t *tmem_slot = (uint32_t *)(bar + 1);
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int h0 = hf_ptr[e], nf = hf_ptr[e + 1] - h0;
  if (nf <= 0) return;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (nf > TF_NF) {  // not a prism's face list (uniform over the CTA)
    if (tid == 0) atomicExch(err, 7);
    return;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < nf) sHF[tid] = hf[h0 + tid];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                 "r"(TF_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // ---- all faces at once: coordinates and tensors of both sides ----
  for (int t = tid; t < nf * 54; t += TF_THREADS) {
    const int f = t / 54, c = t % 54;
    const DgHalfFace &F = sHF[f];
    double *X = sface + f * FD;
    if (c < 36) {
      const int s = c / 18, r = c % 18;
      if (s == 0 || F.el2 >= 0) {
        const int el = s ? F.el2 : F.el1;
        X[c] = xyz[3 * (size_t)el_nodes[6 * (size_t)el + r / 3] + r % 3];
      }
    } else {
      const int tt = c - 36, s = tt / 9, r = tt % 9;
      if (s == 0 || F.el2 >= 0) {
        const int el = s ? F.el2 : F.el1;
        X[c] = D_el ? D_el[9 * (size_t)el + r] : ((r % 4 == 0) ? (k_el ? k_el[el] : 1.0) : 0.0);
      }
    }
  }
  __syncthreads();
  // ---- geometry and monomial factors per (face, point, side); penalty per face ----
  if (tid < nf * 2 * TF_NQ) {
    const int f = tid / (2 * TF_NQ), q = (tid >> 1) % TF_NQ, sd = tid & 1;
    const DgHalfFace &F = sHF[f];
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ti = F.nfv == 4 ? 1 : 0;
    const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
    if (pr <= 3 && q < tf_nqf[pr][ti] && (sd == 0 || interior)) {
      double *X = sface + f * FD;
      v3 ev, vv;
      double aw;
      tf_face_side(F.nfv, tf_fq[pr - 1][ti][q], X, F.loc1, F.side1, X + 36, interior ? X + 18 : nullptr, F.loc2,
                   X + 45, sd, ev, vv, aw);
      double *G = X + 54 + q * TF_GEO;
      if (sd == 0) G[12] = aw;
      dg_point_factors(ev, vv, X + 54 + TF_NQ * TF_GEO + (2 * q + sd) * TF_FAC);
    }
  } else if (tid >= 2 * TF_NF * TF_NQ && tid < 2 * TF_NF * TF_NQ + nf) {
    const int f = tid - 2 * TF_NF * TF_NQ;
    const DgHalfFace &F = sHF[f];
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const double *X = sface + f * FD;
    v3 V[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int l = i < F.nfv ? F.loc1[i] : 0;
      V[i] = {X[3 * l], X[3 * l + 1], X[3 * l + 2]};
    }
    const int pp = interior ? (p1 < p2 ? p1 : p2) : p1;
    sface[f * FD + FD - 2] = pen * pp / sqrt(dg_face_area(V, F.nfv));
  }
  __syncthreads();
  // owner-row scales per (face, point): L = (f a) g + (s_o c a) phi, M = -(s_o f a) phi
  if (tid < nf * TF_NQ) {
    const int f = tid / TF_NQ, q = tid % TF_NQ;
    const DgHalfFace &F = sHF[f];
    double *G = sface + f * FD + 54 + q * TF_GEO;
    const double aw = G[12], so = F.owner_is_2 ? -1.0 : 1.0, fac = F.el2 >= 0 ? 0.5 : 1.0;
    G[13] = fac * aw;
    G[14] = so * sface[f * FD + FD - 2] * aw;
    G[15] = -so * fac * aw;
  }
  // (the per-face loop starts with a barrier)

  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NPAD >> 3) << 17) |
                         ((uint32_t)(TF_M >> 4) << 24);
  // the diagonal-block share: thread (row r < NS, column half) holds columns
  // half * NPAD/2 + [0, NPAD/2)
  const int lq = warp & 3, half = warp >> 2;
  const int r_ep = lq * 32 + (tid & 31);
  double dacc[NPAD / 2];
#pragma unroll
  for (int c = 0; c < NPAD / 2; c++) dacc[c] = 0.0;
  double racc = 0.0;
  bool failed = false, bad_input = false;
  int fail_parity = 0;

  for (int f = 0; f < nf; f++) {
    const DgHalfFace &F = sHF[f];
    const double *sGeo = sface + f * FD + 54, *sFac = sGeo + TF_NQ * TF_GEO;
    const bool interior = F.el2 >= 0;
    const int own2 = F.owner_is_2;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ti = F.nfv == 4 ? 1 : 0;
    const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
    const int nq = tf_nqf[pr][ti];
    const int pnb = own2 ? p1 : p2;  // the other side's degree
    const int ns_nb = interior ? tf_ns[pnb] : 0;
    const int rows = NS + ns_nb;
    const int own_side = own2 ? 2 : 1;
    if (pr > 3 || rows > Dm::ROWS || nq > TF_NQ) {  // a degree-4 neighbour: not this kernel's (uniform)
      bad_input = true;
      break;
    }
    __syncthreads();  // the previous face's shared arrays are free; the scales are written
    // FP64 operands, one basis evaluation per (row, point): A rows = e's
    // functions then the neighbour's (k = 2q: Phi, 2q + 1: Gam), B rows =
    // e's functions (L, M); the K padding is zeroed when slicing
    for (int t = tid; t < rows * nq; t += TF_THREADS) {
      const int r = t / nq, q = t - r * nq;
      const bool own = r < NS;
      const int side = own ? own_side : 3 - own_side, jj = own ? r : r - NS, p = own ? P : pnb;
      const unsigned char *ex = tf_exp[p - 1][jj];
      double phi, g;
      dg_basis_from_factors(sFac + (2 * q + side - 1) * TF_FAC, ex[0], ex[1], ex[2], phi, g);
      // Phi = s_t phi: the sign flip on the integer side
      A64[r * TF_KP + 2 * q] = __longlong_as_double(__double_as_longlong(phi) ^ (side == 2 ? (long long)1 << 63 : 0));
      A64[r * TF_KP + 2 * q + 1] = g;
      if (own) {
        const double *G = sGeo + q * TF_GEO;
        B64[r * TF_KP + 2 * q] = fma(G[13], g, G[14] * phi);
        B64[r * TF_KP + 2 * q + 1] = G[15] * phi;
      }
    }
    __syncthreads();
    if (!interior && tid < NS) {
      double s = 0.0;
      for (int q = 0; q < nq; q++) s += B64[tid * TF_KP + 2 * q];
      racc = fma(gval, s, racc);
    }
    // row exponents (integer max of the exponent fields): threads
    // 0..rows-1 for A, 128..128+NS-1 for B
    if (tid < rows || (tid >= 128 && tid < 128 + NS)) {
      const double *row = tid < 128 ? A64 + tid * TF_KP : B64 + (tid - 128) * TF_KP;
      int emax = 0;
      for (int k = 0; k < 2 * nq; k++) emax = max(emax, tf_biased_exp(row[k]));
      if (tid < 128)
        ea[tid] = tf_row_exp(emax);
      else
        eb[tid - 128] = tf_row_exp(emax);
    }
    __syncthreads();
    // slices: one thread per (row, 8 consecutive k), one 16-byte store per
    // slice (a core-matrix row of the canonical K-major layout); rows of A
    // beyond `rows` and of B beyond NS are never written: their D rows and
    // columns are discarded
    for (int t = tid; t < (rows + NS) * (TF_KP / 8); t += TF_THREADS) {
      const int r = t / (TF_KP / 8), k0 = (t % (TF_KP / 8)) * 8;
      const bool isa = r < rows;
      const int rr = isa ? r : r - rows;
      const double *src = isa ? A64 + rr * TF_KP : B64 + rr * TF_KP;
      const int ex = isa ? ea[rr] : eb[rr];
      unsigned long long fx[8];
      bool neg[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const double v = k0 + u < 2 * nq ? src[k0 + u] : 0.0;
        fx[u] = tf_fixed(v, ex);
        neg[u] = __double_as_longlong(v) < 0;
      }
      uint8_t *dst = (isa ? asl : bsl) + tc_off(rr, k0, TF_KP, 2);
      const int stride = isa ? Dm::A_SLICE : Dm::B_SLICE;
#pragma unroll
      for (int i = 0; i < TF_SL; i++) {
        uint32_t w[4];
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
          int c0 = (int)((fx[u] >> (56 - TF_BITS * (i + 1))) & 255ULL);
          int c1 = (int)((fx[u + 1] >> (56 - TF_BITS * (i + 1))) & 255ULL);
          if (neg[u]) c0 = -c0;
          if (neg[u + 1]) c1 = -c1;
          w[u / 2] = (uint32_t)__bfloat16_as_ushort(__int2bfloat16_rn(c0)) |
                     ((uint32_t)__bfloat16_as_ushort(__int2bfloat16_rn(c1)) << 16);
        }
        *(uint4 *)(dst + i * stride) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = tc_smem(asl), b0 = tc_smem(bsl);
      for (int i = 0; i < TF_SL; i++)
        for (int j = 0; j < TF_SL - i; j++) {
          const int d = i + j;
#pragma unroll
          for (int ks = 0; ks < TF_KP / 16; ks++) {
            const uint64_t ad = tc_desc(a0 + i * Dm::A_SLICE + ks * 256, 128, (TF_KP / 8) * 128);
            const uint64_t bd = tc_desc(b0 + j * Dm::B_SLICE + ks * 256, 128, (TF_KP / 8) * 128);
            tc_mma<0>(tmem + d * NPAD, ad, bd, idesc, (i == 0 && ks == 0) ? 0u : 1u);
          }
        }
      tc_commit(tc_smem(bar));
    }
    __syncthreads();
    const bool waited = tc_wait(tc_smem(bar), f & 1);
    if (__syncthreads_or(!waited)) {
      failed = true;
      fail_parity = f & 1;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: D[r][i] = K[i][r]
    const bool rok = r_ep < rows;
    const int sa = rok ? ea[r_ep] : 0;
    double *oblk = interior ? val + F.blk : nullptr;
#pragma unroll
    for (int grp = 0; grp < NPAD / 16; grp++) {
      const int c0 = half * (NPAD / 2) + grp * 8;
      float C[TF_SL][8];
#pragma unroll
      for (int d = 0; d < TF_SL; d++) tc_ld8(tmem + ((uint32_t)(lq * 32) << 16) + d * NPAD + c0, C[d]);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int i = c0 + c;
        if (!rok || i >= NS) continue;
        // sum_d C_d 2^(-8(d+2)) = (hi 2^24 + lo) 2^-64 with hi = C_0..C_3 and
        // lo = C_4..C_6 in base 256 (|hi| < 2^48.01, |lo| < 2^40.01);
        // T = hi 2^14 + lo / 2^10 (< 2^63), so the sum is T 2^-54, with 9
        // bits beyond the 53 the double rounds to
        long long hi = 0, lo = 0;
#pragma unroll
        for (int d = 0; d < 4; d++) hi = hi * 256 + (long long)__float2int_rn(C[d][c]);
#pragma unroll
        for (int d = 4; d < TF_SL; d++) lo = lo * 256 + (long long)__float2int_rn(C[d][c]);
        const double v = tf_i64_scaled(hi * 16384LL + (lo >> 10), sa + eb[i] - 54);
        if (r_ep < NS)
          dacc[grp * 8 + c] += v;
        else
          oblk[i + (size_t)NS * (r_ep - NS)] = v;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  if (failed) tc_wait(tc_smem(bar), fail_parity);  // let the issued MMAs drain (bounded) before freeing TMEM
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TF_TMEM_COLS));
  if (failed || bad_input) {
    if (tid == 0) atomicExch(err, failed ? 6 : 7);
    return;
  }
  if (r_ep < NS) {
    double *dblk = val + boff_diag[e];
#pragma unroll
    for (int c = 0; c < NPAD / 2; c++) {
      const int i = half * (NPAD / 2) + c;
      if (i < NS) dblk[i + (size_t)NS * r_ep] += dacc[c];
    }
  }
  if (tid < NS) rhs[roff[e] + tid] += racc;
}

bool dg_tc_faces_supported(int p) { return p >= 1 && p <= 3; }

int launch_dg_tc_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                       const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                       const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                       const int *roff, double *val, double *rhs, int *err) {
  if (count <= 0) return 0;
  GB_CHECK(dg_tc_faces_supported(p), "tensor-core DG face kernel covers p = 1..3");
#define GB_TF_LAUNCH(PP)                                                                                      \
  {                                                                                                           \
    const int smem = TfDims<PP>::SMEM;                                                                        \
    GB_CUDA(cudaFuncSetAttribute(dg_tc_faces_kernel<PP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
    dg_tc_faces_kernel<PP><<<count, TF_THREADS, smem, st>>>(count, ent_el, hf_ptr, hf, el_p, el_nodes, xyz,   \
                                                            k_el, D_el, pen, g, boff_diag, roff, val, rhs, err); \
  }
  switch (p) {
    case 1: GB_TF_LAUNCH(1); break;
    case 2: GB_TF_LAUNCH(2); break;
    default: GB_TF_LAUNCH(3); break;
  }
#undef GB_TF_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
