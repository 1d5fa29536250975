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
// First the geometry of all the element's faces at once (one thread per face
// and point, in two passes: first side, whose Jacobian gives the normal, then
// the second side; the long FP64 chains with their divisions and square roots
// run side by side).  Then per face: monomial factors and per-(b, c) basis
// products; one fused pass over (row, point) pairs forming the FP64 operand
// values, each row's exponent (a shuffle max over its 16-lane segment) and
// the BF16 slices, with no FP64 staging; 56 MMAs (M 128, N = NS rounded up to
// 16, K 16) issued by one thread into 7 accumulators; commit to an mbarrier;
// epilogue by the warps whose TMEM lane quarter holds rows (tcgen05.ld: warp
// w reads lane quarter w % 4, column half w / 4).  Every wait has an
// iteration limit: on expiry the CTA records an error, lets its MMAs drain
// (again with a limit), frees its TMEM and returns.

#include "dg_face.cuh"
#include "gbfem_internal.h"
#include "tc_ptx.cuh"

namespace gbfem {

static __device__ const double tf_fq[GB_DG_PMAX][2][GB_DG_MAXNQF][3] = GB_DG_FQ_INIT;
static __device__ const unsigned char tf_exp[GB_DG_PMAX][GB_DG_MAXNS][3] = GB_DG_EXP_INIT;
static __device__ const int tf_ns[GB_DG_PMAX + 1] = GB_DG_NS_INIT;
static __device__ const int tf_nqf[GB_DG_PMAX + 1][2] = GB_DG_NQF_INIT;

constexpr int TF_SL = 7;          // slices per operand, 8 bits each (integers up to 255: exact in BF16)
constexpr int TF_KP = 32;         // K: 2 x (up to 16 face points)
constexpr int TF_NQ = 16;         // face points of the largest rule with max(p1, p2) <= 3
constexpr int TF_NF = 5;          // faces of a prism
constexpr int TF_M = 128;         // MMA M
constexpr int TF_THREADS = 256;
constexpr int TF_TMEM_COLS = 256;  // two CTAs per SM share the 512 columns
constexpr int TF_NCH = 32;         // MMA N per chunk of e's functions: 7 x 32 accumulator columns
// per-point table strides in doubles, odd so that the 16 lanes of a row
// segment (one per point) fall on different shared-memory banks
constexpr int TF_GEO = 17;   // 13 geometry values + 3 owner-row scales, padded
constexpr int TF_FAC = 30;   // monomial factors per point and side
constexpr int TF_FACS = 31;  // their stride
constexpr int TF_UWS = 33;   // 16 (b, c) x 2 basis products per point and side, padded
static_assert(TF_FACS > TF_FAC && TF_UWS > 32 && TF_GEO > 16, "padded strides hold their tables");
static_assert((long long)TF_SL * TF_KP * 255 * 255 < (1LL << 24), "slice sums must stay exact in FP32");
static_assert(TF_NF * (2 * TF_NQ + 1) <= TF_THREADS, "one thread per (face, point, side) and per face");

template <int P>
struct TfDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : 40;
  static constexpr int NPAD = (NS + 15) / 16 * 16;  // MMA N
  static constexpr int ROWS = NS + 40;              // own + neighbour (degree <= 3) functions
  static constexpr int ROWS8 = (ROWS + 7) / 8 * 8;
  // A slices packed ROWS8 rows apart: the M = 128 rows an MMA reads beyond a
  // slice's own rows belong to the next slice (or the tail) and only feed D
  // rows that are discarded
  static constexpr int A_STRIDE = ROWS8 * TF_KP * 2;
  static constexpr int A_BYTES = (TF_SL - 1) * A_STRIDE + TF_M * TF_KP * 2;
  static constexpr int B_SLICE = NPAD * TF_KP * 2;
  static constexpr int OFF_B = A_BYTES;
  static constexpr int OFF_UW = OFF_B + TF_SL * B_SLICE;
  static constexpr int OFF_FAC = OFF_UW + TF_NQ * 2 * TF_UWS * 8;          // [TF_NQ][2][TF_FACS]
  static constexpr int OFF_FACE = OFF_FAC + TF_NQ * 2 * TF_FACS * 8;
  // per face: X [2][18], A [2][9], G [TF_NQ][TF_GEO], EV [TF_NQ][2][6] (point, v), pen, spare
  static constexpr int FACE_DOUBLES = 36 + 18 + TF_NQ * TF_GEO + TF_NQ * 2 * 6 + 2;
  static constexpr int OFF_DIAG = OFF_FACE + TF_NF * FACE_DOUBLES * 8;     // [NS][SD_LD] diagonal-block share
  static constexpr int SD_LD = NS + 1;                                     // odd row stride
  static constexpr int OFF_RACC = OFF_DIAG + NS * SD_LD * 8;               // [NS] boundary rhs sums
  static constexpr int OFF_HF = OFF_RACC + 64 * 8;
  static constexpr int OFF_INT = (OFF_HF + TF_NF * (int)sizeof(DgHalfFace) + 15) / 16 * 16;  // ea, eb, bar, slot
  static constexpr int SMEM = OFF_INT + (128 + 64) * 4 + 64;
  static constexpr int NCHUNK = (NPAD + TF_NCH - 1) / TF_NCH;
  static_assert(TF_SL * (NPAD < TF_NCH ? NPAD : TF_NCH) <= TF_TMEM_COLS, "accumulators fit the TMEM allocation");
  static_assert(SMEM <= 113 * 1024, "shared memory of two CTAs per SM");
  static_assert(OFF_B % 1024 == 0 && OFF_HF % 16 == 0 && OFF_INT % 16 == 0, "alignment");
  static_assert(ROWS <= TF_M && NS <= 64, "rows");
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

// Face-vertex weights of a face rule point: barycentric on triangles,
// bilinear on quadrilaterals (as dg_face_point)
__device__ __forceinline__ void tf_weights(int nfv, const double *fq, double *w) {
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
}

__device__ __forceinline__ v3 tf_local_point(int nfv, const double *w, const unsigned char *loc) {
  v3 e = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (i >= nfv) break;
    e = v3_fma(w[i], prism_vertex_local(loc[i]), e);
  }
  return e;
}

// v = J^-1 A^T n from the Jacobian columns (the operations of dg_face_v)
__device__ __forceinline__ v3 tf_face_v(v3 j1, v3 j2, v3 j3, const double *A, v3 n) {
  const v3 c1 = v3_cross(j2, j3), c2 = v3_cross(j3, j1), c3 = v3_cross(j1, j2);
  const double rdet = 1.0 / v3_dot(j1, c1);
  const v3 an = {A[0] * n.x + A[3] * n.y + A[6] * n.z, A[1] * n.x + A[4] * n.y + A[7] * n.z,
                 A[2] * n.x + A[5] * n.y + A[8] * n.z};
  return {v3_dot(c1, an) * rdet, v3_dot(c2, an) * rdet, v3_dot(c3, an) * rdet};
}

// BF16 bit pattern of the integer c (|c| <= 255): through an FP32 add on the
// FMA pipe (exact), the sign set separately
__device__ __forceinline__ uint32_t tf_bf16_bits(uint32_t mag, bool neg) {
  const float fv = __uint_as_float(0x4B000000u | mag) - 8388608.0f;
  return (__float_as_uint(fv) >> 16) | (neg ? 0x8000u : 0u);
}

template <int P>
__global__ void __launch_bounds__(TF_THREADS, 2) dg_tc_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double pen, double gval,
    const long long *__restrict__ boff_diag, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs, int *err) {
  using Dm = TfDims<P>;
  constexpr int NS = Dm::NS, NPAD = Dm::NPAD, FD = Dm::FACE_DOUBLES;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *asl = smem, *bsl = smem + Dm::OFF_B;
  double *sUW = (double *)(smem + Dm::OFF_UW);       // [TF_NQ][2][TF_UWS]: per (b, c) basis products
  double *sFac = (double *)(smem + Dm::OFF_FAC);     // [TF_NQ][2][TF_FACS]: the current face's factors
  double *sface = (double *)(smem + Dm::OFF_FACE);   // [TF_NF][FD]
  double *sRacc = (double *)(smem + Dm::OFF_RACC);   // [NS]
  double *sD = (double *)(smem + Dm::OFF_DIAG);      // [NS][SD_LD]: row r (trial function), column i
  DgHalfFace *sHF = (DgHalfFace *)(smem + Dm::OFF_HF);
  int *ea = (int *)(smem + Dm::OFF_INT);             // A row exponents (by row = M row)
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
  if (tid < NS) sRacc[tid] = 0.0;
  for (int t = tid; t < NS * Dm::SD_LD; t += TF_THREADS) sD[t] = 0.0;
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
  // ---- geometry: phase 1, per (face, point), the first neighbour's side
  // (point, Jacobian, normal, area weight, v), and the penalty per face;
  // phase 2 the second neighbour's side and the owner-row scales ----
  if (tid < nf * TF_NQ) {
    const int f = tid / TF_NQ, q = tid % TF_NQ;
    const DgHalfFace &F = sHF[f];
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ti = F.nfv == 4 ? 1 : 0;
    const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
    if (pr <= 3 && q < tf_nqf[pr][ti]) {
      double *X = sface + f * FD, *G = X + 54 + q * TF_GEO, *EV = X + 54 + TF_NQ * TF_GEO + q * 12;
      const double *fq = tf_fq[pr - 1][ti][q];
      double w[4];
      tf_weights(F.nfv, fq, w);
      const v3 e1 = tf_local_point(F.nfv, w, F.loc1);
      v3 j1, j2, j3;
      prism_jacobian_columns(X, e1, j1, j2, j3);
      const v3 ds = prism_side_vector(F.side1, j1, j2, j3);
      const double d = sqrt(v3_dot(ds, ds));
      const v3 n = v3_scale(1.0 / d, ds);
      const v3 v1 = tf_face_v(j1, j2, j3, X + 36, n);
      G[12] = d * fq[2];
      G[13] = n.x;  // the normal, for phase 2 (then overwritten by the scales)
      G[14] = n.y;
      G[15] = n.z;
      EV[0] = e1.x; EV[1] = e1.y; EV[2] = e1.z;
      EV[3] = v1.x; EV[4] = v1.y; EV[5] = v1.z;
    }
  } else if (tid >= TF_NF * TF_NQ && tid < TF_NF * TF_NQ + nf) {
    const int f = tid - TF_NF * TF_NQ;
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
  if (tid < nf * TF_NQ) {
    const int f = tid / TF_NQ, q = tid % TF_NQ;
    const DgHalfFace &F = sHF[f];
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ti = F.nfv == 4 ? 1 : 0;
    const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
    if (pr <= 3 && q < tf_nqf[pr][ti]) {
      double *X = sface + f * FD, *G = X + 54 + q * TF_GEO, *EV = X + 54 + TF_NQ * TF_GEO + q * 12;
      if (interior) {
        double w[4];
        tf_weights(F.nfv, tf_fq[pr - 1][ti][q], w);
        const v3 e2 = tf_local_point(F.nfv, w, F.loc2);
        v3 j1, j2, j3;
        prism_jacobian_columns(X + 18, e2, j1, j2, j3);
        const v3 v2 = tf_face_v(j1, j2, j3, X + 45, v3{G[13], G[14], G[15]});
        EV[6] = e2.x; EV[7] = e2.y; EV[8] = e2.z;
        EV[9] = v2.x; EV[10] = v2.y; EV[11] = v2.z;
      }
      // owner-row scales: L = (f a) g + (s_o c a) phi, M = -(s_o f a) phi
      const double aw = G[12], so = F.owner_is_2 ? -1.0 : 1.0, fac = interior ? 0.5 : 1.0;
      G[13] = fac * aw;
      G[14] = so * X[FD - 2] * aw;
      G[15] = -so * fac * aw;
    }
  }
  // (the per-face loop starts with a barrier)

  // epilogue threads: warp w reads TMEM lane quarter w % 4 (rows = M rows =
  // A rows: e's functions 0..NS-1, then the neighbour's) and column half
  // w / 4 of the current chunk of e's functions
  const int lq = warp & 3, half = warp >> 2;
  const int r_ep = lq * 32 + (tid & 31);
  bool failed = false, bad_input = false;
  int fail_parity = 0, ncommit = 0;

  for (int f = 0; f < nf; f++) {
    const DgHalfFace &F = sHF[f];
    const double *sGeo = sface + f * FD + 54, *sEV = sGeo + TF_NQ * TF_GEO;
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
    // monomial factors of this face per (point, side)
    for (int t = tid; t < 2 * nq; t += TF_THREADS) {
      const int q = t >> 1, sd = t & 1;
      if (sd == 1 && !interior) continue;
      const double *ev = sEV + q * 12 + 6 * sd;
      dg_point_factors(v3{ev[0], ev[1], ev[2]}, v3{ev[3], ev[4], ev[5]}, sFac + (2 * q + sd) * TF_FACS);
    }
    __syncthreads();
    // per (point, side, b, c): U = eta^b zeta^c and W, the (eta, zeta) part of v . grad
    for (int t = tid; t < nq * 2 * 16; t += TF_THREADS) {
      const int q = t >> 5, sd = (t >> 4) & 1, bc = t & 15, b = bc >> 2, c = bc & 3;
      if (sd == 1 && !interior) continue;
      const double *T = sFac + (2 * q + sd) * TF_FACS;
      double *uw = sUW + (q * 2 + sd) * TF_UWS + bc * 2;
      uw[0] = T[5 + b] * T[10 + c];
      uw[1] = fma(T[5 + b], T[25 + c], T[20 + b] * T[10 + c]);
    }
    __syncthreads();
    // operands in one pass, a 16-lane segment per row r and a lane per point
    // q (k = 2q: Phi / L, 2q + 1: Gam / M; lanes q >= nq give the K
    // padding): FP64 values (phi = xi^a U, g = v_xi a xi^(a-1) U + xi^a W,
    // the operations of dg_basis_from_factors), the row exponent by a
    // segment max of the exponent fields, then the seven BF16 slices of the
    // pair as one 32-bit word each.  A rows: e's functions then the
    // neighbour's; B rows: e's functions.
    for (int base = 0; base < rows * 16; base += TF_THREADS) {
      const int t = base + tid, r = t >> 4, q = t & 15;
      const bool live = r < rows, own = r < NS;  // uniform over the segment
      double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
      if (live && q < nq) {
        const int side = own ? own_side : 3 - own_side, jj = own ? r : r - NS, p = own ? P : pnb;
        const unsigned char *ex = tf_exp[p - 1][jj];
        const double *T = sFac + (2 * q + side - 1) * TF_FACS;
        const double *uw = sUW + (q * 2 + side - 1) * TF_UWS + (ex[1] * 4 + ex[2]) * 2;
        const double phi = T[ex[0]] * uw[0];
        const double g = fma(T[15 + ex[0]], uw[0], T[ex[0]] * uw[1]);
        // Phi = s_t phi: the sign flip on the integer side
        a0 = __longlong_as_double(__double_as_longlong(phi) ^ (side == 2 ? (long long)1 << 63 : 0));
        a1 = g;
        if (own) {
          const double *G = sGeo + q * TF_GEO;
          b0 = fma(G[13], g, G[14] * phi);
          b1 = G[15] * phi;
        }
      }
      int xa = max(tf_biased_exp(a0), tf_biased_exp(a1)), xb = max(tf_biased_exp(b0), tf_biased_exp(b1));
#pragma unroll
      for (int o = 8; o >= 1; o >>= 1) {
        xa = max(xa, __shfl_xor_sync(0xffffffffu, xa, o));
        xb = max(xb, __shfl_xor_sync(0xffffffffu, xb, o));
      }
      if (!interior) {  // boundary face: the rhs of row r gets g sum_q L (uniform over the CTA)
        double sl = b0;
#pragma unroll
        for (int o = 8; o >= 1; o >>= 1) sl += __shfl_xor_sync(0xffffffffu, sl, o);
        if (live && own && q == 0) sRacc[r] = fma(gval, sl, sRacc[r]);
      }
      if (live) {
        const int EA = tf_row_exp(xa), EB = tf_row_exp(xb);
        if (q == 0) {
          ea[r] = EA;
          if (own) eb[r] = EB;
        }
        const int off = tc_off(r, 2 * q, TF_KP, 2);
        {
          const unsigned long long f0 = tf_fixed(a0, EA), f1 = tf_fixed(a1, EA);
          const uint32_t h0 = (uint32_t)(f0 >> 24), l0 = (uint32_t)f0 & 0xFFFFFFu;
          const uint32_t h1 = (uint32_t)(f1 >> 24), l1 = (uint32_t)f1 & 0xFFFFFFu;
          const bool n0 = __double_as_longlong(a0) < 0, n1 = __double_as_longlong(a1) < 0;
#pragma unroll
          for (int i = 0; i < TF_SL; i++) {
            const uint32_t c0 = i < 4 ? (h0 >> (24 - 8 * i)) & 255u : (l0 >> (16 - 8 * (i - 4))) & 255u;
            const uint32_t c1 = i < 4 ? (h1 >> (24 - 8 * i)) & 255u : (l1 >> (16 - 8 * (i - 4))) & 255u;
            *(uint32_t *)(asl + i * Dm::A_STRIDE + off) = tf_bf16_bits(c0, n0) | (tf_bf16_bits(c1, n1) << 16);
          }
        }
        if (own) {
          const unsigned long long f0 = tf_fixed(b0, EB), f1 = tf_fixed(b1, EB);
          const uint32_t h0 = (uint32_t)(f0 >> 24), l0 = (uint32_t)f0 & 0xFFFFFFu;
          const uint32_t h1 = (uint32_t)(f1 >> 24), l1 = (uint32_t)f1 & 0xFFFFFFu;
          const bool n0 = __double_as_longlong(b0) < 0, n1 = __double_as_longlong(b1) < 0;
#pragma unroll
          for (int i = 0; i < TF_SL; i++) {
            const uint32_t c0 = i < 4 ? (h0 >> (24 - 8 * i)) & 255u : (l0 >> (16 - 8 * (i - 4))) & 255u;
            const uint32_t c1 = i < 4 ? (h1 >> (24 - 8 * i)) & 255u : (l1 >> (16 - 8 * (i - 4))) & 255u;
            *(uint32_t *)(bsl + i * Dm::B_SLICE + off) = tf_bf16_bits(c0, n0) | (tf_bf16_bits(c1, n1) << 16);
          }
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // per chunk of e's functions (N = TF_NCH columns at most): MMAs, commit,
    // wait, epilogue; the accumulators are reused chunk after chunk
    for (int ch = 0; ch < Dm::NCHUNK; ch++) {
      const int clo = ch * TF_NCH, cn = NPAD - clo < TF_NCH ? NPAD - clo : TF_NCH;
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(cn >> 3) << 17) |
                               ((uint32_t)(TF_M >> 4) << 24);
        const uint32_t a0 = tc_smem(asl), b0 = tc_smem(bsl) + (clo / 8) * (TF_KP / 8) * 128;
        for (int i = 0; i < TF_SL; i++)
          for (int j = 0; j < TF_SL - i; j++) {
            const int d = i + j;
#pragma unroll
            for (int ks = 0; ks < TF_KP / 16; ks++) {
              const uint64_t ad = tc_desc(a0 + i * Dm::A_STRIDE + ks * 256, 128, (TF_KP / 8) * 128);
              const uint64_t bd = tc_desc(b0 + j * Dm::B_SLICE + ks * 256, 128, (TF_KP / 8) * 128);
              tc_mma<0>(tmem + d * cn, ad, bd, idesc, (i == 0 && ks == 0) ? 0u : 1u);
            }
          }
        tc_commit(tc_smem(bar));
      }
      __syncthreads();
      const bool waited = tc_wait(tc_smem(bar), ncommit & 1);
      if (__syncthreads_or(!waited)) {
        failed = true;
        fail_parity = ncommit & 1;
        break;
      }
      ncommit++;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // epilogue: D[r][i] = K[i][function r] (warps whose lane quarter holds
      // no row skip it as a whole)
      if (lq * 32 < rows) {
        const bool rok = r_ep < rows;
        const int sa = rok ? ea[r_ep] : 0;
        double *oblk = interior ? val + F.blk : nullptr;
        for (int grp = 0; grp < cn / 16; grp++) {
          const int cl = half * (cn / 2) + grp * 8;  // column within the chunk
          if (clo + cl >= NS) continue;              // padding columns only (uniform over the warp)
          float C[TF_SL][8];
#pragma unroll
          for (int d = 0; d < TF_SL; d++) tc_ld8(tmem + ((uint32_t)(lq * 32) << 16) + d * cn + cl, C[d]);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int c = 0; c < 8; c++) {
            const int i = clo + cl + c;
            if (!rok || i >= NS) continue;
            // sum_d C_d 2^(-8(d+2)) = (hi 2^24 + lo) 2^-64 with hi = C_0..C_3
            // and lo = C_4..C_6 in base 256 (|hi| < 2^48.01, |lo| <
            // 2^40.01); T = hi 2^14 + lo / 2^10 (< 2^63), so the sum is
            // T 2^-54, with 9 bits beyond the 53 the double rounds to
            long long hi = 0, lo = 0;
#pragma unroll
            for (int d = 0; d < 4; d++) hi = hi * 256 + (long long)__float2int_rn(C[d][c]);
#pragma unroll
            for (int d = 4; d < TF_SL; d++) lo = lo * 256 + (long long)__float2int_rn(C[d][c]);
            const double v = tf_i64_scaled(hi * 16384LL + (lo >> 10), sa + eb[i] - 54);
            if (r_ep < NS)
              sD[r_ep * Dm::SD_LD + i] += v;
            else
              oblk[i + (size_t)NS * (r_ep - NS)] = v;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();  // TMEM read before the next chunk's MMAs overwrite it
    }
    if (failed) break;
  }
  if (failed) tc_wait(tc_smem(bar), fail_parity);  // let the issued MMAs drain (bounded) before freeing TMEM
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TF_TMEM_COLS));
  if (failed || bad_input) {
    if (tid == 0) atomicExch(err, failed ? 6 : 7);
    return;
  }
  {
    // the diagonal block is column-major (entry (i, r) at i + NS r): sD's row r
    double *dblk = val + boff_diag[e];
    for (int t = tid; t < NS * NS; t += TF_THREADS) dblk[t] += sD[(t / NS) * Dm::SD_LD + t % NS];
  }
  if (tid < NS) rhs[roff[e] + tid] += sRacc[tid];
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
