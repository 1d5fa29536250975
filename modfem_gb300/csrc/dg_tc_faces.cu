// DG prism face integrals on the tensor cores (tcgen05, sm_103a) with
// FP64-equivalent results: split BF16 products in a persistent, warp-
// specialised kernel (one CTA per SM).
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
// The owner's diagonal-block share is summed over its faces in shared memory
// and added once to the block the volume kernel wrote; the off-diagonal block
// (e, neighbour) is written whole, as in the FP64 kernel (deterministic, no
// atomics).  Covers owners of degree <= 3 whose neighbours all have degree
// <= 3 (2 nq <= 32); the others keep the FP64 face kernel.
//
// Two things the face matrices need do not depend on the owner, and are
// built outside this kernel so that no CTA repeats them:
//  * the per-point geometry of every face (area weight, penalty, and for both
//    sides v = J^-1 A^T n), once per face by dg_face_geometry_kernel, where
//    an owner-computes kernel would form it once per owner;
//  * the reference basis and its three local derivatives at the face points,
//    which depend only on the face's rule, the basis degree and how the face's
//    vertices sit in the element (its "configuration": vertex count and local
//    vertex order, at most 6 per triangle side and 8 per quadrilateral side),
//    so they are tables (dg_face_table_kernel, built once per structure,
//    about 2 MB, L2-resident), where the kernel otherwise evaluated monomial
//    factors per face, point and side.
// Per face one fused pass over (row, point) pairs forms the FP64 operand
// values (phi from the table, g = v . grad phi: three FMAs), each row's
// exponent (a shuffle max over its 16-lane segment) and the BF16 slices, with
// no FP64 staging; 56 MMAs (M 128, N = NS rounded up to 16, K 16) issued by
// one thread into 7 accumulators; an epilogue by the warps whose TMEM lane
// quarter holds rows (tcgen05.ld: warp w reads lane quarter w % 4).  Measured
// on GB300, a tcgen05.mma of these small shapes costs a fixed issue time (the
// same for N = 16 and 32, and for M = 64 and 128), so the kernel keeps the
// MMA count low (one N chunk per face, which needs the whole TMEM) and
// overlaps the three phases of consecutive faces by warp role (below).
// Every wait has an iteration limit: on expiry the CTA records an error, lets
// its MMAs drain (again with a limit), frees its TMEM and returns.

#include <type_traits>

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
constexpr int TF_GEO = 8;    // per face point: f a, c a, v1 (3), v2 (3)
constexpr int TF_GEOS = 9;   // their stride in shared memory: odd, so the 16 points of a row segment hit distinct banks
static_assert((long long)TF_SL * TF_KP * 255 * 255 < (1LL << 24), "slice sums must stay exact in FP32");

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
  static constexpr int FACE_DOUBLES = TF_NQ * TF_GEOS;
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

// An FP32 accumulator value that is an exact integer of magnitude below
// 2^22, as an int32: adding 1.5 * 2^23 puts the integer in the low mantissa
// bits (the ulp there is 1, so the add is exact); FP32 add and integer
// subtract instead of a conversion instruction
__device__ __forceinline__ int tf_exact_int(float c) { return __float_as_int(c + 12582912.0f) - 0x4B400000; }

// Two signed 8-bit slice values as a packed BF16 pair (first in the low
// half): each as the exact FP32 s c (s = +-1) through one FMA on 2^23 + c,
// then one conversion packs both (exact: |c| <= 255).  A zero slice packs as
// +0 whatever its sign; the products it enters are zero either way.
__device__ __forceinline__ uint32_t tf_bf16x2(uint32_t c0, float s0, uint32_t c1, float s1) {
  const float f0 = fmaf(__uint_as_float(0x4B000000u | c0), s0, -8388608.0f * s0);
  const float f1 = fmaf(__uint_as_float(0x4B000000u | c1), s1, -8388608.0f * s1);
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(f1), "f"(f0));
  return r;
}

// The reference basis at the face points of every configuration: one block
// per (configuration, rule degree pr, basis degree pb), a thread per (point,
// function): value and the xi / eta / zeta derivatives, from the monomial
// factors of dg_point_factors (so the values are those of the FP64 kernel).
__global__ void dg_face_table_kernel(const unsigned char *__restrict__ cfg, const long long *__restrict__ tab_off,
                                     double *__restrict__ tab) {
  const int c = blockIdx.x / 9, pr = (blockIdx.x / 3) % 3 + 1, pb = blockIdx.x % 3 + 1;
  const int nfv = cfg[5 * c], ti = nfv == 4 ? 1 : 0;
  const int nq = tf_nqf[pr][ti], ns = tf_ns[pb];
  double *out = tab + tab_off[blockIdx.x];
  for (int t = threadIdx.x; t < nq * ns; t += blockDim.x) {
    const int q = t / ns, j = t % ns;
    double w[4];
    tf_weights(nfv, tf_fq[pr - 1][ti][q], w);
    const v3 e = tf_local_point(nfv, w, cfg + 5 * c + 1);
    double T[30];
    dg_point_factors(e, v3{1.0, 1.0, 1.0}, T);
    const unsigned char *ex = tf_exp[pb - 1][j];
    const int a = ex[0], b = ex[1], cc = ex[2];
    const double u = T[5 + b] * T[10 + cc];
    double *o = out + 4 * (size_t)t;
    o[0] = T[a] * u;
    o[1] = T[15 + a] * u;
    o[2] = T[a] * (T[20 + b] * T[10 + cc]);
    o[3] = T[a] * (T[5 + b] * T[25 + cc]);
  }
}

// Per-point geometry of a face, from its first neighbour's half-face record:
// the point in each side's local coordinates, the first side's Jacobian
// (normal, area weight), both sides' v = J^-1 A^T n; the penalty
// pen min(p1, p2) / sqrt(area) (p1 on the boundary) with mmr_fa_area's split
// of a quadrilateral.  One thread per (face, point); the same operations as
// the FP64 face kernel's dg_face_point.
__global__ void __launch_bounds__(128) dg_face_geometry_kernel(
    int count, const int *__restrict__ faces_hf, const DgHalfFace *__restrict__ hf, const int *__restrict__ el_p,
    const int *__restrict__ el_nodes, const double *__restrict__ xyz, const double *__restrict__ k_el,
    const double *__restrict__ D_el, double pen, double *__restrict__ geo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t / TF_NQ), q = (int)(t % TF_NQ);
  if (i >= count) return;
  const DgHalfFace F = hf[faces_hf[i]];
  const bool interior = F.el2 >= 0;
  const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
  const int ti = F.nfv == 4 ? 1 : 0;
  const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
  double *G = geo + ((size_t)F.face * TF_NQ + q) * TF_GEO;
  if (pr > 3 || q >= tf_nqf[pr][ti]) return;
  double X1[18], X2[18], A1[9], A2[9];
  for (int r = 0; r < 18; r++) X1[r] = xyz[3 * (size_t)el_nodes[6 * (size_t)F.el1 + r / 3] + r % 3];
  for (int r = 0; r < 9; r++)
    A1[r] = D_el ? D_el[9 * (size_t)F.el1 + r] : ((r % 4 == 0) ? (k_el ? k_el[F.el1] : 1.0) : 0.0);
  const double *fq = tf_fq[pr - 1][ti][q];
  double w[4];
  tf_weights(F.nfv, fq, w);
  const v3 e1 = tf_local_point(F.nfv, w, F.loc1);
  v3 j1, j2, j3;
  prism_jacobian_columns(X1, e1, j1, j2, j3);
  const v3 ds = prism_side_vector(F.side1, j1, j2, j3);
  const double d = sqrt(v3_dot(ds, ds));
  const v3 n = v3_scale(1.0 / d, ds);
  const v3 v1 = tf_face_v(j1, j2, j3, A1, n);
  v3 v2 = {0.0, 0.0, 0.0};
  if (interior) {
    for (int r = 0; r < 18; r++) X2[r] = xyz[3 * (size_t)el_nodes[6 * (size_t)F.el2 + r / 3] + r % 3];
    for (int r = 0; r < 9; r++)
      A2[r] = D_el ? D_el[9 * (size_t)F.el2 + r] : ((r % 4 == 0) ? (k_el ? k_el[F.el2] : 1.0) : 0.0);
    const v3 e2 = tf_local_point(F.nfv, w, F.loc2);
    prism_jacobian_columns(X2, e2, j1, j2, j3);
    v2 = tf_face_v(j1, j2, j3, A2, n);
  }
  v3 V[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int l = k < F.nfv ? F.loc1[k] : 0;
    V[k] = {X1[3 * l], X1[3 * l + 1], X1[3 * l + 2]};
  }
  const int pp = interior ? (p1 < p2 ? p1 : p2) : p1;
  const double cpen = pen * pp / sqrt(dg_face_area(V, F.nfv));
  const double aw = d * fq[2];
  G[0] = (interior ? 0.5 : 1.0) * aw;
  G[1] = cpen * aw;
  G[2] = v1.x;
  G[3] = v1.y;
  G[4] = v1.z;
  G[5] = v2.x;
  G[6] = v2.y;
  G[7] = v2.z;
}

// ---------------------------------------------------------------------------
// Pipelined form: one persistent CTA per SM with 512 threads and all 512
// TMEM columns, the phases of consecutive faces overlapped by warp role:
//   warps 0-7 (producers): per face, the operand pass into one of two
//       shared-memory buffers, up to two faces ahead of the epilogue and
//       across owner boundaries; each owner's boundary rhs share;
//   warp 8, one thread: the face's MMAs in one N chunk (N = NPAD <= 48, the
//       seven accumulators 7 NPAD <= 336 columns: 56 MMAs a face at p = 3
//       instead of 112 in two chunks), commit;
//   warps 8-15 (epilogue): accumulators to FP64, the owner rows into the
//       diagonal-block share, the neighbour rows to the off-diagonal block;
//       each owner's diagonal-block share when its last face is done.
// Hand-offs are mbarriers: full[b] (operands of buffer b written), mma[b]
// (its MMAs complete), free[b] (the epilogue is done with buffer b).  One
// elected thread per group waits (bounded, and it gives up early once any
// role has given up) and the group then meets at its named barrier and reads
// the outcome, so every decision is uniform over the group.  The
// arithmetic is that of dg_tc_faces_kernel: bit-identical results.
constexpr int TP_THREADS = 512;
// MMA issuers: lane 0 of warps 8 .. 8 + TP_ISSUERS - 1, each owning whole
// accumulators (d = 6 | 5, 0 | 4, 1 | 3, 2: seven slice pairs, 14 MMAs
// each), so that their issue runs side by side; all commit to mma[b]
constexpr int TP_ISSUERS = 4;
__host__ __device__ constexpr int tp_acc(int k, int m) {  // issuer k's m-th accumulator (-1: none)
  return k == 0 ? (m == 0 ? 6 : -1) : m == 0 ? 6 - k : k - 1;
}

struct TpMeta {
  long long blk;  // block (owner, neighbour); -1 on the boundary
  int rows, pad0, pad1, pad2;
};

template <int P>
struct TpDims {
  using D = TfDims<P>;
  static constexpr int B_BYTES = TF_SL * D::B_SLICE;
  static constexpr int BUF = D::A_BYTES + B_BYTES;  // one operand buffer
  static constexpr int OFF_FACE = 2 * BUF;           // [TF_NF][TF_NQ][TF_GEOS]
  static constexpr int SD_LD = D::NS + 1;
  static constexpr int OFF_DIAG = OFF_FACE + TF_NF * D::FACE_DOUBLES * 8;  // [NS][SD_LD]
  static constexpr int OFF_RACC = OFF_DIAG + D::NS * SD_LD * 8;            // [64]
  static constexpr int OFF_HF = OFF_RACC + 64 * 8;                          // [TF_NF]
  static constexpr int OFF_META = (OFF_HF + TF_NF * (int)sizeof(DgHalfFace) + 15) / 16 * 16;  // [2]
  static constexpr int OFF_EXP = OFF_META + 2 * (int)sizeof(TpMeta);       // [2][128 + 64]
  static constexpr int OFF_BAR = OFF_EXP + 2 * 192 * 4;  // full[2], mma[2], free[2], drain[TP_ISSUERS]
  static constexpr int SMEM_USED = OFF_BAR + 10 * 8 + 32;
  // requested at least 116 KB so that no two CTAs share an SM (each
  // allocates all 512 TMEM columns)
  static constexpr int SMEM = SMEM_USED > 116 * 1024 ? SMEM_USED : 116 * 1024;
  static_assert(BUF % 1024 == 0 && D::A_BYTES % 1024 == 0, "operand buffers 1024-aligned");
  static_assert(TF_SL * D::NPAD <= 512, "one chunk of accumulators fits the TMEM");
  static_assert(SMEM <= 227 * 1024, "shared memory of one CTA");
  static_assert(OFF_BAR % 8 == 0, "mbarrier alignment");
};

// named barrier of one role group (256 threads); the non-aligned form, as
// a group's elected thread may arrive on its own
__device__ __forceinline__ void tp_bar(int id) {
  asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(256) : "memory");
}

__device__ __forceinline__ void tp_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem(bar)) : "memory");
}

// Bounded wait of one thread; gives up early once another role has given up.
__device__ __forceinline__ bool tp_wait1(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  for (long long it = 0; it < TC_WAIT_LIMIT; it++) {
    if (tc_try_wait(tc_smem(bar), parity)) return true;
    if ((it & 255) == 255 && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

// Group wait (256 threads, named barrier id): the elected thread waits, the
// group reads the outcome after the barrier (slot alternates between
// consecutive waits, so a slot is rewritten only after another barrier).
__device__ __forceinline__ bool tp_group_wait(uint64_t *bar, uint32_t parity, bool elected, int id,
                                              volatile int *abort_flag, volatile int *slot) {
  if (elected) *slot = tp_wait1(bar, parity, abort_flag) ? 1 : 0;
  tp_bar(id);
  return *slot != 0;
}

template <int P>
__global__ void __launch_bounds__(TP_THREADS, 1) dg_tc_faces_pipe_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const double *__restrict__ geo, const double *__restrict__ ftab,
    const long long *__restrict__ ftab_off, double gval, const long long *__restrict__ boff_diag,
    const int *__restrict__ roff, double *__restrict__ val, double *__restrict__ rhs, int *err,
    double *__restrict__ share) {
  using Dm = TfDims<P>;
  using Tp = TpDims<P>;
  constexpr int NS = Dm::NS, NPAD = Dm::NPAD, FD = Dm::FACE_DOUBLES, SD_LD = Tp::SD_LD;
  extern __shared__ __align__(1024) uint8_t smem[];
  double *sface = (double *)(smem + Tp::OFF_FACE);
  double *sD = (double *)(smem + Tp::OFF_DIAG);   // row r (trial function), column i
  double *sRacc = (double *)(smem + Tp::OFF_RACC);
  DgHalfFace *sHF = (DgHalfFace *)(smem + Tp::OFF_HF);
  TpMeta *meta = (TpMeta *)(smem + Tp::OFF_META);
  int *sexp = (int *)(smem + Tp::OFF_EXP);        // buffer b: ea at 192 b, eb at 192 b + 128
  uint64_t *bar_full = (uint64_t *)(smem + Tp::OFF_BAR), *bar_mma = bar_full + 2, *bar_free = bar_full + 4;
  uint64_t *bar_drain = bar_full + 6;
  uint32_t *tmem_slot = (uint32_t *)(bar_full + 6 + TP_ISSUERS);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  volatile int *slots = (volatile int *)(tmem_slot + 2);  // [2] producers, [2] epilogue
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    for (int i = 0; i < 6 + TP_ISSUERS; i++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(bar_full + i)),
                   "r"(i == 2 || i == 3 ? TP_ISSUERS : 1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = 0;
  }
  for (int t = tid; t < NS * SD_LD; t += TP_THREADS) sD[t] = 0.0;
  if (tid < 64) sRacc[tid] = 0.0;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  bool issued_any = false;  // this thread issued MMAs (an issuer)

  if (warp < 8) {
    // ------------------------------ producers ------------------------------
    const int ptid = tid;
    int fi = 0;
    bool stop = false;
    for (int o = blockIdx.x; o < count && !stop; o += gridDim.x) {
      const int e = ent_el[o];
      const int h0 = hf_ptr[e], nf = hf_ptr[e + 1] - h0;
      if (nf <= 0) continue;
      if (nf > TF_NF) {  // not a prism's face list (uniform over every role)
        if (ptid == 0) atomicCAS(err, 0, 7);
        break;
      }
      if (ptid < nf) sHF[ptid] = hf[h0 + ptid];
      tp_bar(1);
      for (int t = ptid; t < nf * TF_NQ * TF_GEO; t += 256) {
        const int f = t / (TF_NQ * TF_GEO), r = t % (TF_NQ * TF_GEO);
        sface[f * FD + (r / TF_GEO) * TF_GEOS + r % TF_GEO] = geo[(size_t)sHF[f].face * TF_NQ * TF_GEO + r];
      }
      tp_bar(1);
      for (int f = 0; f < nf; f++, fi++) {
        const int b = fi & 1;
        // buffer b is free once the epilogue finished face fi - 2
        if (fi >= 2 && !tp_group_wait(bar_free + b, ((fi >> 1) - 1) & 1, ptid == 0, 1, abort_flag, slots + (fi & 1))) {
          stop = true;
          break;
        }
        const DgHalfFace &F = sHF[f];
        const double *sGeo = sface + f * FD;
        const bool interior = F.el2 >= 0;
        const int own2 = F.owner_is_2;
        const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
        const int ti = F.nfv == 4 ? 1 : 0;
        const int pr = (interior && tf_nqf[p2][ti] > tf_nqf[p1][ti]) ? p2 : p1;
        const int nq = tf_nqf[pr][ti];
        const int pnb = own2 ? p1 : p2;
        const int ns_nb = interior ? tf_ns[pnb] : 0;
        const int rows = NS + ns_nb;
        const int own_side = own2 ? 2 : 1;
        const int cfg_own = own2 ? F.cfg2 : F.cfg1, cfg_nb = own2 ? F.cfg1 : F.cfg2;
        if (pr > 3 || rows > Dm::ROWS || nq > TF_NQ) {  // a degree-4 neighbour (uniform)
          if (ptid == 0) {
            atomicCAS(err, 0, 7);
            *abort_flag = 1;
          }
          stop = true;
          break;
        }
        uint8_t *asl = smem + b * Tp::BUF, *bsl = asl + Dm::A_BYTES;
        int *ea = sexp + 192 * b, *eb = ea + 128;
        const double *tab_own = ftab + ftab_off[(cfg_own * 3 + pr - 1) * 3 + P - 1];
        const double *tab_nb = interior ? ftab + ftab_off[(cfg_nb * 3 + pr - 1) * 3 + pnb - 1] : tab_own;
        const long long so_bit = own2 ? (long long)1 << 63 : 0;
        auto tab_load = [&](int t, double2 &x01, double2 &x23) {
          const int r = t >> 4, q = t & 15;
          if (r < rows && q < nq) {
            const bool own = r < NS;
            const double *tb = (own ? tab_own : tab_nb) + ((size_t)q * (own ? NS : ns_nb) + (own ? r : r - NS)) * 4;
            x01 = __ldg(reinterpret_cast<const double2 *>(tb));
            x23 = __ldg(reinterpret_cast<const double2 *>(tb) + 1);
          } else {
            x01 = make_double2(0.0, 0.0);
            x23 = x01;
          }
        };
        double2 n01, n23;
        tab_load(ptid, n01, n23);
        for (int base = 0; base < rows * 16; base += 256) {
          const int t = base + ptid, r = t >> 4, q = t & 15;
          const bool live = r < rows, own = r < NS;  // uniform over the segment
          const double2 t01 = n01, t23 = n23;
          if (base + 256 < rows * 16) tab_load(t + 256, n01, n23);
          double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
          if (live && q < nq) {
            const int side = own ? own_side : 3 - own_side;
            const double *G = sGeo + q * TF_GEOS;
            const double *v = G + (side == 1 ? 2 : 5);
            const double phi = t01.x;
            const double g = fma(v[0], t01.y, fma(v[1], t23.x, v[2] * t23.y));
            a0 = __longlong_as_double(__double_as_longlong(phi) ^ (side == 2 ? (long long)1 << 63 : 0));
            a1 = g;
            if (own) {
              const double sphi = __longlong_as_double(__double_as_longlong(phi) ^ so_bit);
              b0 = fma(G[0], g, G[1] * sphi);
              b1 = -(G[0] * sphi);
            }
          }
          int xa = max(tf_biased_exp(a0), tf_biased_exp(a1)), xb = max(tf_biased_exp(b0), tf_biased_exp(b1));
#pragma unroll
          for (int o2 = 8; o2 >= 1; o2 >>= 1) {
            xa = max(xa, __shfl_xor_sync(0xffffffffu, xa, o2));
            xb = max(xb, __shfl_xor_sync(0xffffffffu, xb, o2));
          }
          if (!interior) {
            double sl = b0;
#pragma unroll
            for (int o2 = 8; o2 >= 1; o2 >>= 1) sl += __shfl_xor_sync(0xffffffffu, sl, o2);
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
              const uint32_t h0w = (uint32_t)(f0 >> 24), l0 = (uint32_t)f0 & 0xFFFFFFu;
              const uint32_t h1w = (uint32_t)(f1 >> 24), l1 = (uint32_t)f1 & 0xFFFFFFu;
              const float s0 = __double_as_longlong(a0) < 0 ? -1.0f : 1.0f, s1 = __double_as_longlong(a1) < 0 ? -1.0f : 1.0f;
#pragma unroll
              for (int i = 0; i < TF_SL; i++) {
                const uint32_t c0 = i < 4 ? (h0w >> (24 - 8 * i)) & 255u : (l0 >> (16 - 8 * (i - 4))) & 255u;
                const uint32_t c1 = i < 4 ? (h1w >> (24 - 8 * i)) & 255u : (l1 >> (16 - 8 * (i - 4))) & 255u;
                *(uint32_t *)(asl + i * Dm::A_STRIDE + off) = tf_bf16x2(c0, s0, c1, s1);
              }
            }
            if (own) {
              const unsigned long long f0 = tf_fixed(b0, EB), f1 = tf_fixed(b1, EB);
              const uint32_t h0w = (uint32_t)(f0 >> 24), l0 = (uint32_t)f0 & 0xFFFFFFu;
              const uint32_t h1w = (uint32_t)(f1 >> 24), l1 = (uint32_t)f1 & 0xFFFFFFu;
              const float s0 = __double_as_longlong(b0) < 0 ? -1.0f : 1.0f, s1 = __double_as_longlong(b1) < 0 ? -1.0f : 1.0f;
#pragma unroll
              for (int i = 0; i < TF_SL; i++) {
                const uint32_t c0 = i < 4 ? (h0w >> (24 - 8 * i)) & 255u : (l0 >> (16 - 8 * (i - 4))) & 255u;
                const uint32_t c1 = i < 4 ? (h1w >> (24 - 8 * i)) & 255u : (l1 >> (16 - 8 * (i - 4))) & 255u;
                *(uint32_t *)(bsl + i * Dm::B_SLICE + off) = tf_bf16x2(c0, s0, c1, s1);
              }
            }
          }
        }
        if (ptid == 0) {
          meta[b].blk = interior ? F.blk : -1;
          meta[b].rows = rows;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tp_bar(1);
        if (ptid == 0) tp_arrive(bar_full + b);
      }
      if (stop) break;
      // the owner's boundary rhs share (complete after the last barrier);
      // the next owner's first writes to sRacc follow its first barrier
      if (ptid < NS) {
        const double v = sRacc[ptid];
        sRacc[ptid] = 0.0;
        if (share)
          share[(size_t)o * (NS * NS + NS) + NS * NS + ptid] = v;
        else
          rhs[roff[e] + ptid] += v;
      }
    }
  } else {
    // ----------------------------- MMA + epilogue -----------------------------
    const int etid = tid - 256, ew = warp - 8, lq = ew & 3, half = ew >> 2;
    const int r_ep = lq * 32 + (tid & 31);
    const int issuer = (tid & 31) == 0 && ew < TP_ISSUERS ? ew : -1;
    int fi = 0;
    bool stop = false;
    for (int o = blockIdx.x; o < count && !stop; o += gridDim.x) {
      const int e = ent_el[o];
      const int nf = hf_ptr[e + 1] - hf_ptr[e];
      if (nf <= 0) continue;
      if (nf > TF_NF) break;
      for (int f = 0; f < nf; f++, fi++) {
        const int b = fi & 1;
        if (issuer >= 0 && tp_wait1(bar_full + b, (fi >> 1) & 1, abort_flag)) {
          // operands of face fi written; the accumulators are free (this
          // group finished face fi - 1 before getting here)
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NPAD >> 3) << 17) |
                                 ((uint32_t)(TF_M >> 4) << 24);
          const uint64_t ad0 = tc_desc(tc_smem(smem + b * Tp::BUF), 128, (TF_KP / 8) * 128);
          const uint64_t bd0 = tc_desc(tc_smem(smem + b * Tp::BUF + Dm::A_BYTES), 128, (TF_KP / 8) * 128);
          auto issue = [&](auto KK) {
            constexpr int K = decltype(KK)::value;
#pragma unroll
            for (int m = 0; m < 2; m++) {
              const int d = tp_acc(K, m);
              if (d < 0) continue;
#pragma unroll
              for (int i = 0; i <= d; i++)
#pragma unroll
                for (int ks = 0; ks < TF_KP / 16; ks++)
                  tc_mma<0>(tmem + d * NPAD, ad0 + (uint64_t)((i * Dm::A_STRIDE + ks * 256) >> 4),
                            bd0 + (uint64_t)(((d - i) * Dm::B_SLICE + ks * 256) >> 4), idesc,
                            (i == 0 && ks == 0) ? 0u : 1u);
            }
          };
          switch (issuer) {
            case 0: issue(std::integral_constant<int, 0>{}); break;
            case 1: issue(std::integral_constant<int, 1>{}); break;
            case 2: issue(std::integral_constant<int, 2>{}); break;
            default: issue(std::integral_constant<int, 3>{}); break;
          }
          tc_commit(tc_smem(bar_mma + b));
          issued_any = true;
        }
        __syncwarp();  // the issuing warps reconverged before their aligned TMEM loads
        if (!tp_group_wait(bar_mma + b, (fi >> 1) & 1, etid == 0, 2, abort_flag, slots + 2 + (fi & 1))) {
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int rows = meta[b].rows;
        const long long blk = meta[b].blk;
        const int *ea = sexp + 192 * b, *eb = ea + 128;
        if (lq * 32 < rows) {
          const bool rok = r_ep < rows;
          const int sa = rok ? ea[r_ep] : 0;
          double *oblk = blk >= 0 ? val + blk : nullptr;
#pragma unroll
          for (int grp = 0; grp < NPAD / 16; grp++) {
            const int cl = half * (NPAD / 2) + grp * 8;
            if (cl >= NS) continue;  // padding columns only (uniform over the warp)
            float C[TF_SL][8];
#pragma unroll
            for (int d = 0; d < TF_SL; d++) tc_ld8(tmem + ((uint32_t)(lq * 32) << 16) + d * NPAD + cl, C[d]);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int c = 0; c < 8; c++) {
              const int i = cl + c;
              if (!rok || i >= NS) continue;
              // u_ab = C_a 256 + C_b from the float bits (exact-integer
              // trick, its offset folded into one constant; modulo 2^32,
              // the true values fit int32); then
              // T = u01 2^30 + u23 2^14 + floor((u45 256 + C_6) / 2^10)
              // with the floor in int32 (u45 = 4 q + r, 0 <= r < 4)
              const uint32_t K2 = 257u * 0x4B400000u;
              const int u01 = (int)((uint32_t)__float_as_int(C[0][c] + 12582912.0f) * 256u +
                                    (uint32_t)__float_as_int(C[1][c] + 12582912.0f) - K2);
              const int u23 = (int)((uint32_t)__float_as_int(C[2][c] + 12582912.0f) * 256u +
                                    (uint32_t)__float_as_int(C[3][c] + 12582912.0f) - K2);
              const int u45 = (int)((uint32_t)__float_as_int(C[4][c] + 12582912.0f) * 256u +
                                    (uint32_t)__float_as_int(C[5][c] + 12582912.0f) - K2);
              const int lo10 = (u45 >> 2) + ((((u45 & 3) << 8) + tf_exact_int(C[6][c])) >> 10);
              const long long T = (long long)u01 * (1LL << 30) + (long long)u23 * (1LL << 14) + lo10;
              const double v = tf_i64_scaled(T, sa + eb[i] - 54);
              if (r_ep < NS)
                sD[r_ep * SD_LD + i] += v;
              else
                oblk[i + (size_t)NS * (r_ep - NS)] = v;
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        tp_bar(2);  // TMEM, meta and exponents of buffer b read
        if (etid == 0) tp_arrive(bar_free + b);
      }
      if (stop) break;
      // the owner's diagonal-block share (complete after the last barrier),
      // then cleared for the next owner
      if (share) {
        double *sd = share + (size_t)o * (NS * NS + NS);
        for (int t = etid; t < NS * NS; t += 256) {
          double &s = sD[(t / NS) * SD_LD + t % NS];
          sd[t] = s;
          s = 0.0;
        }
      } else {
        double *dblk = val + boff_diag[e];
        for (int t = etid; t < NS * NS; t += 256) {
          double &s = sD[(t / NS) * SD_LD + t % NS];
          dblk[t] += s;
          s = 0.0;
        }
      }
      tp_bar(2);
    }
  }
  // an issuer whose MMAs may still run (a role gave up after they were
  // issued) lets them finish (bounded) before the TMEM is freed
  if (warp >= 8 && (tid & 31) == 0 && warp - 8 < TP_ISSUERS && issued_any) {
    tc_commit(tc_smem(bar_drain + (warp - 8)));
    tc_wait(tc_smem(bar_drain + (warp - 8)), 0);
  }
  __syncwarp();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  if (tid == 0 && *abort_flag) atomicCAS(err, 0, 6);
}

bool dg_tc_faces_supported(int p) { return p >= 1 && p <= 3; }

// The owners' diagonal-block and rhs shares from scratch (one slot of
// NS^2 + NS values per owner, in list order) added to the blocks and rows the
// volume kernel wrote: one block per owner.
template <int NS>
__global__ void __launch_bounds__(256) dg_face_share_add_kernel(int count, const int *__restrict__ ent_el,
                                                                const double *__restrict__ share,
                                                                const long long *__restrict__ boff_diag,
                                                                const int *__restrict__ roff, double *__restrict__ val,
                                                                double *__restrict__ rhs) {
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const double *sd = share + (size_t)bi * (NS * NS + NS);
  double *dblk = val + boff_diag[e];
  for (int t = threadIdx.x; t < NS * NS; t += blockDim.x) dblk[t] += sd[t];
  if (threadIdx.x < NS) rhs[roff[e] + threadIdx.x] += sd[NS * NS + threadIdx.x];
}

int launch_dg_face_share_add(cudaStream_t st, int p, int count, const int *ent_el, const double *share,
                             const long long *boff_diag, const int *roff, double *val, double *rhs) {
  if (count <= 0) return 0;
  switch (p) {
    case 1: dg_face_share_add_kernel<6><<<count, 256, 0, st>>>(count, ent_el, share, boff_diag, roff, val, rhs); break;
    case 2: dg_face_share_add_kernel<18><<<count, 256, 0, st>>>(count, ent_el, share, boff_diag, roff, val, rhs); break;
    default: dg_face_share_add_kernel<40><<<count, 256, 0, st>>>(count, ent_el, share, boff_diag, roff, val, rhs); break;
  }
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_dg_tc_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                       const DgHalfFace *hf, const int *el_p, const double *geo, const double *ftab,
                       const long long *ftab_off, double g, const long long *boff_diag, const int *roff,
                       double *val, double *rhs, int *err, double *share) {
  if (count <= 0) return 0;
  GB_CHECK(dg_tc_faces_supported(p), "tensor-core DG face kernel covers p = 1..3");
  GB_CHECK(geo && ftab && ftab_off, "tensor-core DG faces need the face geometry and basis tables");
  // persistent: one CTA per SM (each takes the whole TMEM), owners strided
  int dev = 0, nsm = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = count < nsm ? count : nsm;
#define GB_TF_LAUNCH(PP)                                                                                          \
  {                                                                                                               \
    const int smem = TpDims<PP>::SMEM;                                                                            \
    GB_CUDA(cudaFuncSetAttribute(dg_tc_faces_pipe_kernel<PP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
    dg_tc_faces_pipe_kernel<PP><<<grid, TP_THREADS, smem, st>>>(count, ent_el, hf_ptr, hf, el_p, geo, ftab,       \
                                                                ftab_off, g, boff_diag, roff, val, rhs, err, share); \
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

long long dg_face_table_size(int ncfg, const unsigned char *cfg, long long *tab_off) {
  long long off = 0;
  for (int c = 0; c < ncfg; c++) {
    const int ti = cfg[5 * c] == 4 ? 1 : 0;
    for (int pr = 1; pr <= 3; pr++)
      for (int pb = 1; pb <= 3; pb++) {
        tab_off[(c * 3 + pr - 1) * 3 + pb - 1] = off;
        off += 4LL * GB_DG_NQF[pr][ti] * GB_DG_NS[pb];
      }
  }
  return off;
}

int launch_dg_face_tables(cudaStream_t st, int ncfg, const unsigned char *cfg, const long long *tab_off,
                          double *tab) {
  if (ncfg <= 0) return 0;
  dg_face_table_kernel<<<ncfg * 9, 256, 0, st>>>(cfg, tab_off, tab);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_dg_face_geometry(cudaStream_t st, int count, const int *faces_hf, const DgHalfFace *hf,
                            const int *el_p, const int *el_nodes, const double *xyz, const double *k_el,
                            const double *D_el, double pen, double *geo) {
  if (count <= 0) return 0;
  const long long threads = (long long)count * TF_NQ;
  dg_face_geometry_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(count, faces_hf, hf, el_p, el_nodes,
                                                                            xyz, k_el, D_el, pen, geo);
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
