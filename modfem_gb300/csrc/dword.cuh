// Double-word ("float-float") arithmetic for element math on the FP32 pipe.
//
// GB300 issues FP64 at 1/64 of the FP32 rate.  A double-word value is the
// unevaluated sum h + l of two floats with |l| <= ulp(h) (about 48
// significant bits, relative rounding of order 2^-47 per operation), so an
// element matrix computed with these operations lies within about 1e-14 of
// its FP64 counterpart at a fraction of the FP64 pipe's issue cost.
//
// Building blocks (published algorithms, restated here):
//  * TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e == a + b exactly, 6 ops;
//  * FastTwoSum (Dekker 1971), |a| >= |b|: 3 ops;
//  * TwoProd with a fused multiply-add: p + e == a * b exactly, 2 ops;
//  * sums and products of double words after Joldes, Muller and Popescu,
//    "Tight and rigorous error bounds for basic building blocks of
//    double-word arithmetic", ACM TOMS 44(2), 2017: the "sloppy" sum (error
//    bounded relative to |x| + |y|, as for an FP64 sum of the same operands)
//    and the product with the l*l term dropped;
//  * reciprocal: a float reciprocal refined by one Newton step
//    r' = r + r (1 - x r) in double-word arithmetic.
// Conversions go through the integer pipe (bit fields); the only FP64
// instruction is the final h + l of a double word widened to double.
//
// Every float operation is an explicit round-to-nearest intrinsic on the
// device (no contraction into fused operations); the host build (for the CPU
// check of the element math) must be compiled with -ffp-contract=off.
#pragma once

#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define DW_HD __host__ __device__ __forceinline__
#else
#define DW_HD inline
#endif

namespace gbfem {

DW_HD float f_add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DW_HD float f_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DW_HD float f_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DW_HD float f_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

DW_HD unsigned f_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  unsigned u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
DW_HD float f_from_bits(unsigned u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}
DW_HD unsigned long long d_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
DW_HD double d_from_bits(unsigned long long u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

#if defined(__CUDACC__)
#define DW_CX __host__ __device__ constexpr
#else
#define DW_CX constexpr
#endif

struct alignas(8) dw {
  float h, l;
  dw() = default;
  // constants: split at compile time (literal arguments fold)
  DW_CX dw(double c) : h((float)c), l((float)(c - (double)(float)c)) {}
  DW_CX dw(float hh, float ll) : h(hh), l(ll) {}
};

// s + e == a + b exactly
DW_HD dw two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_sub(s, a);
  const float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return dw(s, e);
}
// s + e == a + b exactly when |a| >= |b| (or a == 0)
DW_HD dw fast_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return dw(s, f_sub(b, f_sub(s, a)));
}

DW_HD dw operator-(dw x) { return dw(-x.h, -x.l); }
DW_HD dw operator+(dw x, dw y) {
  const dw s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, f_add(s.l, f_add(x.l, y.l)));
}
DW_HD dw operator-(dw x, dw y) { return x + (-y); }
DW_HD dw operator*(dw x, dw y) {
  const float p = f_mul(x.h, y.h);
  float e = f_fma(x.h, y.h, -p);
  e = f_fma(x.h, y.l, e);
  e = f_fma(x.l, y.h, e);
  return fast_two_sum(p, e);
}
// x * y + z with one renormalisation
DW_HD dw t_fma(dw x, dw y, dw z) {
  const float p = f_mul(x.h, y.h);
  float e = f_fma(x.h, y.h, -p);
  e = f_fma(x.h, y.l, e);
  e = f_fma(x.l, y.h, e);
  const dw s = two_sum(p, z.h);
  return fast_two_sum(s.h, f_add(s.l, f_add(e, z.l)));
}
DW_HD dw t_abs(dw x) { return x.h < 0.0f ? -x : x; }
DW_HD dw &operator+=(dw &x, dw y) { return x = x + y; }
DW_HD dw &operator-=(dw &x, dw y) { return x = x - y; }

// a * b - c * d with one renormalisation (two exact products, one TwoSum)
DW_HD dw dw_fms(dw a, dw b, dw c, dw d) {
  const float p1 = f_mul(a.h, b.h), p2 = f_mul(c.h, d.h);
  float e1 = f_fma(a.h, b.h, -p1), e2 = f_fma(c.h, d.h, -p2);
  e1 = f_fma(a.h, b.l, e1);
  e2 = f_fma(c.h, d.l, e2);
  e1 = f_fma(a.l, b.h, e1);
  e2 = f_fma(c.l, d.h, e2);
  const dw s = two_sum(p1, -p2);
  return fast_two_sum(s.h, f_add(s.l, f_sub(e1, e2)));
}

// a0 b0 + a1 b1 + a2 b2 with one renormalisation
DW_HD dw dw_dot3(dw a0, dw b0, dw a1, dw b1, dw a2, dw b2) {
  const float p0 = f_mul(a0.h, b0.h), p1 = f_mul(a1.h, b1.h), p2 = f_mul(a2.h, b2.h);
  float e0 = f_fma(a0.h, b0.h, -p0), e1 = f_fma(a1.h, b1.h, -p1), e2 = f_fma(a2.h, b2.h, -p2);
  e0 = f_fma(a0.h, b0.l, e0);
  e1 = f_fma(a1.h, b1.l, e1);
  e2 = f_fma(a2.h, b2.l, e2);
  e0 = f_fma(a0.l, b0.h, e0);
  e1 = f_fma(a1.l, b1.h, e1);
  e2 = f_fma(a2.l, b2.h, e2);
  const dw s = two_sum(p0, p1);
  const dw s2 = two_sum(s.h, p2);
  return fast_two_sum(s2.h, f_add(f_add(s.l, s2.l), f_add(e0, f_add(e1, e2))));
}

// 1/x: hardware reciprocal estimate, one Newton step r + r (1 - x r) (the
// residual formed with fused multiply-adds)
DW_HD dw dw_recip(dw x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x.h));
#else
  const float r = 1.0f / x.h;
#endif
  float t = f_fma(-x.h, r, 1.0f);
  t = f_fma(-x.l, r, t);
  return fast_two_sum(r, f_mul(r, t));
}

// double -> double word: the leading 24 significand bits (truncation) and
// the remaining 29 bits rounded to a float, from the bit fields.  Below
// 2^-74 the low word is dropped (24 bits kept), below 2^-126 the value reads
// as zero; from 2^128 up it reads as infinity.  Integer and conversion pipes
// only: no branch the compiler could turn into predicated FP64 work.
DW_HD dw dw_from_double(double x) {
  const unsigned long long b = d_bits(x);
  const int E = (int)((b >> 52) & 0x7FF);
  const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
  const int ef = E - 896;  // float biased exponent of the high word
  unsigned hb = sgn | ((unsigned)ef << 23) | (unsigned)((b >> 29) & 0x7FFFFFu);
  hb = ef <= 0 ? sgn : (ef >= 255 ? (sgn | 0x7F800000u) : hb);
  const unsigned r = (unsigned)(b & 0x1FFFFFFFu);  // x - h = r 2^(E-1075)
  const int es = E - 948;                         // float biased exponent of 2^(E-1075)
  const float scale = f_from_bits(es >= 1 && ef < 255 ? (sgn | ((unsigned)es << 23)) : 0u);
  return dw(f_from_bits(hb), f_mul((float)r, scale));
}

// float -> double by bit fields (exact for normal floats; zero and
// subnormals give a signed zero, infinities and NaNs pass through)
DW_HD double f_to_double_bits(float x) {
  const unsigned b = f_bits(x);
  const unsigned e = (b >> 23) & 0xFFu;
  unsigned hi = (((b & 0x7FFFFFFFu) >> 3) + (896u << 20)) | (b & 0x80000000u);
  hi = e == 0 ? (b & 0x80000000u) : (e == 255 ? (hi | 0x7FF00000u) : hi);
  const unsigned lo = e == 0 ? 0u : (b << 29);
  return d_from_bits(((unsigned long long)hi << 32) | lo);
}

// double word -> double: both words widened by bit fields, one FP64 add
// (h + l rounded to 53 bits)
DW_HD double dw_to_double(dw v) { return f_to_double_bits(v.h) + f_to_double_bits(v.l); }

// double -> double word as a float2 (h, l)
DW_HD float2 dw_f2(double v) {
  const dw d = dw_from_double(v);
  float2 r;
  r.x = d.h;
  r.y = d.l;
  return r;
}

// Accumulator of a long sum of double-word products: the high parts summed
// by TwoSum into h, every rounding error (of the products' TwoProd and of
// the TwoSums) collected in the float e and folded into the pair (h, l) every
// few terms.  Error of order u^2 = 2^-48 of the summed magnitudes.
struct DwAcc {
  float h, l, e;  // value h + l + e
};
DW_HD void dwacc_prod(DwAcc &a, float2 x, float2 y) {
  const float p = f_mul(x.x, y.x);
  float pe = f_fma(x.x, y.x, -p);
  pe = f_fma(x.x, y.y, pe);
  pe = f_fma(x.y, y.x, pe);
  const dw s = two_sum(a.h, p);
  a.h = s.h;
  a.e = f_add(a.e, f_add(s.l, pe));
}
DW_HD void dwacc_fold(DwAcc &a) {
  const dw r = fast_two_sum(a.h, f_add(a.l, a.e));
  a.h = r.h;
  a.l = r.l;
  a.e = 0.0f;
}
DW_HD double dwacc_value(DwAcc a) {
  dwacc_fold(a);
  return dw_to_double(dw(a.h, a.l));
}
#if defined(__CUDACC__)
// Entries k = k0 + m THR (m < PER, k < kend) of an NS-row block: row
// i = k % NS, table column j = k / NS + col_lo; sum over the points of
// L_i Phi_j + M_i Gam_j into a[m].  The PER chains run interleaved (each
// TwoSum waits on its predecessor in the same chain); with THR a multiple of
// NS every entry of a thread has the same row and the L, M loads are shared.
template <int NS, int THR, int PER>
__device__ __forceinline__ void dwacc_face_block(DwAcc (&a)[PER], const float2 *sL, const float2 *sM,
                                                 const float2 *sPhi, const float2 *sGam, int nq, int ncol, int k0,
                                                 int kend, int col_lo) {
  int ii[PER], jj[PER];
  bool ok[PER];
#pragma unroll
  for (int m = 0; m < PER; m++) {
    const int k = k0 + m * THR;
    ok[m] = k < kend;
    ii[m] = ok[m] ? k % NS : 0;
    jj[m] = ok[m] ? k / NS + col_lo : 0;
  }
  for (int q = 0; q < nq; q++) {
    const float2 *Lq = sL + q * NS, *Mq = sM + q * NS, *Pq = sPhi + q * ncol, *Gq = sGam + q * ncol;
    float2 L0 = Lq[ii[0]], M0 = Mq[ii[0]];
#pragma unroll
    for (int m = 0; m < PER; m++) {
      if (!ok[m]) continue;
      const float2 L = (THR % NS == 0) ? L0 : Lq[ii[m]], M = (THR % NS == 0) ? M0 : Mq[ii[m]];
      dwacc_prod(a[m], L, Pq[jj[m]]);
      dwacc_prod(a[m], M, Gq[jj[m]]);
    }
    if ((q & 3) == 3) {
#pragma unroll
      for (int m = 0; m < PER; m++) dwacc_fold(a[m]);
    }
  }
#pragma unroll
  for (int m = 0; m < PER; m++) dwacc_fold(a[m]);
}

// A TI x TJ tile of an NS-row block per thread: rows i0 .. i0 + TI - 1 (all
// below NS), table columns col_lo + j0 + y for j0 + y < jend (columns past
// jend repeat column j0 and are not to be stored).  A point's L, M values
// are loaded once per tile row and its Phi, Gam values once per tile column
// (TI + TJ pairs of loads for TI TJ entries instead of four loads an entry);
// each entry gets the products and folds of dwacc_face_block in the same
// order, so the sums are bit-identical.
template <int NS, int TI, int TJ>
__device__ __forceinline__ void dwacc_face_tile(DwAcc (&a)[TI][TJ], const float2 *sL, const float2 *sM,
                                                const float2 *sPhi, const float2 *sGam, int nq, int ncol, int i0,
                                                int j0, int jend, int col_lo) {
  for (int q = 0; q < nq; q++) {
    const float2 *Lq = sL + q * NS + i0, *Mq = sM + q * NS + i0;
    const float2 *Pq = sPhi + q * ncol + col_lo, *Gq = sGam + q * ncol + col_lo;
    float2 L[TI], M[TI], P[TJ], G[TJ];
#pragma unroll
    for (int x = 0; x < TI; x++) {
      L[x] = Lq[x];
      M[x] = Mq[x];
    }
#pragma unroll
    for (int y = 0; y < TJ; y++) {
      const int j = j0 + y < jend ? j0 + y : j0;
      P[y] = Pq[j];
      G[y] = Gq[j];
    }
#pragma unroll
    for (int x = 0; x < TI; x++)
#pragma unroll
      for (int y = 0; y < TJ; y++) {
        dwacc_prod(a[x][y], L[x], P[y]);
        dwacc_prod(a[x][y], M[x], G[y]);
      }
    if ((q & 3) == 3) {
#pragma unroll
      for (int x = 0; x < TI; x++)
#pragma unroll
        for (int y = 0; y < TJ; y++) dwacc_fold(a[x][y]);
    }
  }
#pragma unroll
  for (int x = 0; x < TI; x++)
#pragma unroll
    for (int y = 0; y < TJ; y++) dwacc_fold(a[x][y]);
}
#endif

}  // namespace gbfem
