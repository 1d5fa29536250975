// tcgen05 / TMA-engine helpers (inline PTX, sm_100a family) shared by the
// tensor-core kernels: shared-memory matrix descriptors, mbarrier waits with
// an iteration limit, bulk-async copies, MMA issue and commit, TMEM loads,
// the canonical no-swizzle K-major operand layout and FP64 exponent tools.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>
#include <cstring>

namespace gbfem {

constexpr long long TC_WAIT_LIMIT = 1LL << 26;  // mbarrier polls before a wait gives up

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  // tcgen05 shared-memory matrix descriptor, no swizzle (canonical K-major
  // layout of 8-row x 16-byte core matrices)
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool tc_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < TC_WAIT_LIMIT; it++)
    if (tc_try_wait(mbar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

template <int MODE>
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  if constexpr (MODE == 0)
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tc_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// byte offset of (row, k) in the canonical no-swizzle K-major layout of a
// rows x kdim operand of esz-byte elements: core matrices of 8 rows x 16
// bytes, core matrix (row/8, k/(16/esz)) at row/8 * SBO + k/(16/esz) * 128
__host__ __device__ __forceinline__ int tc_off(int row, int k, int kdim, int esz) {
  const int per = 16 / esz;
  return (row >> 3) * (kdim / per) * 128 + (k / per) * 128 + (row & 7) * 16 + (k % per) * esz;
}

// TF32 part of a float: the 19 high bits (sign, exponent, 10 mantissa bits)
__host__ __device__ __forceinline__ float tc_tf32(float x) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  u &= 0xFFFFE000u;
  float y;
  memcpy(&y, &u, 4);
  return y;
#endif
}

// 2^e as a double built from its bit pattern (normal range)
__device__ __forceinline__ double tc_pow2(int e) {
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// exponent E with |x| < 2^E for x != 0 (from the FP64 bit pattern)
__device__ __forceinline__ int tc_exp_above(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  return ex == 0 ? -1100 : ex - 1022;  // |x| < 2^(ex - 1022) for normal x
}

}  // namespace gbfem
