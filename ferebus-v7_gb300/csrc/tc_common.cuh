// Shared device helpers of the tcgen05 kernels: mbarriers with bounded waits,
// shared-memory matrix descriptors, kind::f16 MMA issue and commit, TMA and
// bulk copies, the FP64 -> 55-bit fixed-point conversion, and the exact
// conversions of level sums.
#pragma once
#include "fgpu_internal.h"

#include <cuda_fp16.h>

namespace fgpu {
namespace {

// one k-chunk of 16 of the digit planes in shared memory (no swizzle,
// K-major core matrices): A = 128 rows, B = 64 rows, 7 planes each
constexpr uint32_t A_STAGE = NSLICE * 4096;  // 7 planes x 2 k-groups x 128 rows x 16 B
constexpr uint32_t B_STAGE = NSLICE * 2048;  // 7 planes x 2 k-groups x 64 rows x 16 B
constexpr uint32_t STAGE = A_STAGE + B_STAGE;  // 43008 B

__device__ __forceinline__ uint32_t su32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
// wait for the phase of `parity` to complete, giving up after `limit` polls
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, int limit) {
  for (int it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
// the kernels' bounded wait: 2^22 polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) { return mbar_wait_n(bar, parity, 1 << 22); }

// After a bounded wait gave up: wait (bounded) until the copies issued into
// a `nstage`-deep ring have landed, so that no copy writes this CTA's shared
// memory after it exits.  `issued` counts the k-chunks whose copies were
// issued; chunk c went to stage c % nstage and completes that stage's phase
// c / nstage, and the last chunk of each stage is the only one that can
// still be in flight (a stage is reissued only after its previous chunk was
// consumed, i.e. had landed).
__device__ __forceinline__ void drain_ring(uint64_t* full, int nstage, uint32_t issued) {
  for (int st = 0; st < nstage && (uint32_t)st < issued; ++st) {
    const uint32_t last = issued - 1 - ((issued - 1 - (uint32_t)st) % (uint32_t)nstage);
    mbar_wait(&full[st], (last / nstage) & 1);
  }
}

// one non-blocking probe of an mbarrier phase
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// tcgen05 shared-memory descriptor, no swizzle, K-major core matrices
// (8 rows x 16 bytes): lbo = byte stride between core matrices along K,
// sbo = along M/N; descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// kind::f16 instruction descriptor: f32 accumulator, f16 A/B, both K-major, M=128, N=64.
constexpr uint32_t IDESC_128x64 = (1u << 4) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC_128x64), "r"(accumulate));
}
__device__ __forceinline__ void mma_f16_desc(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
// After a bounded wait gave up: one more commit tracks every MMA this thread
// issued; waiting (bounded) on it means none still writes TMEM when the CTA
// deallocates it.  `drain` is an mbarrier of count 1 used for nothing else.
__device__ __forceinline__ void drain_mmas(uint64_t* drain) {
  mma_commit(drain);
  mbar_wait(drain, 0);
}

// round(x * 2^(55 - e)) for |x| <= 2^e, with integer operations only.
// Sets *bad when the scale bound is violated (|x| > 2^(e+3)).
__device__ __forceinline__ long long to_fixed55(double x, int e, bool* bad) {
  const long long bits = __double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7FF);
  if (E == 0) return 0;  // zero or subnormal (below 2^-1022: far under the 2^-55 resolution)
  if (E == 0x7FF) {
    *bad = true;
    return 0;
  }
  const long long M = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  const int sh = E - 1075 + 55 - e;
  long long F;
  if (sh >= 0) {
    if (sh > 3) {
      *bad = true;
      return 0;
    }
    F = M << sh;
  } else if (sh > -63) {
    F = (M + (1LL << (-sh - 1))) >> (-sh);
  } else {
    F = 0;
  }
  return bits < 0 ? -F : F;
}

__device__ __forceinline__ void tma_load_5d(void* dst, const void* tmap, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(su32(dst)),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)),
      "l"(src), "r"(bytes), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

// W 2^e rounded to the nearest double (ties to even) with integer
// operations only, W a signed 64-bit integer: the same double as the exact
// product correctly rounded, without the FP64 pipe.  Results below 2^-1022
// (never reached by the factor's scales) flush to 0.
__device__ __forceinline__ double w64_to_double(long long W, int e) {
  if (W == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)W >> 63;
  unsigned long long a = sgn ? 0ULL - (unsigned long long)W : (unsigned long long)W;
  const int lz = __clzll((long long)a);
  a <<= lz;  // leading one at bit 63
  unsigned long long mant = a >> 11;  // 53 bits
  const unsigned rb = (unsigned)a & 0x7FFu;
  if (rb > 0x400u || (rb == 0x400u && (mant & 1))) ++mant;
  int be = 63 - lz + e + 1023;  // biased exponent of 1.f
  if (mant >> 53) {
    mant >>= 1;
    ++be;
  }
  if (be <= 0) return sgn ? -0.0 : 0.0;
  if (be >= 2047) return __longlong_as_double((long long)((sgn << 63) | 0x7FF0000000000000ULL));
  return __longlong_as_double((long long)((sgn << 63) | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFULL)));
}

// The exact integer W = sum_l S_l 256^(6 - l) of 7 level sums, in wrapping
// 64-bit arithmetic: callers guarantee |W| < 2^63 (partial level sums may
// exceed it; the wrapped total is still exact).
__device__ __forceinline__ long long levels_to_w64(const int S[7]) {
  unsigned long long w = (unsigned long long)(long long)S[6];
  w += (unsigned long long)(long long)S[5] << 8;
  w += (unsigned long long)(long long)S[4] << 16;
  w += (unsigned long long)(long long)S[3] << 24;
  w += (unsigned long long)(long long)S[2] << 32;
  w += (unsigned long long)(long long)S[1] << 40;
  w += (unsigned long long)(long long)S[0] << 48;
  return (long long)w;
}

// Exact integer level sums without the conversion unit.  For an
// integer-valued float x with -2^22 <= x < 2^22, x + 1.5 2^23 is exact and
// its bits are b = 0x4B000000 + (x + 2^22).  Callers establish the range
// first: by a bound on the contraction, or by checking the raw sums of a
// warp's group (|x| < 2^22) and converting with F2I otherwise.
__device__ __forceinline__ uint32_t level_bits(uint32_t v) {
  return __float_as_uint(__uint_as_float(v) + 12582912.0f);
}

// W = sum_l x_l 256^(6 - l) from the valid bits b_l of column jj's 7 level
// sums, in wrapping 64-bit arithmetic.  Adjacent levels pair up exactly in
// 32 bits: b_l 256 + b_(l+1) = (x_l + 2^22) 256 + (x_(l+1) + 2^22) +
// 0x4B000000 (the top byte of b_l leaves modulo 2^32, bit 23 is clear), below
// 2^32; the offsets leave as one constant.
constexpr unsigned long long LEVEL_BITS_BIAS =
    (1ULL << 22) * 0x0001010101010101ULL + 0x4B000000ULL * ((1ULL << 40) + (1ULL << 24) + (1ULL << 8) + 1ULL);
__device__ __forceinline__ long long level_bits_to_w64(const uint32_t (&b)[7][8], int jj) {
  const uint32_t p01 = b[0][jj] * 256u + b[1][jj];
  const uint32_t p23 = b[2][jj] * 256u + b[3][jj];
  const uint32_t p45 = b[4][jj] * 256u + b[5][jj];
  unsigned long long w = (unsigned long long)p45 * 256u + b[6][jj];
  w += (unsigned long long)p23 << 24;
  w += (unsigned long long)p01 << 40;
  return (long long)(w - LEVEL_BITS_BIAS);
}

// an integer-valued float x with |x| <= 2^22 as an int, exactly, without a
// conversion instruction: x + 1.5 * 2^23 lies in [2^23, 2^24], where the
// float's low mantissa bits are x + 2^22 (one FADD and one IADD)
__device__ __forceinline__ int small_f2i(float x) { return __float_as_int(x + 12582912.0f) - 0x4B400000; }

}  // namespace
}  // namespace fgpu
