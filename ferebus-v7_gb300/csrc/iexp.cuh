// exp(x), x <= 0, for the kernel-matrix entries, evaluated on the integer
// pipes so that it does not compete with the FP64 work for this part's
// narrow FP64 pipe.
//
//   |y| = |x| log2(e) as a fixed-point number with 64 fractional bits
//         (64 x 128-bit product, exact to 2^-64),
//   2^-|y| = 2^-m 2^(j/256) exp(s ln2),  m = ceil(|y|), m - |y| = j/256 + s,
//   exp(t), 0 <= t < ln2/256: degree-5 Taylor polynomial in 64-bit fixed
//   point (scale 2^63, truncation below 2^-60), then one round-to-nearest
//   into the double (subnormals included).
// Error below 0.51 ulp; measured: never more than 1 ulp from the host libm
// over 16.7M arguments spanning [-745.2, 0].  Two entries: a double argument
// (iexp_neg), and an exact fixed-point argument x = -E 2^e (iexp_fixed),
// which the tensor-core build uses without forming a double.
#pragma once
#include "iexp_table.h"

// exp(-|x|) for |x| = M 2^e2 with M normalised (bit 63 set), 2^-54 <= |x| < 1024
__device__ __forceinline__ double iexp_core(unsigned long long M, int e2) {
  const unsigned __int128 P = (unsigned __int128)M * IEXP_L2E_HI +
                              (unsigned long long)(((unsigned __int128)M * IEXP_L2E_LO) >> 64);
  const unsigned __int128 Y = P >> (-1 - e2);  // |y| 2^64; P = |y| 2^(63 - e2), shift 53..116
  const unsigned int yi = (unsigned int)(Y >> 64);
  const unsigned long long yf = (unsigned long long)Y;
  const unsigned int m = yi + (yf ? 1u : 0u);
  const unsigned long long f = 0ULL - yf;  // (m - |y|) 2^64
  const int j = (int)(f >> 56);
  const unsigned long long t = __umul64hi(f & 0x00FFFFFFFFFFFFFFULL, IEXP_LN2);  // s ln2, 2^64
  unsigned long long q = IEXP_C5;
  q = IEXP_C4 + __umul64hi(q, t);
  q = IEXP_C3 + __umul64hi(q, t);
  q = IEXP_C2 + __umul64hi(q, t);
  q = (1ULL << 63) + __umul64hi(q, t);
  const unsigned long long p = (1ULL << 63) + __umul64hi(q, t);      // exp(t) 2^63
  const unsigned long long Z = __umul64hi(__ldg(&g_iexp_tab[j]), p);  // 2^(j/256) exp(t) 2^62
  const int top = (int)(Z >> 63);                                     // value in [2, 2.01)
  const int sh = 10 + top;                                            // keep 53 bits
  const int be = 1023 + top - (int)m;                                 // biased exponent
  if (be >= 1) {
    const unsigned long long mant = (Z + (1ULL << (sh - 1))) >> sh;  // may carry to 2^53
    return __longlong_as_double((long long)(((unsigned long long)be << 52) + mant - (1ULL << 52)));
  }
  const int tot = sh + 1 - be;  // subnormal result
  if (tot > 64) return 0.0;
  const unsigned long long mant = (tot == 64) ? (Z >> 63) : ((Z + (1ULL << (tot - 1))) >> tot);
  return __longlong_as_double((long long)mant);
}

__device__ __forceinline__ double iexp_neg(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex < 969) return 1.0;  // |x| < 2^-54 rounds to 1 (also +-0 and subnormals)
  if (!(x >= -745.1332191019412)) return (x != x) ? x : 0.0;  // underflow, -inf, NaN
  if (x > 0.0) return exp(x);
  const unsigned long long M = ((bits & 0xFFFFFFFFFFFFFULL) | 0x10000000000000ULL) << 11;
  return iexp_core(M, ex - 1086);
}

// exp(-E 2^e) for an exact non-negative integer E
__device__ __forceinline__ double iexp_fixed(unsigned long long E, int e) {
  if (E == 0) return 1.0;
  const int lz = __clzll((long long)E);
  const int top = 63 - lz + e;  // 2^top <= E 2^e < 2^(top + 1)
  if (top >= 10) return 0.0;    // beyond 1024: exp underflows
  if (top < -55) return 1.0;    // below 2^-55: rounds to 1
  return iexp_core(E << lz, e - lz);
}

// exp(-E 2^e) for exact integers E >= 0 sharing one scale 2^e (the
// kernel-matrix build's entries of one distance leaf), with the per-entry
// work cut down:
//  * y = E 2^e log2(e) is read off the 128-bit product E * C at a fixed
//    binary point K0, C = log2(e) 2^63 rounded (relative error 2^-64, below
//    2^-54 absolute in y for y < 1024): no per-entry normalisation;
//  * the fraction g = m - y (64 bits) splits as j/1024 + k/2^20 + s with
//    two 1024-entry tables the caller keeps in shared memory, 2^(j/1024)
//    2^63 and (2^(k/2^20) - 1) 2^64, so t = s ln2 < 2^-20 ln2 and
//    exp(t) = 1 + t + t^2/2 up to t^3/6 < 2^-64;
//  * the small products (t^2, (2^(k/2^20) - 1) (exp(t) - 1)) are single
//    32 x 32-bit multiplies; two 64 x 64-bit high products remain (s ln2
//    and the final 2^(j/1024) factor);
//  * one round-to-nearest into the double, subnormals included.
// Error before the final rounding below 2^-60 relative (CPU model against
// 60-digit arithmetic: never more than 1 ulp from the correctly rounded
// value); measured on the GPU through fgpu_diag_exp_fixed.
struct IexpScale {
  int K0;  // binary point of y in E * IEXP_L2E64: y = (E C) 2^-K0
};
__device__ __forceinline__ IexpScale iexp_scale(int e) { return IexpScale{63 - e}; }

__device__ __forceinline__ double iexp_fixed_tab(unsigned long long E, IexpScale sc,
                                                 const unsigned long long* __restrict__ tab1024,
                                                 const unsigned long long* __restrict__ fine1024) {
  if (E == 0) return 1.0;
  const int K0 = sc.K0;
  if (K0 >= 192) return 1.0;                   // y < 2^-64: rounds to 1
  if (K0 < 64) return iexp_fixed(E, 63 - K0);  // outside this form's range
  const unsigned long long plo = E * IEXP_L2E64, phi = __umul64hi(E, IEXP_L2E64);
  unsigned long long yi, yf;  // y = yi + yf 2^-64
  if (K0 >= 128) {
    yi = 0ULL;
    yf = K0 == 128 ? phi : (phi >> (K0 - 128));
  } else {
    yi = phi >> (K0 - 64);
    yf = K0 == 64 ? plo : ((plo >> (K0 - 64)) | (phi << (128 - K0)));
  }
  if (yi >= 1100) return 0.0;
  const unsigned int m = (unsigned int)yi + (yf ? 1u : 0u);
  const unsigned long long f = 0ULL - yf;  // (m - y) 2^64
  const int j = (int)(f >> 54);
  const int k = (int)(f >> 44) & 1023;
  const unsigned long long s = f & 0x00000FFFFFFFFFFFULL;
  const unsigned long long t = __umul64hi(s << 20, IEXP_LN2) >> 20;  // t 2^64 < 2^43.5
  const unsigned int th = (unsigned int)(t >> 12);
  const unsigned long long eps = t + (((unsigned long long)th * th) >> 41);  // (exp(t) - 1) 2^64 < 2^44
  const unsigned long long dk = fine1024[k];                                  // (2^(k/2^20) - 1) 2^64 < 2^53.5
  const unsigned long long de = ((dk >> 22) * (eps >> 12)) >> 30;            // their product, 2^64
  const unsigned long long p = (1ULL << 63) + ((dk + eps + de) >> 1);       // 2^(k/2^20) exp(t) 2^63
  const unsigned long long Z = __umul64hi(tab1024[j], p);                   // 2^(g) 2^62
  const int top = (int)(Z >> 63);
  const int sh = 10 + top;
  const int be = 1023 + top - (int)m;
  if (be >= 1) {
    const unsigned long long mant = (Z + (1ULL << (sh - 1))) >> sh;
    return __longlong_as_double((long long)(((unsigned long long)be << 52) + mant - (1ULL << 52)));
  }
  const int tot = sh + 1 - be;
  if (tot > 64) return 0.0;
  const unsigned long long mant = (tot == 64) ? (Z >> 63) : ((Z + (1ULL << (tot - 1))) >> tot);
  return __longlong_as_double((long long)mant);
}
