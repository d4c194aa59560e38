// fpbits.cuh -- FP64 <-> FP32 conversions and power-of-two scaling by
// integer bit operations, and an error-free FP32 two-sum.
//
// The FP64 pipe of the GB300 retires about two operations per clock per SM,
// so one FP64 conversion per element caps a streaming pass far below HBM
// speed; these IEEE-754 widenings / narrowings run on the integer pipes.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace j3g {

// v truncated to a float (20 of its mantissa bits), for magnitude and mean
// estimates only: |v| below the float normal range gives a signed zero,
// beyond it the largest float; infinities and NaNs keep their class.
__device__ __forceinline__ float approx_f32(double v) {
  const uint32_t h = (uint32_t)((unsigned long long)__double_as_longlong(v) >> 32);
  const uint32_t s = h & 0x80000000u, e = (h >> 20) & 0x7ffu, m = h & 0xfffffu;
  if (e == 0x7ffu) return __uint_as_float(s | 0x7f800000u | (m ? 0x400000u : 0u));
  if (e <= 896u) return __uint_as_float(s);
  if (e >= 1151u) return __uint_as_float(s | 0x7f7fffffu);
  return __uint_as_float(s | ((e - 896u) << 23) | (m << 3));
}

// v rounded to the nearest float (ties to even) for |v| below 2^128; values
// below 2^-126 in magnitude become a signed zero (they are far below what
// the fp16 hi / lo split of a scaled row keeps).  Larger finite values give
// the largest float, infinities and NaNs keep their class.
__device__ __forceinline__ float f64_to_f32_ftz(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const uint32_t s = (uint32_t)(b >> 32) & 0x80000000u;
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e == 0x7ffu)
    return __uint_as_float(s | 0x7f800000u | ((b & 0xfffffffffffffull) ? 0x400000u : 0u));
  if (e <= 896u) return __uint_as_float(s);
  unsigned long long m = b & 0xfffffffffffffull;
  // round the 52-bit mantissa to 23 bits, ties to even; a carry out of the
  // mantissa bumps the exponent (the mantissa then reads zero)
  m += 0xfffffffull + ((m >> 29) & 1ull);
  const uint32_t e2 = e + (uint32_t)(m >> 52);
  if (e2 >= 1151u) return __uint_as_float(s | 0x7f7fffffu);
  return __uint_as_float(s | ((e2 - 896u) << 23) | (uint32_t)((m >> 29) & 0x7fffffu));
}

// Exact widening of a float (including subnormals) to a double.
__device__ __forceinline__ double f32_to_f64(float f) {
  const uint32_t u = __float_as_uint(f);
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0xffu)
    return __longlong_as_double((long long)(s | 0x7ff0000000000000ull |
                                            ((unsigned long long)m << 29)));
  if (e == 0u) {
    if (m == 0u) return __longlong_as_double((long long)s);
    const int sh = __clz(m) - 8;  // bring the leading one to bit 23
    m = (m << sh) & 0x7fffffu;
    e = 1u - (uint32_t)sh;  // biased float exponent of the normalised value
    return __longlong_as_double(
        (long long)(s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29)));
  }
  return __longlong_as_double(
      (long long)(s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29)));
}

// d * 2^k by FP64 multiplies: the rare cases of scale_pow2, out of line so
// that the compiler cannot evaluate them for every element (a select of both
// arms would put FP64 work on every element, and the FP64 pipe retires about
// two operations per clock per SM).
static __device__ __noinline__ double scale_pow2_mul(double d, int k) {
  return d * ldexp(1.0, k);
}

// d * 2^k for a normal d whose result stays normal, by an exponent add;
// zeros pass through; other cases (subnormal, out of range) multiply.
__device__ __forceinline__ double scale_pow2(double d, int k) {
  const long long b = __double_as_longlong(d);
  if ((b & 0x7fffffffffffffffLL) == 0) return d;
  const int e = (int)((b >> 52) & 0x7ff);
  if (e > 0 && e < 0x7ff && e + k > 0 && e + k < 0x7ff)
    return __longlong_as_double(b + ((long long)k << 52));
  return scale_pow2_mul(d, k);
}

// scale_pow2(f32_to_f64(f), k), bit for bit: a normal float whose scaled
// double stays normal takes one exponent rebias (a few integer operations);
// zeros, subnormals, infinities, NaNs and out-of-range results take the
// general path.
__device__ __forceinline__ double widen_pow2(float f, int k) {
  const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xffu;
  const int eb = (int)e + 896 + k;  // biased exponent of the result
  if (e - 1u < 254u && eb > 0 && eb < 0x7ff)
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            ((unsigned long long)eb << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
  return scale_pow2(f32_to_f64(f), k);
}

// d * 2^k by an exponent add, branch-free: exact while the result stays a
// normal double (then bit for bit d * 2^k); results below the normal range
// and subnormal d become a signed zero, results above it a signed infinity;
// infinities and NaNs pass through.
__device__ __forceinline__ double scale_pow2_ftz(double d, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned long long s = b & 0x8000000000000000ull;
  const int e = (int)((b >> 52) & 0x7ff), ek = e + k;
  const unsigned long long scaled =
      ek <= 0 ? s : (ek >= 0x7ff ? (s | 0x7ff0000000000000ull) : b + ((unsigned long long)(long long)k << 52));
  return __longlong_as_double((long long)(e == 0x7ff ? b : (e == 0 ? s : scaled)));
}

// f * 2^k by an exponent add, branch-free: exact while the result stays a
// normal float; results below the normal range and subnormal f become a
// signed zero, results above it a signed infinity; infinities and NaNs pass
// through.
__device__ __forceinline__ float scale_f32_ftz(float f, int k) {
  const uint32_t u = __float_as_uint(f), s = u & 0x80000000u;
  const int e = (int)((u >> 23) & 0xffu), ek = e + k;
  const uint32_t scaled = ek <= 0 ? s : (ek >= 0xff ? (s | 0x7f800000u) : u + ((uint32_t)k << 23));
  return __uint_as_float(e == 0xff ? u : (e == 0 ? s : scaled));
}

// Exponent k of a power-of-two float 2^k (normal range).
__device__ __forceinline__ int pow2_exponent(float p) {
  return (int)((__float_as_uint(p) >> 23) & 0xffu) - 127;
}

// Error-free FP32 sum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

}  // namespace j3g
