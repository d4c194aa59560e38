// fp64_math.cuh -- FP64 natural logarithm and two-argument arctangent with
// few FP64 operations, for kernels bound by the GB300's narrow FP64 pipe.
//
// Exponent / mantissa splits, breakpoint indices, the reciprocal seed and
// the final sign are integer or FP32 work; only the arithmetic that needs 53
// bits runs in FP64:
//   flog    -- P. T. P. Tang's table-driven logarithm (ACM TOMS 16(4), 1990):
//              x = 2^k m, m near F_j = 1 + j/128, u = (m - F_j)/F_j,
//              log x = k ln2 + log F_j + log1p(u), log1p by its Taylor series
//              to u^7 (|u| <= 2^-8); 13 FP64 operations.
//   fatan2  -- t = min(|y|,|x|) / max(|y|,|x|) from an FP32 reciprocal seed
//              and one Newton step, atan t from the Taylor series of atan
//              about the nearest breakpoint c_j = j/64 (degree 8,
//              |t - c_j| <= 1/128), then the octant: pi/2 - atan t when
//              |y| > |x|, pi - that when x is negative, the sign of y;
//              about 20 FP64 operations; fatan2_pair gives atan2(y, x) and
//              atan2(x, y) from one ratio and series.
// Both are within about one unit in the last place of the exact value; the
// tables come from gen_fp64_tables.py.  Zeros are handled in the fast path of
// fatan2 with IEEE's signed results; subnormal, infinite and NaN operands
// (and non-positive ones for flog) take CUDA's log / atan2.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "fp64_tables.h"
#include "fpbits.cuh"

namespace j3g {

// k (|k| < 2^11) as a double, by integer operations.
__device__ __forceinline__ double small_int_to_f64(int k) {
  if (k == 0) return 0.0;
  const unsigned long long s = k < 0 ? 0x8000000000000000ull : 0ull;
  const uint32_t a = (uint32_t)(k < 0 ? -k : k);
  const int p = 31 - __clz(a);
  const unsigned long long mant = ((unsigned long long)a << (52 - p)) & 0xfffffffffffffull;
  return __longlong_as_double((long long)(s | ((unsigned long long)(1023 + p) << 52) | mant));
}

__device__ __forceinline__ double flog(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52);  // with the sign bit: positive normals are 1..0x7fe
  if (e - 1u >= 0x7feu) return log(x);
  const unsigned long long mant = b & 0xfffffffffffffull;
  const uint32_t j = (uint32_t)((mant + (1ull << 44)) >> 45);  // nearest 1/128: 0..128
  const double m = __longlong_as_double((long long)(mant | 0x3ff0000000000000ull));
  const double F = __longlong_as_double(
      (long long)(((unsigned long long)(1023u + (j >> 7)) << 52) |
                  ((unsigned long long)(j & 127u) << 45)));
  const double *row = fp64tab::kLogTable[j];
  const double f = __dsub_rn(m, F);  // exact: m and F are within 1/256
  const double u = __dmul_rn(f, __ldg(row));
  // log1p(u) = u + u^2 (-1/2 + u/3 - u^2/4 + u^3/5 - u^4/6 + u^5/7)
  double q = __fma_rn(u, 1.0 / 7.0, -1.0 / 6.0);
  q = __fma_rn(u, q, 0.2);
  q = __fma_rn(u, q, -0.25);
  q = __fma_rn(u, q, 1.0 / 3.0);
  q = __fma_rn(u, q, -0.5);
  const double kd = small_int_to_f64((int)e - 1023);
  // k ln2_lead + lead(log F_j) is exact (both are multiples of 2^-42)
  const double hi = __fma_rn(kd, fp64tab::kLn2Lead, __ldg(row + 1));
  double lo = __fma_rn(kd, fp64tab::kLn2Trail, __ldg(row + 2));
  lo = __fma_rn(__dmul_rn(u, u), q, lo);  // + u^2 q, rounded once
  lo = __dadd_rn(lo, u);
  return __dadd_rn(hi, lo);
}

// atan t for t = min(a, b) / max(a, b), a and b the magnitude bits of the
// operands; false if the operands need CUDA's atan2 (subnormal, infinite,
// NaN, or a ratio below 2^-1000).
__device__ __forceinline__ bool atan_ratio(unsigned long long ay, unsigned long long ax,
                                           double &ta) {
  const uint32_t ey = (uint32_t)(ay >> 52), ex = (uint32_t)(ax >> 52);
  if (!((ay == 0 || ey - 1u < 0x7feu) && (ax == 0 || ex - 1u < 0x7feu))) return false;
  const bool swap = ay > ax;  // magnitudes compare as integers
  const unsigned long long bnum = swap ? ax : ay, bden = swap ? ay : ax;
  double t = 0.0;
  if (bnum != 0) {
    const uint32_t en = (uint32_t)(bnum >> 52), ed = (uint32_t)(bden >> 52);
    if (ed - en > 1000u) return false;
    // num and den scaled by one power of two so that den is in [1, 2)
    const long long sh = (long long)(1023 - (int)ed) << 52;
    const double num = __longlong_as_double((long long)bnum + sh);
    const double den = __longlong_as_double((long long)bden + sh);
    const double r0 = f32_to_f64(__frcp_rn(f64_to_f32_ftz(den)));
    const double r1 = __fma_rn(r0, __fma_rn(-den, r0, 1.0), r0);
    const double t0 = __dmul_rn(num, r1);
    t = __fma_rn(__fma_rn(-den, t0, num), r1, t0);
  }
  // nearest breakpoint c_j = j/64 and d = t - c_j (exact)
  const int j = __float2int_rn(__fmul_rn(f64_to_f32_ftz(t), 64.0f));
  const double c =
      j == 0 ? 0.0 : __longlong_as_double(__double_as_longlong(small_int_to_f64(j)) -
                                          (6ll << 52));
  const double d = __dsub_rn(t, c);
  const double *a = fp64tab::kAtanTable[j];
  double p = __ldg(a + 9);
#pragma unroll
  for (int n = 8; n >= 2; --n) p = __fma_rn(p, d, __ldg(a + n));
  ta = __dadd_rn(__ldg(a), __fma_rn(d, p, __ldg(a + 1)));
  return true;
}

// The angle of (x, y) from atan t: pi/2 - atan t when |y| > |x|, pi minus
// that when x is negative (sign bit), with the sign of y.
__device__ __forceinline__ double atan2_octant(double ta, bool swap, unsigned long long bx,
                                               unsigned long long by) {
  double th = swap ? __dadd_rn(fp64tab::kPio2Hi, __fma_rn(-1.0, ta, fp64tab::kPio2Lo)) : ta;
  if (bx >> 63) th = __dadd_rn(fp64tab::kPiHi, __fma_rn(-1.0, th, fp64tab::kPiLo));
  return __longlong_as_double(__double_as_longlong(th) | (long long)(by & 0x8000000000000000ull));
}

__device__ __forceinline__ double fatan2(double y, double x) {
  const unsigned long long by = (unsigned long long)__double_as_longlong(y);
  const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
  const unsigned long long ay = by & 0x7fffffffffffffffull, ax = bx & 0x7fffffffffffffffull;
  double ta;
  if (!atan_ratio(ay, ax, ta)) return atan2(y, x);
  return atan2_octant(ta, ay > ax, bx, by);
}

// fatan2(y, x) and fatan2(x, y) with one shared ratio and series: the two
// angles need the same t = min/max (bit for bit the two separate calls).
__device__ __forceinline__ void fatan2_pair(double y, double x, double &yx, double &xy) {
  const unsigned long long by = (unsigned long long)__double_as_longlong(y);
  const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
  const unsigned long long ay = by & 0x7fffffffffffffffull, ax = bx & 0x7fffffffffffffffull;
  double ta;
  if (!atan_ratio(ay, ax, ta)) {
    yx = atan2(y, x);
    xy = atan2(x, y);
    return;
  }
  yx = atan2_octant(ta, ay > ax, bx, by);
  xy = atan2_octant(ta, ax > ay, by, bx);
}

}  // namespace j3g
