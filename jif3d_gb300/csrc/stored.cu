// stored.cu -- the device-resident sensitivity matrix and its HBM-streaming
// products (the GPU counterpart of FullSensitivityGravMagCalculator's cached
// path, GravMag/FullSensitivityGravMagCalculator.h:136-221: d = J m and
// g = 2 J^T r without recomputing any box term).
//
// Storage: J with rows = station x stored component and columns = cells,
// padded to a multiple of 64 columns with zeros, as
//   FP32                       4 B per element, row-major, or
//   FP16 hi + lo, row scale    2 x 2 B per element: J[r][c] ~= s_r (hi + lo),
//                              s_r a power of two with max|J/s_r| in (2^13, 2^14],
//                              hi = fp16(J/s_r), lo = fp16(J/s_r - hi) (22
//                              significant bits), in 128 x 64 tiles (stored.h,
//                              tiled_index), plus the transposed copy used as
//                              the K-major operand of the adjoint GEMM.
// Streaming products accumulate in FP32 in short chains and in FP64 across
// chains; the tensor-core products are in gemm_tc.cu.
#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>

#include "fpbits.cuh"
#include "stored.h"

namespace j3g {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int NT>
__device__ __forceinline__ double block_sum_d(double v, double *red) {
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) r += red[w];
    red[0] = r;
  }
  __syncthreads();
  r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Power-of-two scale that brings max|v| into (2^13, 2^14]: the fp16 parts
// of v / scale stay far from overflow and mostly above the subnormal range,
// and dividing by it is exact.
__device__ __forceinline__ double pow2_scale(double maxabs) {
  if (!(maxabs > 0.0)) return 1.0;
  int e;
  frexp(maxabs, &e);  // maxabs in [2^(e-1), 2^e)
  return ldexp(1.0, e - 14);
}

__device__ __forceinline__ void split_half(double v, __half &h, __half &l) {
  h = __double2half(v);
  l = __double2half(v - (double)__half2float(h));
}

template <class T>
__device__ __forceinline__ double block_max_abs(const T &get, long long n, double *red) {
  double m = 0.0;
  for (long long c = threadIdx.x; c < n; c += kT) m = fmax(m, fabs(get(c)));
  m = warp_max_d(m);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < kT / 32; ++w) mm = fmax(mm, red[w]);
    red[0] = mm;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

// One block per row: power-of-two row scale and fp16 hi / lo split of an FP64
// row (padding columns zero).  scale[row0 + r] receives the scale and, when
// given, rowsum[row0 + r] the FP64 sum of the row (J 1, used to add back the
// mean of a centred model).
__global__ void k_split_rows(const double *__restrict__ rows, long long ld_in, long long ncol,
                             __half *__restrict__ hi, __half *__restrict__ lo, long long ld_out,
                             float *__restrict__ scale, double *__restrict__ rowsum,
                             long long row0) {
  const long long r = blockIdx.x;
  const double *p = rows + r * ld_in;
  __shared__ double red[kT / 32];
  const double sc = pow2_scale(block_max_abs([&](long long c) { return p[c]; }, ncol, red));
  if (threadIdx.x == 0) scale[row0 + r] = (float)sc;
  if (rowsum) {
    double acc = 0.0;
    for (long long c = threadIdx.x; c < ncol; c += kT) acc += p[c];
    acc = block_sum_d<kT>(acc, red);
    if (threadIdx.x == 0) rowsum[row0 + r] = acc;
  }
  const double inv = 1.0 / sc;
  for (long long c = threadIdx.x; c < ld_out; c += kT) {
    __half hv, lv;
    split_half(c < ncol ? p[c] * inv : 0.0, hv, lv);
    const long long o = tiled_index(row0 + r, c, ld_out);
    hi[o] = hv;
    lo[o] = lv;
  }
}

// 32x32 blocked transpose of a 16-bit matrix, (r, c) -> (c, r), both in the
// tiled layout (a 32-wide block never straddles a 64-column tile).
__global__ void k_transpose16(const uint16_t *__restrict__ in, long long ld_in, long long rows,
                              long long cols, uint16_t *__restrict__ out, long long ld_out) {
  __shared__ uint16_t tile[32][34];
  const long long c0 = (long long)blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  // row blocks loop over grid y (at most 65535 blocks)
  for (long long r0 = (long long)blockIdx.y * 32; r0 < ld_out; r0 += (long long)gridDim.y * 32) {
    __syncthreads();  // the previous block's tile has been written out
    for (int k = ty; k < 32; k += 8) {
      const long long r = r0 + k, c = c0 + tx;
      tile[k][tx] = (r < rows && c < cols) ? in[tiled_index(r, c, ld_in)] : (uint16_t)0;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
      const long long c = c0 + k, r = r0 + tx;
      if (c < cols && r < ld_out) out[tiled_index(c, r, ld_out)] = tile[tx][k];
    }
  }
}

// Splitting an FP64 matrix [nrow][ld_src] (the adjoint's scaled residual
// rows) into fp16 hi / lo rows [nrow_pad][ld_dst], in three grid-wide passes
// so that a few hundred long rows still fill the GPU:
//   k_row_stats     per (row, column chunk): max |v|
//   k_row_finalize  per row: power-of-two scale
//   k_split_chunks  per (row, column chunk): v / scale -> hi + lo
// Short rows go in one pass (k_split_rows_small).
// v = src[r][c] * colscale[c] (colscale optional).
constexpr int kChunk = 8192;
constexpr long long kSmallRow = 16384;  // rows up to this length split in one pass
constexpr int kBatch = 8;  // loads in flight per thread in the streaming passes
static_assert(kChunk % (kT * kBatch) == 0, "chunk must be whole load batches");
// Column chunk of a split: kChunk, or one load batch per thread (kT * kBatch)
// when the rows are few and short (residual vectors), so that the grid still
// has a few blocks per SM.
inline long long split_chunk(int nrow_pad, long long ld_dst) {
  const long long blocks = (long long)nrow_pad * ((ld_dst + kChunk - 1) / kChunk);
  return blocks >= 1024 ? kChunk : kT * kBatch;
}

__device__ __forceinline__ double scaled_val(const double *src, long long ld_src, int nrow,
                                             long long ncol, const float *colscale, long long r,
                                             long long c) {
  if (r >= nrow || c >= ncol) return 0.0;
  const double v = src[r * ld_src + c];
  return colscale ? v * (double)colscale[c] : v;
}

__global__ void k_row_stats(const double *__restrict__ src, long long ld_src, int nrow,
                            long long ncol, const float *__restrict__ colscale,
                            double *__restrict__ part_max, int nchunk, int chunk) {
  const long long r = blockIdx.y;
  const long long c0 = (long long)blockIdx.x * chunk + threadIdx.x;
  // the scale needs only the binade of max |v|: truncating the mantissa keeps
  // it, so the maximum runs in FP32 on truncated values
  float mf = 0.0f;
  for (int j0 = 0; j0 < chunk / kT; j0 += kBatch) {
    double v[kBatch];  // a batch of independent loads in flight per thread
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      v[u] = scaled_val(src, ld_src, nrow, ncol, colscale, r, c0 + (long long)(j0 + u) * kT);
#pragma unroll
    for (int u = 0; u < kBatch; ++u) mf = fmaxf(mf, fabsf(approx_f32(v[u])));
  }
  __shared__ double red[kT / 32];
  const double m = warp_max_d((double)mf);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < kT / 32; ++w) mm = fmax(mm, red[w]);
    part_max[r * nchunk + blockIdx.x] = mm;
  }
}

__global__ void k_row_finalize(int nrow_pad, int nchunk, const double *__restrict__ part_max,
                               float *__restrict__ rowscale) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrow_pad) return;
  double mx = 0.0;
  for (int k = 0; k < nchunk; ++k) mx = fmax(mx, part_max[(long long)r * nchunk + k]);
  rowscale[r] = (float)pow2_scale(mx);
}

__global__ void k_split_chunks(const double *__restrict__ src, long long ld_src, int nrow,
                               long long ncol, const float *__restrict__ colscale,
                               const float *__restrict__ rowscale, __half *__restrict__ hi,
                               __half *__restrict__ lo, long long ld_dst, int chunk) {
  const long long r = blockIdx.y;
  const long long c0 = (long long)blockIdx.x * chunk + threadIdx.x;
  const double inv = 1.0 / (double)rowscale[r];  // a power of two: exact
  for (int j0 = 0; j0 < chunk / kT; j0 += kBatch) {
    double v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      v[u] = scaled_val(src, ld_src, nrow, ncol, colscale, r, c0 + (long long)(j0 + u) * kT);
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const long long c = c0 + (long long)(j0 + u) * kT;
      if (c >= ld_dst) break;
      // v / scale (exact), then FP32: the 24-bit float keeps more than the
      // 22 bits that hi + lo carry
      const float x = (r < nrow && c < ncol) ? f64_to_f32_ftz(v[u] * inv) : 0.0f;
      const __half hv = __float2half_rn(x);
      hi[r * ld_dst + c] = hv;
      lo[r * ld_dst + c] = __float2half_rn(__fsub_rn(x, __half2float(hv)));
    }
  }
}

// Models for the forward product, split in one pass over HBM (the three
// passes above read every model twice).  Any centre is exact -- c * (J 1) is
// added back after the product; it only has to take out the bulk of a large
// uniform part -- so each row's centre is an estimate from a sample of its
// values.  The power-of-two scale only sets the fp16 exponent range (hi and
// lo keep 11 bits each at any scale that keeps them normal), so a row scale
// taken from the same sample serves every K split of the product whose
// values it bounds; a split with larger values takes its own, larger scale
// (its block splits the columns again once it has their maximum).  The
// split-sum kernel applies each split's scale (sexp) to its partial sums.
constexpr int kCentreRuns = 64;    // contiguous runs sampled per model row
constexpr int kCentreRun = 32;     // values per run
constexpr int kScaleMargin = 2;    // binades of headroom on the sampled scale
__global__ void __launch_bounds__(kT) k_model_centre(const double *__restrict__ src,
                                                     long long ld_src, int nrow, long long ncol,
                                                     double *__restrict__ centre,
                                                     int *__restrict__ eref) {
  constexpr int kPer = kCentreRuns * kCentreRun / kT;
  const int r = blockIdx.x;
  // rows of up to kCentreRuns * kCentreRun values are taken whole; longer
  // ones as kCentreRuns runs of kCentreRun values, run j from j * (ncol /
  // kCentreRuns) (inside the row: ncol / kCentreRuns >= kCentreRun).  The
  // estimates run in float on truncated values (the FP64 pipe would be the
  // slowest part of this short kernel): the centre only has to be near the
  // row's values, and the scale needs only the binade of their spread.
  const long long ns = min(ncol, (long long)kCentreRuns * kCentreRun);
  const bool whole = ncol <= (long long)kCentreRuns * kCentreRun;
  float v[kPer];
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const int i = threadIdx.x + u * kT;
    const long long c =
        whole ? i : (long long)(i / kCentreRun) * (ncol / kCentreRuns) + i % kCentreRun;
    v[u] = (r < nrow && i < ns) ? approx_f32(src[(long long)r * ld_src + c]) : 0.0f;
  }
  float s = 0.0f;
#pragma unroll
  for (int u = 0; u < kPer; ++u) s += v[u];
  __shared__ float red[kT / 32];
  __shared__ float sh_c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.0f;
    for (int w = 0; w < kT / 32; ++w) a += red[w];
    // values beyond the float range make the estimate infinite: centre 0
    // (the split takes such values in FP64)
    sh_c = (ns > 0 && isfinite(a)) ? a / (float)ns : 0.0f;
  }
  __syncthreads();
  const float c32 = sh_c;
  float mf = 0.0f;
#pragma unroll
  for (int u = 0; u < kPer; ++u)
    if (threadIdx.x + u * kT < ns) mf = fmaxf(mf, fabsf(v[u] - c32));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mf = fmaxf(mf, __shfl_down_sync(0xffffffffu, mf, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mf;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.0f;
    for (int w = 0; w < kT / 32; ++w) m = fmaxf(m, red[w]);
    centre[r] = (double)c32;
    // frexp exponent of the sampled maximum (m in [2^(E-1), 2^E), E = biased
    // exponent - 126), minus 14, plus the margin; an all-equal (or
    // subnormal) sample leaves the scale to the splits' own maxima
    const uint32_t be = (__float_as_uint(m) >> 23) & 0xffu;
    eref[r] = be ? (int)be - 126 - 14 + kScaleMargin : INT_MIN / 2;
  }
}

// v - c in float arithmetic, for a double v and a centre c = ch + cl given as
// a float pair: v = vh + vl with vh its sign, exponent and leading 20
// fraction bits (exact) and vl its low 32 fraction bits (rounded to float),
// d = (vh - ch) + (vl - cl), accurate to about 2^-23 |d| + 2^-44 |v| with no
// FP64 operation.  |v| below 2^-126 counts as zero; bad is set for |v| of
// 2^128 or more (and infinities, NaNs), which the caller takes in FP64.
__device__ __forceinline__ float centred_f32(double v, float ch, float cl, bool &bad) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const uint32_t h = (uint32_t)(b >> 32), l = (uint32_t)b;
  const uint32_t s = h & 0x80000000u, e = (h >> 20) & 0x7ffu;
  bad |= e >= 1151u;
  const bool tiny = e <= 896u;
  const float vh = __uint_as_float(tiny ? s : (s | ((e - 896u) << 23) | ((h & 0xfffffu) << 3)));
  const int pe = (int)e - 948;  // biased float exponent of 2^(e - 1075)
  const float vl = (!tiny && pe > 0)
                       ? __uint2float_rn(l) * __uint_as_float(s | ((uint32_t)pe << 23))
                       : 0.0f;
  return __fadd_rn(__fsub_rn(vh, ch), __fsub_rn(vl, cl));
}

// One block per (model row, K split), streaming: d = v - centre in float
// arithmetic (centred_f32), split at once with the row's sampled exponent
// e0 = eref[row] into hi + lo of d / 2^e0 (a float multiply by a power of
// two, exact), while the block takes max |d|.  The split's exponent is
// e = max(e0, frexp exponent of max |d| - 14) (sexp[row][split]), so
// |d| / 2^e < 2^14; where it is not e0 -- values above the row's sample --
// the block splits its columns again with e (a second read, from L2).  A
// split with a value beyond the float range or an exponent outside
// [-100, 100] is split again in FP64: d = v - centre, then one rounding of
// d / 2^e to float.  Each thread takes column pairs, kSplitBatch of them per
// batch of loads.
constexpr int kSplitThreads = 256;
constexpr int kSplitBatch = 4;
__global__ void __launch_bounds__(kSplitThreads) k_split_models(
    const double *__restrict__ src, long long ld_src, int nrow, long long ncol,
    const double *__restrict__ centre, const int *__restrict__ eref, __half *__restrict__ hi,
    __half *__restrict__ lo, long long ld_dst, long long cols_per_split, int nsp,
    int *__restrict__ sexp) {
  constexpr int NT = kSplitThreads;
  const long long r = blockIdx.y;
  const long long c0 = (long long)blockIdx.x * cols_per_split;
  const long long c1 = min(ld_dst, c0 + cols_per_split);
  const bool row_ok = r < nrow;
  const double cr = row_ok ? centre[r] : 0.0;
  const int er = row_ok ? eref[r] : INT_MIN / 2;
  const int e0 = er == INT_MIN / 2 ? 0 : er;  // the provisional exponent
  const float ch = f64_to_f32_ftz(cr), cl = f64_to_f32_ftz(cr - (double)ch);
  // columns relative to c0: this split's (jn, even) and the row's values in it
  const int jn = (int)(c1 - c0);
  const int jend = row_ok ? (int)max(0LL, min(c1, ncol) - c0) : 0;
  const double *rp = src + r * ld_src + c0;
  __half2 *hp = reinterpret_cast<__half2 *>(hi + r * ld_dst + c0);
  __half2 *lp = reinterpret_cast<__half2 *>(lo + r * ld_dst + c0);
  auto put = [&](int p, float x0, float x1) {  // column pair 2p, 2p + 1
    const __half2 hv = __floats2half2_rn(x0, x1);
    const float2 hf = __half22float2(hv);
    hp[p] = hv;
    lp[p] = __floats2half2_rn(__fsub_rn(x0, hf.x), __fsub_rn(x1, hf.y));
  };
  // float pass at a given exponent: split and store every pair, return max |d|
  auto float_pass = [&](int ex, bool &bad) {
    const float inv = __uint_as_float((uint32_t)(127 - ex) << 23);  // 2^-ex
    float m = 0.0f;
    for (int p0 = (int)threadIdx.x; 2 * p0 < jn; p0 += NT * kSplitBatch) {
      double v[2 * kSplitBatch];  // a batch of loads in flight
#pragma unroll
      for (int u = 0; u < 2 * kSplitBatch; ++u) {
        const int j = 2 * (p0 + (u >> 1) * NT) + (u & 1);
        v[u] = j < jend ? rp[j] : 0.0;
      }
#pragma unroll
      for (int k = 0; k < kSplitBatch; ++k) {
        const int p = p0 + k * NT;
        if (2 * p >= jn) break;
        const float x0 = 2 * p < jend ? centred_f32(v[2 * k], ch, cl, bad) : 0.0f;
        const float x1 = 2 * p + 1 < jend ? centred_f32(v[2 * k + 1], ch, cl, bad) : 0.0f;
        m = fmaxf(m, fmaxf(fabsf(x0), fabsf(x1)));
        put(p, x0 * inv, x1 * inv);
      }
    }
    return m;
  };
  const bool fast0 = e0 >= -100 && e0 <= 100;
  bool bad = !fast0;
  float mf = 0.0f;
  if (fast0) mf = float_pass(e0, bad);
  // the split's exponent from the binade of its largest |d|: in float, m in
  // [2^(E-1), 2^E) with E = biased exponent - 126 (rounding to float can lift
  // a maximum just below 2^E to 2^E, which only raises E); in FP64 (values
  // beyond the float range), E = biased exponent - 1022
  const bool fp64 = __syncthreads_or(bad) != 0;
  int el;
  if (!fp64) {
    const uint32_t be = (__float_as_uint(mf) >> 23) & 0xffu;
    el = be ? (int)be - 126 - 14 : INT_MIN / 2;
  } else {
    el = INT_MIN / 2;
    for (int j = (int)threadIdx.x; j < jend; j += NT) {
      const int be = (int)(((unsigned long long)__double_as_longlong(rp[j] - cr) >> 52) & 0x7ff);
      if (be) el = max(el, be - 1022 - 14);
    }
  }
  __shared__ int red[NT / 32];
  __shared__ int sh_e;
  el = __reduce_max_sync(0xffffffffu, el);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = el;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = INT_MIN / 2;
    for (int w = 0; w < NT / 32; ++w) m = max(m, red[w]);
    int e = max(er, m);
    if (e == INT_MIN / 2) e = 0;  // all zero
    sh_e = e;
    sexp[r * nsp + blockIdx.x] = e;
  }
  __syncthreads();
  const int e = sh_e;
  if (!fp64 && e == e0) return;  // the first pass stands
  if (!fp64 && e >= -100 && e <= 100) {
    bool unused = false;
    float_pass(e, unused);
  } else {
    // 2^-e as a double (split exponents of finite doubles stay within
    // -1100 .. 1040; beyond the normal range the scaling saturates)
    const double inv64 = __longlong_as_double((long long)min(2046, max(1, 1023 - e)) << 52);
    for (int p = (int)threadIdx.x; 2 * p < jn; p += NT) {
      const float x0 = 2 * p < jend ? f64_to_f32_ftz((rp[2 * p] - cr) * inv64) : 0.0f;
      const float x1 = 2 * p + 1 < jend ? f64_to_f32_ftz((rp[2 * p + 1] - cr) * inv64) : 0.0f;
      put(p, x0, x1);
    }
  }
}

// Rows without centring that a block covers alone (the scaled residuals of
// the adjoint): max |v|, the power-of-two scale and the split in one launch,
// one block per row; the row is read twice (the second time from cache).
// Same values as the statistics / split passes (a maximum is order-free).
constexpr int kSmallT = 512;  // threads per row in k_split_rows_small
__global__ void __launch_bounds__(kSmallT) k_split_rows_small(
    const double *__restrict__ src, long long ld_src, int nrow, long long ncol,
    const float *__restrict__ colscale, float *__restrict__ rowscale, __half *__restrict__ hi,
    __half *__restrict__ lo, long long ld_dst) {
  const long long r = blockIdx.x;
  float mf = 0.0f;
  for (long long c0 = threadIdx.x; c0 < ld_dst; c0 += (long long)kSmallT * kBatch) {
    double v[kBatch];  // a batch of independent loads in flight per thread
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      v[u] = scaled_val(src, ld_src, nrow, ncol, colscale, r, c0 + (long long)u * kSmallT);
#pragma unroll
    for (int u = 0; u < kBatch; ++u) mf = fmaxf(mf, fabsf(approx_f32(v[u])));
  }
  __shared__ double red[kSmallT / 32];
  __shared__ float sh_scale;
  double m = warp_max_d((double)mf);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < kSmallT / 32; ++w) mm = fmax(mm, red[w]);
    sh_scale = (float)pow2_scale(mm);
    rowscale[r] = sh_scale;
  }
  __syncthreads();
  const double inv = 1.0 / (double)sh_scale;  // a power of two: exact
  for (long long c0 = threadIdx.x; c0 < ld_dst; c0 += (long long)kSmallT * kBatch) {
    double v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      v[u] = scaled_val(src, ld_src, nrow, ncol, colscale, r, c0 + (long long)u * kSmallT);
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const long long c = c0 + (long long)u * kSmallT;
      if (c >= ld_dst) break;
      const float x = (r < nrow && c < ncol) ? f64_to_f32_ftz(fma(v[u], inv, 0.0)) : 0.0f;
      const __half hv = __float2half_rn(x);
      hi[r * ld_dst + c] = hv;
      lo[r * ld_dst + c] = __float2half_rn(__fsub_rn(x, __half2float(hv)));
    }
  }
}

__global__ void k_to_f32(const double *__restrict__ src, long long n, long long npad,
                         float *__restrict__ dst) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npad;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = t < n ? (float)src[t] : 0.0f;
}

// d[r] = sum_c J[r][c] x[c]; one block per row, float4 streaming loads,
// FP32 chains of 16 flushed into an FP64 sum.
__global__ void __launch_bounds__(kT) k_gemv_f32(const float *__restrict__ J, long long ld,
                                                 const float *__restrict__ x,
                                                 double *__restrict__ out) {
  const long long r = blockIdx.x;
  const float4 *p = reinterpret_cast<const float4 *>(J + r * ld);
  const float4 *xv = reinterpret_cast<const float4 *>(x);
  const long long n4 = ld / 4;
  double accd = 0.0;
  long long i = threadIdx.x;
  for (; i + 3 * kT < n4; i += 4 * kT) {
    float4 a0 = __ldcs(p + i), a1 = __ldcs(p + i + kT), a2 = __ldcs(p + i + 2 * kT),
           a3 = __ldcs(p + i + 3 * kT);
    float4 b0 = xv[i], b1 = xv[i + kT], b2 = xv[i + 2 * kT], b3 = xv[i + 3 * kT];
    float acc = a0.x * b0.x;
    acc = fmaf(a0.y, b0.y, acc); acc = fmaf(a0.z, b0.z, acc); acc = fmaf(a0.w, b0.w, acc);
    acc = fmaf(a1.x, b1.x, acc); acc = fmaf(a1.y, b1.y, acc); acc = fmaf(a1.z, b1.z, acc);
    acc = fmaf(a1.w, b1.w, acc); acc = fmaf(a2.x, b2.x, acc); acc = fmaf(a2.y, b2.y, acc);
    acc = fmaf(a2.z, b2.z, acc); acc = fmaf(a2.w, b2.w, acc); acc = fmaf(a3.x, b3.x, acc);
    acc = fmaf(a3.y, b3.y, acc); acc = fmaf(a3.z, b3.z, acc); acc = fmaf(a3.w, b3.w, acc);
    accd += (double)acc;
  }
  for (; i < n4; i += kT) {
    const float4 a = __ldcs(p + i), b = xv[i];
    float acc = a.x * b.x;
    acc = fmaf(a.y, b.y, acc); acc = fmaf(a.z, b.z, acc); acc = fmaf(a.w, b.w, acc);
    accd += (double)acc;
  }
  __shared__ double red[kT / 32];
  accd = block_sum_d<kT>(accd, red);
  if (threadIdx.x == 0) out[r] = accd;
}

// part[chunk][c] = sum_{r in chunk} J[r][c] w[r]; block = 1024 columns x RC rows.
// Rows go in groups of 16, summed in row order in an FP32 chain that is added
// into the FP64 column sums once per group; a group's loads are issued in
// batches of 8 float4 (128 bytes in flight per thread, four blocks per SM).
constexpr int kRC = 128;
constexpr int kRG = 16;  // rows per FP32 chain
constexpr int kRB = 8;   // rows per load batch
static_assert(kRC % kRG == 0 && kRG % kRB == 0, "chunks are whole row groups and batches");
__global__ void __launch_bounds__(kT, 4) k_gemv_t_f32(const float *__restrict__ J, long long ld,
                                                   int nrows, const double *__restrict__ w,
                                                   double *__restrict__ part) {
  const long long c4 = (long long)blockIdx.x * kT + threadIdx.x;  // float4 column index
  const bool active = c4 * 4 < ld;
  const int nchunk = (nrows + kRC - 1) / kRC;
  __shared__ float ws[kRC];
  // row chunks loop over grid y (at most 65535 blocks)
  for (int chunk = blockIdx.y; chunk < nchunk; chunk += gridDim.y) {
    const int r0 = chunk * kRC, r1 = min(nrows, r0 + kRC);
    __syncthreads();  // the previous chunk's weights are no longer read
    for (int t = threadIdx.x; t < kRC; t += kT) ws[t] = (r0 + t < r1) ? (float)w[r0 + t] : 0.0f;
    __syncthreads();
    if (!active) continue;
    double d0 = 0, d1 = 0, d2 = 0, d3 = 0;
    const float4 *col = reinterpret_cast<const float4 *>(J) + c4;
    const long long ld4 = ld / 4;
    for (int g = r0; g < r1; g += kRG) {
      float f0 = 0, f1 = 0, f2 = 0, f3 = 0;
#pragma unroll
      for (int h = 0; h < kRG; h += kRB) {
        const int nb = min(kRB, r1 - g - h);  // rows of this batch (<= 0: none)
        float4 a[kRB];
#pragma unroll
        for (int u = 0; u < kRB; ++u)
          a[u] = u < nb ? __ldcs(col + (long long)(g + h + u) * ld4)
                        : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kRB; ++u) {
          if (u < nb) {
            const float wr = ws[g - r0 + h + u];
            f0 = fmaf(a[u].x, wr, f0);
            f1 = fmaf(a[u].y, wr, f1);
            f2 = fmaf(a[u].z, wr, f2);
            f3 = fmaf(a[u].w, wr, f3);
          }
        }
      }
      d0 += f0; d1 += f1; d2 += f2; d3 += f3;
    }
    double *o = part + (long long)chunk * ld + c4 * 4;
    o[0] = d0; o[1] = d1; o[2] = d2; o[3] = d3;
  }
}

__global__ void k_sum_parts(const double *__restrict__ part, int nchunk, long long ld,
                            long long ncol, double factor, double *__restrict__ out) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  double v = 0.0;
  for (int k = 0; k < nchunk; ++k) v += part[(long long)k * ld + c];
  out[c] = factor * v;
}

// out[n][r] = factor * rowscale[r] * modscale[n] * sum_s P[s][n][r]
// (FP64 reduction of split-K partials; either scale may be absent)
// sexp (optional, [nmod][nsplit]): split s of model n carries the scale
// 2^sexp[n][s] (models split per K split, k_split_models) in place of modscale.
__global__ void k_splitk_reduce(const float *__restrict__ P, int nsplit, long long slice,
                                int nmod, int nrow, long long ldp, const float *__restrict__ rowscale,
                                const float *__restrict__ modscale, const int *__restrict__ sexp,
                                const double *__restrict__ modmean,
                                const double *__restrict__ rowsum, double factor,
                                double *__restrict__ out, long long ld_out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nmod * nrow) return;
  const int n = t / nrow, r = t % nrow;
  const float *p = P + (long long)n * ldp + r;
  const int *se = sexp ? sexp + (long long)n * nsplit : nullptr;
  auto part = [&](int s) {
    const double x = (double)p[(long long)s * slice];
    return se ? x * ldexp(1.0, se[s]) : x;
  };
  // independent partial sums keep several loads in flight
  double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
  int s = 0;
  for (; s + 3 < nsplit; s += 4) {
    v0 += part(s);
    v1 += part(s + 1);
    v2 += part(s + 2);
    v3 += part(s + 3);
  }
  for (; s < nsplit; ++s) v0 += part(s);
  double v = (v0 + v1) + (v2 + v3);
  if (rowscale) v *= (double)rowscale[r];
  if (modscale) v *= (double)modscale[n];
  if (modmean) v += modmean[n] * rowsum[r];  // the model mean removed before the product
  out[(long long)n * ld_out + r] = factor * v;
}

// The same over groups of four consecutive rows (nrow, ldp and slice
// multiples of 4, P 16-byte aligned); grid (row blocks, models), no index
// division.  A thread takes G groups kT quads apart within one model --
// consecutive threads read consecutive float4s -- and U splits at a time:
// for a few splits G = 2 quads x 2 splits (four loads per thread, twice the
// threads of four quads: 108 instead of 115 us for the 2-split adjoint of
// 256 x 131072 outputs), for many 1 quad x 4 splits with the next batch
// loading while one is added up.  The split sums accumulate as unevaluated
// FP32 pairs (hi + lo, error-free two-sum), about 48 bits -- as good as an
// FP64 sum of FP32 partials -- without the FP64 pipe.  With more than kPairSplits splits
// one FP64 add per output widens the pair; with fewer the pair is rounded to
// FP32 first (relative 2^-24, below the FP32 rounding each partial already
// carries) so that the pass stays at HBM speed: one FP64 operation per output
// costs as much as the whole memory traffic on this GPU's FP64 pipe.  The
// power-of-two scales and the factor (a power of two, 2^kfac; other factors
// take k_splitk_reduce) are exponent adds.
constexpr int kPairSplits = 4;
// G: row quads per thread (2 for a few splits; 1 for many, so that more
// threads share the splits' loads); U: splits per load batch.  The next
// batch of loads is issued before the current one is added up.
template <bool PAIR, int G>  // PAIR: widen hi + lo in FP64 (more than kPairSplits splits)
__global__ void __launch_bounds__(kT) k_splitk_reduce4(
    const float *__restrict__ P, int nsplit, long long slice, int nrow, long long ldp,
    const float *__restrict__ rowscale, const float *__restrict__ modscale,
    const int *__restrict__ sexp, const double *__restrict__ modmean,
    const double *__restrict__ rowsum, int kfac, double *__restrict__ out, long long ld_out) {
  constexpr int U = G == 1 ? 4 : 2;
  const int nq = nrow / 4;
  const int n = blockIdx.y;
  // per-split scales 2^sexp[n][s]: each split's partials are brought to the
  // largest of them in FP32 (an exponent add, exact but for contributions
  // below 2^-126 of that scale, which flush to zero; most splits of a model
  // share one scale and skip it) and that one is applied with the other
  // scales at the end
  const int *se = sexp ? sexp + (long long)n * nsplit : nullptr;
  int ebase = 0;
  if (se) {
    // one load per lane and a warp maximum (every thread of the block gets
    // here): a loop over the splits in each thread was a chain of round trips
    int e = INT_MIN;
    for (int s = threadIdx.x & 31; s < nsplit; s += 32) e = max(e, se[s]);
    ebase = __reduce_max_sync(0xffffffffu, e);
  }
  const int q0 = blockIdx.x * (kT * G) + threadIdx.x;
  const long long s4 = slice / 4;
  const float4 *p = reinterpret_cast<const float4 *>(P + (long long)n * ldp);
  float hi[G][4], lo[G][4];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int i = 0; i < 4; ++i) hi[g][i] = lo[g][i] = 0.0f;
  float4 q[G][U];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int qi = q0 + g * kT;
      q[g][u] = (qi < nq && u < nsplit) ? __ldcs(p + (long long)u * s4 + qi)
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  for (int s = 0; s < nsplit; s += U) {
    // many splits: the next batch loads while this one is added up; a few
    // splits: plain batches (the extra registers cost occupancy)
    constexpr bool kAhead = G == 1;
    float4 nx[G][U];
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int qi = q0 + g * kT;
        nx[g][u] = (kAhead && qi < nq && s + U + u < nsplit)
                       ? __ldcs(p + (long long)(s + U + u) * s4 + qi)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (s + u >= nsplit) continue;
        float x[4] = {q[g][u].x, q[g][u].y, q[g][u].z, q[g][u].w};
        if (se) {
          const int k = se[s + u] - ebase;
          if (k != 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i) x[i] = scale_f32_ftz(x[i], k);
          }
        }
        if (nsplit == 1) {
          // one split: the two-sum onto zero is x + 0 (a zero's sign made
          // positive) with no error term, bit for bit
#pragma unroll
          for (int i = 0; i < 4; ++i) hi[g][i] = __fadd_rn(x[i], 0.0f);
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float sres, err;
            two_sum(hi[g][i], x[i], sres, err);
            hi[g][i] = sres;
            lo[g][i] = __fadd_rn(lo[g][i], err);
          }
        }
      }
    if (kAhead) {
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int u = 0; u < U; ++u) q[g][u] = nx[g][u];
    } else if (s + U < nsplit) {
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int qi = q0 + g * kT;
          q[g][u] = (qi < nq && s + U + u < nsplit) ? __ldcs(p + (long long)(s + U + u) * s4 + qi)
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
  }
  const int kmod = (modscale ? pow2_exponent(modscale[n]) : 0) + ebase + kfac;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int qi = q0 + g * kT;
    if (qi >= nq) continue;
    const int r = qi * 4;
    double res[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      // a compile-time choice: as a run-time select both arms were evaluated
      const int k = kmod + (rowscale ? pow2_exponent(rowscale[r + i]) : 0);
      double v = PAIR ? scale_pow2(f32_to_f64(hi[g][i]) + f32_to_f64(lo[g][i]), k)
                      : widen_pow2(__fadd_rn(hi[g][i], lo[g][i]), k);
      if (modmean) v = fma(modmean[n], scale_pow2(rowsum[r + i], kfac), v);
      res[i] = v;
    }
    double *o = out + (long long)n * ld_out + r;
    // whole 16-byte stores where the output row allows (full sectors per warp)
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
      __stcs(reinterpret_cast<double2 *>(o), make_double2(res[0], res[1]));
      __stcs(reinterpret_cast<double2 *>(o) + 1, make_double2(res[2], res[3]));
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) o[i] = res[i];
    }
  }
}

// Per (station, model): stored-row sums -> raw data (+ background) -> transform.
// sums [nmod][ld_sums] with row s*NS + q; models [nmod][ld_models] (background
// values at column ngrid); data [nmod][ld_data]; raw_out [nmod][nmeas*raw] optional.
// KIND is a template argument so that the component arrays stay in
// registers; one thread per (station, model), a block of kAsm stations of one
// model (blockIdx.y).  Each station's values are a short record (7 sums, 10
// raw values), so the block moves its stations' records through shared
// memory: coalesced reads and writes instead of one strided access per value.
constexpr int kAsm = 128;

// count records of W doubles, src to dst, by the whole block: each thread
// issues a batch of kCopyBatch loads before it stores them, so that a copy
// from global memory costs one round trip per batch instead of one per value.
constexpr int kCopyBatch = 8;
template <int W>
__device__ __forceinline__ void copy_records(double *dst, const double *src, int count) {
  const int n = count * W, nt = blockDim.x;
  for (int i0 = threadIdx.x; i0 < n; i0 += nt * kCopyBatch) {
    double v[kCopyBatch];
#pragma unroll
    for (int u = 0; u < kCopyBatch; ++u) {
      const int i = i0 + u * nt;
      v[u] = i < n ? src[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kCopyBatch; ++u) {
      const int i = i0 + u * nt;
      if (i < n) dst[i] = v[u];
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kAsm)
k_stored_assemble(int transform, double tbx, double tby, double tbz, int nmeas,
                  const double *__restrict__ sums, long long ld_sums,
                  const double *__restrict__ bgsens, int nbg, const double *__restrict__ models,
                  long long ld_models, long long ngrid, MagField mf,
                  double *__restrict__ raw_out, double *__restrict__ data, long long ld_data) {
  constexpr int kind = KIND;
  constexpr int raw = kind_raw(kind);
  constexpr int ns = stored_rows(kind);
  __shared__ double in_rec[kAsm * ns], out_rec[kAsm * raw];
  const int s0 = blockIdx.x * kAsm, n = blockIdx.y;
  const int count = min(kAsm, nmeas - s0), t = threadIdx.x, s = s0 + t;
  copy_records<ns>(in_rec, sums + n * ld_sums + (long long)s0 * ns, count);
  __syncthreads();
  double r[10];
  if (t < count) {
    const double *sm = in_rec + t * ns;
    if constexpr (stored_is_raw(kind)) {
#pragma unroll
      for (int c = 0; c < raw; ++c) r[c] = sm[c];
    } else {
      double u[NC_COUNT];
#pragma unroll
      for (int c = 0; c < NC_COUNT; ++c) u[c] = 0.0;
#pragma unroll
      for (int q = 0; q < ns; ++q) u[slot_comp(kind, q)] = sm[q];
      raw_from_comps(kind, u, mf, r);
    }
    const double *bgval = models + n * ld_models + ngrid;
#pragma unroll
    for (int c = 0; c < raw; ++c) {
      double bg = 0.0;
      for (int j = 0; j < nbg; ++j)
        bg = add(bg, mul(bgsens[((long long)s * raw + c) * nbg + j], bgval[j]));
      r[c] = add(r[c], bg);
      out_rec[t * raw + c] = r[c];
    }
  }
  __syncthreads();
  if (raw_out)
    copy_records<raw>(raw_out + n * (long long)nmeas * raw + (long long)s0 * raw, out_rec, count);
  double *d = data + n * ld_data;
  if (transform == TR_NONE) {
    copy_records<raw>(d + (long long)s0 * raw, out_rec, count);
  } else if (t < count) {
    if (transform == TR_FTG_INVARIANT) {
      d[s] = sub(sub(sub(add(add(mul(r[0], r[4]), mul(r[4], r[8])), mul(r[0], r[8])),
                         mul(r[3], r[1])),
                     mul(r[7], r[5])),
                 mul(r[2], r[6]));
    } else if (transform == TR_TOTAL_FIELD) {
      d[s] = sqrt(add(add(mul(r[0], r[0]), mul(r[1], r[1])), mul(r[2], r[2])));
    } else {
      d[s] = add(add(mul(tbx, r[0]), mul(tby, r[1])), mul(tbz, r[2]));
    }
  }
}
// Raw-row weights of one station: the misfit back-projected through the
// transform's derivative at the station's raw data d (Gravity/GravityTransforms.h:
// 72-93, Magnetics/MagneticTransforms.h:65-75, 136-145); w = the misfit
// itself without a transform.
template <int RAW>
__device__ __forceinline__ void station_weights(int transform, double tbx, double tby,
                                                double tbz, const double *mis_raw, double m,
                                                const double *d, double *w) {
  if (transform == TR_NONE) {
#pragma unroll
    for (int c = 0; c < RAW; ++c) w[c] = mis_raw[c];
  } else if (transform == TR_FTG_INVARIANT) {
    w[0] = mul(m, add(d[4], d[8])); w[1] = mul(m, -d[3]); w[2] = mul(m, -d[6]);
    w[3] = mul(m, -d[1]); w[4] = mul(m, add(d[0], d[8])); w[5] = mul(m, -d[7]);
    w[6] = mul(m, -d[2]); w[7] = mul(m, -d[5]); w[8] = mul(m, add(d[0], d[4]));
  } else if (transform == TR_TOTAL_FIELD) {
    const double tt = sqrt(add(add(mul(d[0], d[0]), mul(d[1], d[1])), mul(d[2], d[2])));
    for (int c = 0; c < 3; ++c) w[c] = mul(m, d[c] / tt);
  } else {
    w[0] = mul(m, tbx); w[1] = mul(m, tby); w[2] = mul(m, tbz);
  }
}

// Stored-row weights of one station from its raw-row weights.
template <int KIND>
__device__ __forceinline__ void stored_weights(const double *w, const MagField &mf, double *st) {
  constexpr int kind = KIND;
  constexpr int raw = kind_raw(kind);
  constexpr int ns = stored_rows(kind);
  if constexpr (stored_is_raw(kind)) {
#pragma unroll
    for (int c = 0; c < raw; ++c) st[c] = w[c];
  } else {
    double u[NC_COUNT];
    comps_from_raw_weights(kind, w, mf, u);
#pragma unroll
    for (int q = 0; q < ns; ++q) st[q] = u[slot_comp(kind, q)];
  }
}

template <int KIND>
__global__ void __launch_bounds__(kAsm)
k_stored_weights(int transform, double tbx, double tby, double tbz, int nmeas,
                 const double *__restrict__ misfit, long long ld_misfit,
                 const double *__restrict__ rawd, MagField mf, double *__restrict__ w_raw,
                 double *__restrict__ w_st, long long ld_w) {
  constexpr int kind = KIND;
  constexpr int raw = kind_raw(kind);
  constexpr int ns = stored_rows(kind);
  __shared__ double raw_rec[kAsm * raw], st_rec[kAsm * ns];
  const int s0 = blockIdx.x * kAsm, n = blockIdx.y;
  const int count = min(kAsm, nmeas - s0), t = threadIdx.x, s = s0 + t;
  const double *mis = misfit + n * ld_misfit;
  if (transform == TR_NONE) copy_records<raw>(raw_rec, mis + (long long)s0 * raw, count);
  __syncthreads();
  if (t < count) {
    double w[10];
    const bool plain = transform == TR_NONE;
    station_weights<raw>(transform, tbx, tby, tbz, raw_rec + t * raw, plain ? 0.0 : mis[s],
                         plain ? nullptr : rawd + n * (long long)nmeas * raw + (long long)s * raw,
                         w);
#pragma unroll
    for (int c = 0; c < raw; ++c) raw_rec[t * raw + c] = w[c];
    stored_weights<kind>(w, mf, st_rec + t * ns);
  }
  __syncthreads();
  copy_records<raw>(w_raw + n * (long long)nmeas * raw + (long long)s0 * raw, raw_rec, count);
  copy_records<ns>(w_st + n * ld_w + (long long)s0 * ns, st_rec, count);
}

// The stored-row weights of one model and their fp16 split in one launch, for
// surveys of at most kWsCtas * kWsThreads stations: a cluster of kWsCtas
// CTAs per model, CTA q taking stations q * kWsThreads.. (one per thread),
// computes every station's weights (k_stored_weights' arithmetic, raw-row
// weights written to w_raw), scales them by J's row scales, takes the row's
// maximum -- each CTA's through distributed shared memory -- and splits them
// (k_split_rows_small's arithmetic): the same values as the two launches,
// without the weights' round trip through HBM.  The stations' records move
// through shared memory, so that every global access is coalesced and the
// split runs one thread per element.  Rows n >= nmod are zero padding
// (scale 1), as in the split.
constexpr int kWsCtas = 4;
constexpr int kWsThreads = 256;
template <int KIND>
__global__ void __cluster_dims__(kWsCtas, 1, 1) __launch_bounds__(kWsThreads)
k_weights_split(int transform, double tbx, double tby, double tbz, int nmeas, int nmod,
                const double *__restrict__ misfit, long long ld_misfit,
                const double *__restrict__ rawd, MagField mf, double *__restrict__ w_raw,
                const float *__restrict__ colscale, float *__restrict__ rowscale,
                __half *__restrict__ hi, __half *__restrict__ lo, long long ld_dst) {
  namespace cg = cooperative_groups;
  constexpr int kind = KIND;
  constexpr int raw = kind_raw(kind);
  constexpr int ns = stored_rows(kind);
  // the records (misfits, then raw-row weights), then the scaled stored
  // weights in the same space, and J's row scales loaded where they are used:
  // one 20 KB array instead of two (35 KB) and 32 registers instead of 42 fit
  // eight CTAs to an SM instead of five, so that a launch's 1024 CTAs run in
  // one round instead of two
  static_assert(ns <= raw, "the stored weights reuse the records' space");
  __shared__ double rec[kWsThreads * raw];
  double *stw = rec;
  __shared__ float red[kWsThreads / 32];
  __shared__ float cta_max;
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank(), n = blockIdx.x / kWsCtas, t = threadIdx.x;
  const int s0 = q * kWsThreads, count = max(0, min(kWsThreads, nmeas - s0)), s = s0 + t;
  const bool live = n < nmod;
  const bool plain = transform == TR_NONE;
  const double *mis = misfit + (long long)n * ld_misfit;
  float mf32 = 0.0f;
  if (plain) {
    // the misfits are the raw-row weights
    if (live) copy_records<raw>(rec, mis + (long long)s0 * raw, count);
  } else if (live && t < count) {
    double w[10];
    station_weights<raw>(transform, tbx, tby, tbz, nullptr, mis[s],
                         rawd + (long long)n * nmeas * raw + (long long)s * raw, w);
#pragma unroll
    for (int c = 0; c < raw; ++c) rec[t * raw + c] = w[c];
  }
  __syncthreads();  // the raw-row weights of every station are in
  if (live) copy_records<raw>(w_raw + (long long)n * nmeas * raw + (long long)s0 * raw, rec, count);
  double xs[ns];
  if (live && t < count) {
    double v[ns];
    stored_weights<kind>(rec + t * raw, mf, v);
#pragma unroll
    for (int k = 0; k < ns; ++k) {
      // times J's row scale, a power of two: an exponent add
      xs[k] = scale_pow2_ftz(v[k], pow2_exponent(colscale[(long long)s * ns + k]));
      mf32 = fmaxf(mf32, fabsf(approx_f32(xs[k])));
    }
  }
  __syncthreads();  // every record is read: the space takes the stored weights
  if (live && t < count) {
#pragma unroll
    for (int k = 0; k < ns; ++k) stw[t * ns + k] = xs[k];
  }
  // the maxima in float (the truncated values are floats; an FP64 maximum
  // would only load the FP64 pipe)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mf32 = fmaxf(mf32, __shfl_down_sync(0xffffffffu, mf32, o));
  if ((t & 31) == 0) red[t >> 5] = mf32;
  __syncthreads();  // the stored weights and the warps' maxima are in
  if (t == 0) {
    float mm = 0.0f;
    for (int w = 0; w < kWsThreads / 32; ++w) mm = fmaxf(mm, red[w]);
    cta_max = mm;
  }
  cluster.sync();  // every CTA's maximum is in
  float mm = 0.0f;
  for (int r = 0; r < kWsCtas; ++r) mm = fmaxf(mm, *cluster.map_shared_rank(&cta_max, r));
  __shared__ float sh_scale;
  if (t == 0) sh_scale = (float)pow2_scale((double)mm);
  __syncthreads();
  const float scale = sh_scale;
  if (q == 0 && t == 0) rowscale[n] = scale;
  const int kinv = -pow2_exponent(scale);  // dividing by the scale: an exponent add
  __half *h = hi + (long long)n * ld_dst + (long long)s0 * ns;
  __half *l = lo + (long long)n * ld_dst + (long long)s0 * ns;
  for (int i = t; i < count * ns; i += kWsThreads) {
    const float x = live ? f64_to_f32_ftz(scale_pow2_ftz(stw[i], kinv)) : 0.0f;
    const __half hv = __float2half_rn(x);
    h[i] = hv;
    l[i] = __float2half_rn(__fsub_rn(x, __half2float(hv)));
  }
  if (q == kWsCtas - 1) {  // padding columns
    __half *hr = hi + (long long)n * ld_dst, *lr = lo + (long long)n * ld_dst;
    for (long long c = (long long)nmeas * ns + t; c < ld_dst; c += kWsThreads) {
      hr[c] = __float2half_rn(0.0f);
      lr[c] = __float2half_rn(0.0f);
    }
  }
  cluster.sync();  // no CTA leaves while another may read its maximum
}

// grads[n][ngrid + j] = 2 sum_s sum_r w_raw[n][s][r] bgsens[s][r][j]; block (j, n)
__global__ void k_bg_grad_batched(int raw, int nmeas, int nbg, const double *__restrict__ w_raw,
                                  const double *__restrict__ bgsens, double *__restrict__ grads,
                                  long long ld_grads, long long ngrid) {
  const int j = blockIdx.x, n = blockIdx.y;
  const double *w = w_raw + n * (long long)nmeas * raw;
  double acc = 0.0;
  for (int s = threadIdx.x; s < nmeas; s += kT)
    for (int r = 0; r < raw; ++r)
      acc = fma(w[(long long)s * raw + r], bgsens[((long long)s * raw + r) * nbg + j], acc);
  __shared__ double red[kT / 32];
  acc = block_sum_d<kT>(acc, red);
  if (threadIdx.x == 0) grads[n * ld_grads + ngrid + j] = 2.0 * acc;
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }
inline int grid_for(long long n) {
  long long b = (n + kT - 1) / kT;
  return (int)(b > 152 * 64 ? 152 * 64 : (b < 1 ? 1 : b));
}

}  // namespace

cudaError_t launch_split_rows(const double *rows, long long ld_in, long long ncol, int nrows,
                              void *hi, void *lo, long long ld_out, float *scale, double *rowsum,
                              long long row0, cudaStream_t st) {
  if (nrows == 0) return cudaSuccess;
  k_split_rows<<<nrows, kT, 0, st>>>(rows, ld_in, ncol, static_cast<__half *>(hi),
                                     static_cast<__half *>(lo), ld_out, scale, rowsum, row0);
  return cudaGetLastError();
}

cudaError_t launch_transpose16(const void *in, long long ld_in, long long rows, long long cols,
                               void *out, long long ld_out, cudaStream_t st) {
  dim3 grid(cdiv(cols, 32), std::min(cdiv(ld_out, 32), 65535));
  k_transpose16<<<grid, 256, 0, st>>>(static_cast<const uint16_t *>(in), ld_in, rows, cols,
                                      static_cast<uint16_t *>(out), ld_out);
  return cudaGetLastError();
}

int split_matrix_launches(long long ld_dst) { return ld_dst <= kSmallRow ? 1 : 3; }

long long split_matrix_work(int nrow_pad, long long ld_dst) {
  const long long chunk = split_chunk(nrow_pad, ld_dst);
  return (long long)nrow_pad * ((ld_dst + chunk - 1) / chunk);
}

cudaError_t launch_split_matrix(const double *src, long long ld_src, int nrow, long long ncol,
                                const float *colscale, void *hi, void *lo, long long ld_dst,
                                int nrow_pad, float *rowscale, double *work, cudaStream_t st) {
  if (nrow_pad == 0) return cudaSuccess;
  const int chunk = (int)split_chunk(nrow_pad, ld_dst);
  const int nchunk = cdiv(ld_dst, chunk);
  if (ld_dst <= kSmallRow) {
    k_split_rows_small<<<nrow_pad, kSmallT, 0, st>>>(src, ld_src, nrow, ncol, colscale, rowscale,
                                                static_cast<__half *>(hi),
                                                static_cast<__half *>(lo), ld_dst);
    return cudaGetLastError();
  }
  dim3 grid(nchunk, nrow_pad);
  k_row_stats<<<grid, kT, 0, st>>>(src, ld_src, nrow, ncol, colscale, work, nchunk, chunk);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_row_finalize<<<cdiv(nrow_pad, 128), 128, 0, st>>>(nrow_pad, nchunk, work, rowscale);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_split_chunks<<<grid, kT, 0, st>>>(src, ld_src, nrow, ncol, colscale, rowscale,
                                      static_cast<__half *>(hi), static_cast<__half *>(lo),
                                      ld_dst, chunk);
  return cudaGetLastError();
}

cudaError_t launch_split_models(const double *src, long long ld_src, int nrow, long long ncol,
                                void *hi, void *lo, long long ld_dst, int nrow_pad,
                                long long cols_per_split, int nsp, double *centre, int *sexp,
                                cudaStream_t st) {
  if (nrow_pad == 0) return cudaSuccess;
  if (nrow_pad > 65535 || cols_per_split <= 0 || (long long)nsp * cols_per_split < ld_dst)
    return cudaErrorInvalidValue;
  int *eref = sexp + (long long)nrow_pad * nsp;  // the sampled row exponents
  k_model_centre<<<nrow_pad, kT, 0, st>>>(src, ld_src, nrow, ncol, centre, eref);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 grid(nsp, nrow_pad);
  __half *h = static_cast<__half *>(hi), *l = static_cast<__half *>(lo);
  k_split_models<<<grid, kSplitThreads, 0, st>>>(src, ld_src, nrow, ncol, centre, eref, h, l,
                                                  ld_dst, cols_per_split, nsp, sexp);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(const double *src, long long n, long long npad, float *dst,
                          cudaStream_t st) {
  k_to_f32<<<grid_for(npad), kT, 0, st>>>(src, n, npad, dst);
  return cudaGetLastError();
}

cudaError_t launch_gemv_f32(const float *J, long long ld, int nrows, const float *x, double *out,
                            cudaStream_t st) {
  if (nrows == 0) return cudaSuccess;
  k_gemv_f32<<<nrows, kT, 0, st>>>(J, ld, x, out);
  return cudaGetLastError();
}

int gemv_t_chunks(int nrows) { return cdiv(nrows, kRC); }

cudaError_t launch_gemv_t_f32(const float *J, long long ld, int nrows, const double *w,
                              double *part, long long ncol, double factor, double *out,
                              cudaStream_t st) {
  const int nchunk = gemv_t_chunks(nrows);
  dim3 grid(cdiv(ld / 4, kT), std::min(nchunk, 65535));
  k_gemv_t_f32<<<grid, kT, 0, st>>>(J, ld, nrows, w, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_sum_parts<<<cdiv(ncol, kT), kT, 0, st>>>(part, nchunk, ld, ncol, factor, out);
  return cudaGetLastError();
}

cudaError_t launch_splitk_reduce(const float *P, int nsplit, long long slice, int nmod, int nrow,
                                 long long ldp, const float *rowscale, const float *modscale,
                                 const int *sexp, const double *modmean, const double *rowsum,
                                 double factor, double *out, long long ld_out, cudaStream_t st) {
  const long long n = (long long)nmod * nrow;
  if (n == 0) return cudaSuccess;
  int kf = 0;
  const bool fpow2 = factor != 0.0 && std::frexp(factor, &kf) == 0.5;  // factor = 2^(kf-1)
  if (fpow2 && nrow % 4 == 0 && ldp % 4 == 0 && slice % 4 == 0 && nmod <= 65535 &&
      (reinterpret_cast<uintptr_t>(P) & 15) == 0) {
    if (nsplit > kPairSplits) {  // many splits: one quad per thread, 4 splits per batch
      dim3 grid(cdiv(nrow / 4, (long long)kT), nmod);
      k_splitk_reduce4<true, 1><<<grid, kT, 0, st>>>(P, nsplit, slice, nrow, ldp, rowscale,
                                                     modscale, sexp, modmean, rowsum, kf - 1,
                                                     out, ld_out);
    } else {
      dim3 grid(cdiv(nrow / 4, (long long)kT * 2), nmod);
      k_splitk_reduce4<false, 2><<<grid, kT, 0, st>>>(P, nsplit, slice, nrow, ldp, rowscale,
                                                      modscale, sexp, modmean, rowsum, kf - 1,
                                                      out, ld_out);
    }
    return cudaGetLastError();
  }
  k_splitk_reduce<<<cdiv(n, kT), kT, 0, st>>>(P, nsplit, slice, nmod, nrow, ldp, rowscale,
                                               modscale, sexp, modmean, rowsum, factor, out,
                                               ld_out);
  return cudaGetLastError();
}

cudaError_t launch_stored_assemble(int kind, int transform, double tbx, double tby, double tbz,
                                   int nmeas, int nmod, const double *sums, long long ld_sums,
                                   const double *bgsens, int nbg, const double *models,
                                   long long ld_models, long long ngrid, const MagField &mf,
                                   double *raw_out, double *data, long long ld_data,
                                   cudaStream_t st) {
  if ((long long)nmeas * nmod == 0) return cudaSuccess;
  const dim3 grid(cdiv(nmeas, kAsm), nmod);
#define J3G_ASSEMBLE(K)                                                                       \
  k_stored_assemble<K><<<grid, kAsm, 0, st>>>(transform, tbx, tby, tbz, nmeas, sums, ld_sums,  \
                                             bgsens, nbg, models, ld_models, ngrid, mf,        \
                                             raw_out, data, ld_data)
  switch (kind) {
    case KIND_SCALAR: J3G_ASSEMBLE(KIND_SCALAR); break;
    case KIND_TENSOR: J3G_ASSEMBLE(KIND_TENSOR); break;
    case KIND_MAGNETIC: J3G_ASSEMBLE(KIND_MAGNETIC); break;
    case KIND_JOINT: J3G_ASSEMBLE(KIND_JOINT); break;
    case KIND_MAG_GRADIENT: J3G_ASSEMBLE(KIND_MAG_GRADIENT); break;
    case KIND_MAGNETIZATION: J3G_ASSEMBLE(KIND_MAGNETIZATION); break;
    default: return cudaErrorInvalidValue;
  }
#undef J3G_ASSEMBLE
  return cudaGetLastError();
}

cudaError_t launch_stored_weights(int kind, int transform, double tbx, double tby, double tbz,
                                  int nmeas, int nmod, const double *misfit, long long ld_misfit,
                                  const double *rawd, const MagField &mf, double *w_raw,
                                  double *w_st, long long ld_w, cudaStream_t st) {
  if ((long long)nmeas * nmod == 0) return cudaSuccess;
  const dim3 grid(cdiv(nmeas, kAsm), nmod);
#define J3G_WEIGHTS(K)                                                                         \
  k_stored_weights<K><<<grid, kAsm, 0, st>>>(transform, tbx, tby, tbz, nmeas, misfit, ld_misfit, \
                                            rawd, mf, w_raw, w_st, ld_w)
  switch (kind) {
    case KIND_SCALAR: J3G_WEIGHTS(KIND_SCALAR); break;
    case KIND_TENSOR: J3G_WEIGHTS(KIND_TENSOR); break;
    case KIND_MAGNETIC: J3G_WEIGHTS(KIND_MAGNETIC); break;
    case KIND_JOINT: J3G_WEIGHTS(KIND_JOINT); break;
    case KIND_MAG_GRADIENT: J3G_WEIGHTS(KIND_MAG_GRADIENT); break;
    case KIND_MAGNETIZATION: J3G_WEIGHTS(KIND_MAGNETIZATION); break;
    default: return cudaErrorInvalidValue;
  }
#undef J3G_WEIGHTS
  return cudaGetLastError();
}

bool weights_split_fits(int nmeas, long long ld_dst, int nrow_pad) {
  return nmeas <= kWsThreads * kWsCtas && ld_dst <= kSmallRow && nrow_pad >= 1;
}

cudaError_t launch_weights_split(int kind, int transform, double tbx, double tby, double tbz,
                                 int nmeas, int nmod, int nrow_pad, const double *misfit,
                                 long long ld_misfit, const double *rawd, const MagField &mf,
                                 double *w_raw, const float *colscale, float *rowscale, void *hi,
                                 void *lo, long long ld_dst, cudaStream_t st) {
  if (!weights_split_fits(nmeas, ld_dst, nrow_pad)) return cudaErrorInvalidValue;
  if ((long long)nmeas * stored_rows(kind) > ld_dst) return cudaErrorInvalidValue;
#define J3G_WS(K)                                                                             \
  k_weights_split<K><<<nrow_pad * kWsCtas, kWsThreads, 0, st>>>(                              \
      transform, tbx, tby, tbz, nmeas, nmod, misfit, ld_misfit, rawd, mf, w_raw, colscale,     \
      rowscale, static_cast<__half *>(hi), static_cast<__half *>(lo), ld_dst)
  switch (kind) {
    case KIND_SCALAR: J3G_WS(KIND_SCALAR); break;
    case KIND_TENSOR: J3G_WS(KIND_TENSOR); break;
    case KIND_MAGNETIC: J3G_WS(KIND_MAGNETIC); break;
    case KIND_JOINT: J3G_WS(KIND_JOINT); break;
    case KIND_MAG_GRADIENT: J3G_WS(KIND_MAG_GRADIENT); break;
    case KIND_MAGNETIZATION: J3G_WS(KIND_MAGNETIZATION); break;
    default: return cudaErrorInvalidValue;
  }
#undef J3G_WS
  return cudaGetLastError();
}

cudaError_t launch_bg_grad_batched(int raw, int nmeas, int nbg, int nmod, const double *w_raw,
                                   const double *bgsens, double *grads, long long ld_grads,
                                   long long ngrid, cudaStream_t st) {
  if (nbg == 0 || nmod == 0) return cudaSuccess;
  k_bg_grad_batched<<<dim3(nbg, nmod), kT, 0, st>>>(raw, nmeas, nbg, w_raw, bgsens, grads,
                                                     ld_grads, ngrid);
  return cudaGetLastError();
}

}  // namespace j3g
