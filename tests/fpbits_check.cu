// Device check of the integer-pipe FP64 <-> FP32 conversions (fpbits.cuh)
// against CUDA's own conversions.  Built and run by tests/test_gpu_fpbits.py;
// prints one line "name mismatches tested" per check.
#include <cstdio>
#include <cuda_runtime.h>

#include "fpbits.cuh"

using namespace j3g;

__device__ unsigned long long mix64(unsigned long long x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// every float bit pattern: exact widening (NaNs only need to stay NaN)
__global__ void k_widen(unsigned long long *bad) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       i < (1ull << 32); i += stride) {
    const float f = __uint_as_float((uint32_t)i);
    const double got = f32_to_f64(f), want = (double)f;
    if (f != f) {
      nb += !(got != got);
    } else {
      nb += __double_as_longlong(got) != __double_as_longlong(want);
    }
  }
  atomicAdd(bad, nb);
}

// random doubles over the whole float exponent range, half of them built as
// exact ties of the 23-bit rounding; compared where CUDA's result is a
// normal float (the integer form flushes below 2^-126 and saturates above)
__global__ void k_narrow(unsigned long long n, unsigned long long *bad,
                         unsigned long long *tested) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb = 0, nt = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    const unsigned long long r = mix64(i);
    unsigned long long m = r & 0xfffffffffffffull;
    if (i & 1) m = (m & ~0x1fffffffull) | 0x10000000ull;  // a tie
    if ((i & 7) == 2) m = 0xfffffffffffffull;            // carry into the exponent
    const unsigned long long e = 880 + (mix64(r) % 290);  // 2^-143 .. 2^146
    const double v = __longlong_as_double((long long)(((r >> 63) << 63) | (e << 52) | m));
    const float want = __double2float_rn(v);
    const float got = f64_to_f32_ftz(v);
    if (fabs(v) < 1.1754943508222875e-38) {  // below 2^-126: a signed zero
      ++nt;
      nb += __float_as_uint(got) != ((uint32_t)(r >> 63) << 31);
    } else if (fabsf(want) <= 3.40282347e38f) {  // CUDA's result finite
      ++nt;
      nb += __float_as_uint(got) != __float_as_uint(want);
    }
  }
  atomicAdd(bad, nb);
  atomicAdd(tested, nt);
}

// truncation estimate: same sign and binade, |error| < 2^-20 |v|; power-of-two
// scaling against a multiply; two-sum exact in FP64
__global__ void k_misc(unsigned long long n, unsigned long long *bad) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb[3] = {0, 0, 0};
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    const unsigned long long r = mix64(i ^ 0x5555ull);
    const unsigned long long e = 900 + (mix64(r) % 240);
    const double v =
        __longlong_as_double((long long)(((r >> 63) << 63) | (e << 52) | (r & 0xfffffffffffffull)));
    const float a = approx_f32(v);
    int ev, ea;
    frexp(v, &ev);
    frexpf(a, &ea);
    nb[0] += !(ev == ea && (a < 0) == (v < 0) && fabs((double)a - v) < ldexp(fabs(v), -20));
    const int k = (int)(mix64(r + 1) % 121) - 60;
    nb[1] += __double_as_longlong(scale_pow2(v, k)) != __double_as_longlong(v * ldexp(1.0, k));
    const double z = (r & 2) ? -0.0 : 0.0;  // zeros keep their sign
    nb[1] += __double_as_longlong(scale_pow2(z, k)) != __double_as_longlong(z);
    const float x = __uint_as_float((uint32_t)r & 0xbfffffffu);  // finite, |x| < 2
    const float y = __uint_as_float((uint32_t)(r >> 32) & 0xbfffffffu);
    float s, err;
    two_sum(x, y, s, err);
    nb[2] += ((double)s + (double)err) != ((double)x + (double)y);
  }
  for (int q = 0; q < 3; ++q) atomicAdd(bad + q, nb[q]);
}

int main() {
  unsigned long long *d;
  if (cudaMalloc(&d, 8 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(d, 0, 8 * sizeof(unsigned long long));
  const unsigned long long n = 1ull << 28;
  k_widen<<<152 * 8, 256>>>(d);
  k_narrow<<<152 * 8, 256>>>(n, d + 1, d + 2);
  k_misc<<<152 * 8, 256>>>(n, d + 3);
  unsigned long long h[8];
  if (cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  printf("widen %llu %llu\n", h[0], 1ull << 32);
  printf("narrow %llu %llu\n", h[1], h[2]);
  printf("approx %llu %llu\n", h[3], n);
  printf("scale_pow2 %llu %llu\n", h[4], n);
  printf("two_sum %llu %llu\n", h[5], n);
  cudaFree(d);
  return 0;
}
