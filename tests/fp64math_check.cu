// Device check of the FP64 logarithm and arctangent of fp64_math.cuh
// against CUDA's log / atan2 (on the device, 2^26 random arguments each) and
// against the host C library (a sample copied back), plus special operands.
// Built and run by tests/test_gpu_fp64math.py; prints lines
//   "<name> max_ulp count_above_1ulp count_above_2ulp tested".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>
#include <vector>

#include "fp64_math.cuh"

using namespace j3g;

__host__ __device__ unsigned long long mix64(unsigned long long x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__host__ __device__ double as_double(unsigned long long u) {
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
}

// distance in units in the last place of two finite doubles
__host__ __device__ unsigned long long ulp_dist(double a, double b) {
  long long ia, ib;
  memcpy(&ia, &a, sizeof ia);
  memcpy(&ib, &b, sizeof ib);
  if (ia < 0) ia = (long long)0x8000000000000000ull - ia;
  if (ib < 0) ib = (long long)0x8000000000000000ull - ib;
  return (unsigned long long)(ia > ib ? ia - ib : ib - ia);
}

// i-th log argument: a third uniform in [0.5, 2), a third within 2^-10 of 1,
// a third over 2^-300 .. 2^300
__host__ __device__ double log_arg(unsigned long long i) {
  const unsigned long long r = mix64(i);
  const unsigned long long m = r & 0xfffffffffffffull;
  switch (i % 3) {
    case 0: return (r >> 63) ? 1.0 + (double)m * 0x1p-52 : 0.5 + (double)m * 0x1p-53;
    case 1: return 1.0 + ((double)(long long)(m - (1ull << 51)) * 0x1p-61);
    default: {
      const unsigned long long e = 723 + (mix64(r) % 601);
      return as_double((e << 52) | m);
    }
  }
}

// i-th atan2 argument pair: random signs, |y| / |x| over 2^-70 .. 2^70
__host__ __device__ void atan2_arg(unsigned long long i, double &y, double &x) {
  const unsigned long long r = mix64(i ^ 0xabcdefull), s = mix64(r);
  const unsigned long long ex = 1000 + (s % 48), ey = (i & 3) == 0 ? ex - 2 + (s >> 32) % 5
                                                                   : 953 + ((s >> 16) % 141);
  x = as_double(((r >> 63) << 63) | (ex << 52) | (r & 0xfffffffffffffull));
  y = as_double((((r >> 62) & 1) << 63) | (ey << 52) | (mix64(s) & 0xfffffffffffffull));
}

__global__ void k_vs_cuda(int which, unsigned long long n, unsigned long long *stats) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long mx = 0, c1 = 0, c2 = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    double got, want;
    if (which == 0) {
      const double x = log_arg(i);
      got = flog(x);
      want = log(x);
    } else {
      double y, x;
      atan2_arg(i, y, x);
      got = fatan2(y, x);
      want = atan2(y, x);
    }
    const unsigned long long d = ulp_dist(got, want);
    mx = d > mx ? d : mx;
    c1 += d > 1;
    c2 += d > 2;
  }
  atomicMax(stats, mx);
  atomicAdd(stats + 1, c1);
  atomicAdd(stats + 2, c2);
}

// fatan2_pair against the two separate calls: bit for bit
__global__ void k_pair(unsigned long long n, unsigned long long *bad) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long nb = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    double y, x, a, b;
    atan2_arg(i, y, x);
    if (i % 7 == 3) y = (i & 8) ? x : -x;  // equal magnitudes
    fatan2_pair(y, x, a, b);
    nb += __double_as_longlong(a) != __double_as_longlong(fatan2(y, x));
    nb += __double_as_longlong(b) != __double_as_longlong(fatan2(x, y));
  }
  atomicAdd(bad, nb);
}

__global__ void k_sample(int which, unsigned long long n, double *out) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (which == 0) {
    out[i] = flog(log_arg(i));
  } else {
    double y, x;
    atan2_arg(i, y, x);
    out[i] = fatan2(y, x);
  }
}

__global__ void k_specials(const double *a, const double *b, int n, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[4 * i + 0] = flog(a[i]);
  out[4 * i + 1] = log(a[i]);
  out[4 * i + 2] = fatan2(a[i], b[i]);
  out[4 * i + 3] = atan2(a[i], b[i]);
}

static void check(cudaError_t e) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
    std::exit(1);
  }
}

int main() {
  const unsigned long long n = 1ull << 26;
  unsigned long long *stats;
  check(cudaMalloc(&stats, 3 * sizeof(unsigned long long)));
  const char *names[2] = {"log_vs_cuda", "atan2_vs_cuda"};
  for (int w = 0; w < 2; ++w) {
    check(cudaMemset(stats, 0, 3 * sizeof(unsigned long long)));
    k_vs_cuda<<<152 * 8, 256>>>(w, n, stats);
    check(cudaGetLastError());
    unsigned long long h[3];
    check(cudaMemcpy(h, stats, sizeof h, cudaMemcpyDeviceToHost));
    std::printf("%s %llu %llu %llu %llu\n", names[w], h[0], h[1], h[2], n);
  }
  check(cudaMemset(stats, 0, sizeof(unsigned long long)));
  k_pair<<<152 * 8, 256>>>(n, stats);
  check(cudaGetLastError());
  unsigned long long pair_bad = 0;
  check(cudaMemcpy(&pair_bad, stats, sizeof pair_bad, cudaMemcpyDeviceToHost));
  std::printf("pair %llu 0 0 %llu\n", pair_bad, 2 * n);
  // against the host C library on a sample
  const unsigned long long ns = 1ull << 20;
  double *dout;
  check(cudaMalloc(&dout, ns * sizeof(double)));
  std::vector<double> out(ns);
  const char *hnames[2] = {"log_vs_host", "atan2_vs_host"};
  for (int w = 0; w < 2; ++w) {
    k_sample<<<(unsigned)((ns + 255) / 256), 256>>>(w, ns, dout);
    check(cudaGetLastError());
    check(cudaMemcpy(out.data(), dout, ns * sizeof(double), cudaMemcpyDeviceToHost));
    unsigned long long mx = 0, c1 = 0, c2 = 0;
    for (unsigned long long i = 0; i < ns; ++i) {
      double want;
      if (w == 0) {
        want = std::log(log_arg(i));
      } else {
        double y, x;
        atan2_arg(i, y, x);
        want = std::atan2(y, x);
      }
      const unsigned long long d = ulp_dist(out[i], want);
      mx = d > mx ? d : mx;
      c1 += d > 1;
      c2 += d > 2;
    }
    std::printf("%s %llu %llu %llu %llu\n", hnames[w], mx, c1, c2, ns);
  }
  // special operands: both functions must agree with CUDA's bit for bit
  // (NaN only in class), including signed zeros and the octant boundaries
  const double inf = INFINITY, nan = NAN, tiny = 0x1p-1070, big = 0x1.fffffffffffffp+1023;
  std::vector<double> a = {0.0, -0.0, 1.0, -1.0, inf, -inf, nan, tiny, big, 1.0, 1.0, -2.0,
                           0.0, -0.0, 0.0, -0.0, 3.0, -3.0, 1e-300, 1e300, 1.0, -1.0, 0x1p-1022};
  std::vector<double> b = {1.0, 1.0, -0.0, 0.0, 1.0, -1.0, 1.0, 1.0, 1.0, 1.0, -1.0, -2.0,
                           -0.0, -0.0, 0.0, 0.0, 0.0, -0.0, 1e300, 1e-300, inf, -inf, 1.0};
  const int ns2 = (int)a.size();
  double *da, *db, *ds;
  check(cudaMalloc(&da, ns2 * sizeof(double)));
  check(cudaMalloc(&db, ns2 * sizeof(double)));
  check(cudaMalloc(&ds, 4 * ns2 * sizeof(double)));
  check(cudaMemcpy(da, a.data(), ns2 * sizeof(double), cudaMemcpyHostToDevice));
  check(cudaMemcpy(db, b.data(), ns2 * sizeof(double), cudaMemcpyHostToDevice));
  k_specials<<<1, 64>>>(da, db, ns2, ds);
  check(cudaGetLastError());
  std::vector<double> s(4 * ns2);
  check(cudaMemcpy(s.data(), ds, s.size() * sizeof(double), cudaMemcpyDeviceToHost));
  unsigned long long bad = 0;
  for (int i = 0; i < ns2; ++i)
    for (int k = 0; k < 2; ++k) {
      const double g = s[4 * i + 2 * k], w = s[4 * i + 2 * k + 1];
      const bool same = (g != g) ? (w != w) : (ulp_dist(g, w) <= 1 && std::signbit(g) == std::signbit(w));
      if (!same) {
        ++bad;
        std::fprintf(stderr, "special %d %s(%a, %a): %a vs %a\n", i, k ? "atan2" : "log", a[i],
                     b[i], g, w);
      }
    }
  std::printf("specials %llu 0 0 %d\n", bad, 2 * ns2);
  return 0;
}
