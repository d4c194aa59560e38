// probes.cu -- measurement kernels for the FP64 roofline (not on the compute
// path).  Each kernel evaluates one math function n_iter times per thread on
// a moving argument; profiling them with ncu's FP64 instruction counters gives
// the flop weight of one call (the baseline kernel is the loop alone).
// 1 sqrt, 2 log, 3 atan2 (CUDA's), 4 flog, 5 fatan2 (fp64_math.cuh).
#include <cuda_runtime.h>

#include "../../include/jif3d_gb300.h"
#include "fp64_math.cuh"

namespace {

template <int WHICH>
__global__ void k_probe_math(double *out, int n_iter) {
  double x = 1.0 + threadIdx.x * 1e-3, acc = 0.0;
  for (int i = 0; i < n_iter; ++i) {
    if (WHICH == 1) acc += sqrt(x);
    else if (WHICH == 2) acc += log(x);
    else if (WHICH == 3) acc += atan2(x - 300.0, 0.5 * x + 1.0);
    else if (WHICH == 4) acc += j3g::flog(x);
    else if (WHICH == 5) acc += j3g::fatan2(x - 300.0, 0.5 * x + 1.0);
    else acc += x;
    x = x * 1.0000001 + 0.37;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace

extern "C" int j3g_probe_math(int device, int n_iter) {
  if (n_iter <= 0) return J3G_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return J3G_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return J3G_ERR_CUDA;
  const int threads = 256, blocks = sms;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * threads * blocks) != cudaSuccess) return J3G_ERR_NOMEM;
  k_probe_math<0><<<blocks, threads>>>(d, n_iter);
  k_probe_math<1><<<blocks, threads>>>(d, n_iter);
  k_probe_math<2><<<blocks, threads>>>(d, n_iter);
  k_probe_math<3><<<blocks, threads>>>(d, n_iter);
  k_probe_math<4><<<blocks, threads>>>(d, n_iter);
  k_probe_math<5><<<blocks, threads>>>(d, n_iter);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(d);
  return e == cudaSuccess ? J3G_OK : J3G_ERR_CUDA;
}
