// Microkernels for counting the FP64 instructions of one call of each math
// function the node kernels use: CUDA's sqrt / log / atan2 and the library's
// flog / fatan2 (jif3d_gb300/csrc/fp64_math.cuh).  Each kernel evaluates its
// function n_iter times per thread on a moving argument; kernel 0 is the loop
// alone, whose counts are subtracted.  Profiled with ncu's FP64 instruction
// counters (DFMA counted as 2 flops, DADD and DMUL as 1) these give the flop
// weights of the FP64 roofline.  Measurement only: built and run by
// tests/test_gpu_fp64math.py, and under ncu by hand:
//   nvcc -O3 -std=c++17 -gencode=arch=compute_103a,code=sm_103a \
//        -I jif3d_gb300/csrc tests/fp64_weights_probe.cu -o fp64_weights_probe
//   ncu --clock-control none --metrics sm__sass_thread_inst_executed_op_dfma_pred_on.sum,\
//       sm__sass_thread_inst_executed_op_dadd_pred_on.sum,\
//       sm__sass_thread_inst_executed_op_dmul_pred_on.sum --csv ./fp64_weights_probe
#include <cstdio>
#include <cuda_runtime.h>

#include "fp64_math.cuh"

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

int main() {
  const int n_iter = 1000, threads = 256;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return 1;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * threads * sms) != cudaSuccess) return 1;
  k_probe_math<0><<<sms, threads>>>(d, n_iter);
  k_probe_math<1><<<sms, threads>>>(d, n_iter);
  k_probe_math<2><<<sms, threads>>>(d, n_iter);
  k_probe_math<3><<<sms, threads>>>(d, n_iter);
  k_probe_math<4><<<sms, threads>>>(d, n_iter);
  k_probe_math<5><<<sms, threads>>>(d, n_iter);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(d);
  std::printf("calls per kernel %d\n", n_iter * threads * sms);
  return e == cudaSuccess ? 0 : 1;
}
