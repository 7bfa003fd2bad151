// Measured FMA-pipe peaks of the current GPU (the CUDA-core counterpart of jBLAS's machine
// constants, deps/build.jl:26-34, which its code generator reads instead of guessing).
//
// A register-only loop: every thread runs 8 independent FMA chains x = fma(x, a, b) (8 chains
// keep the pipe's latency covered), on 4 resident blocks of 256 threads per SM, timed with CUDA
// events around a second launch after a warm-up launch.  The result feeds the rooflines of the
// CUDA-core kernels (native FP64/FP32, grouped, semiring), which the tensor-core peaks of the
// pool's measured-peaks file do not cover.
#include <cuda_runtime.h>

#include "gb_common.cuh"

namespace gb {

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T* __restrict__ sink, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = static_cast<T>(threadIdx.x + c) * static_cast<T>(1e-3);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  T s = x[0];
#pragma unroll
  for (int c = 1; c < 8; ++c) s += x[c];
  if (s == static_cast<T>(-1.2345)) sink[0] = s;   // keeps the chains live; never true for these inputs
}

template <typename T>
static int time_peak(int sms, int iters, T* sink, double* tflops) {
  const int blocks = 4 * sms;
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  // a = 1 - 2^-20 and b = 2^-10 keep x bounded near b / (1 - a) without subnormals or overflow
  const T a = static_cast<T>(1.0 - 1.0 / 1048576.0), b = static_cast<T>(1.0 / 1024.0);
  fma_peak_kernel<T><<<blocks, 256>>>(sink, iters, a, b);
  cudaEventRecord(e0);
  fma_peak_kernel<T><<<blocks, 256>>>(sink, iters, a, b);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return gb_set_cuda_error(e, "peak timing");
  const double flops = 2.0 * 8.0 * static_cast<double>(iters) * blocks * 256.0;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return GB_OK;
}

int measure_fma_peaks(int sms, double* fp64_tflops, double* fp32_tflops) {
  void* sink = nullptr;
  GB_CUDA_TRY(cudaMalloc(&sink, 16));
  int rc = GB_OK;
  // about 10 GFLOP of FP64 (a few ms) and 80 GFLOP of FP32 (about 1 ms)
  if (fp64_tflops) rc = time_peak<double>(sms, 4096, static_cast<double*>(sink), fp64_tflops);
  if (!rc && fp32_tflops) rc = time_peak<float>(sms, 32768, static_cast<float*>(sink), fp32_tflops);
  cudaFree(sink);
  return rc;
}

}  // namespace gb
