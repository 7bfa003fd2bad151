// Internal launchers for the CUDA-core GEMM (GB_MODE_NATIVE); see native_gemm.cu.  `sms` is the
// device's SM count (tile choice).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {
int native_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int sms,
                    cudaStream_t s);
int native_gemm_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                    int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int sms,
                    cudaStream_t s);
// D (M x N) = D + A (M x K) * B (K x N) as jBLAS's kernel! chain: per element the FMA chain
// starts from D's value (no transposes).
int native_kernel_onto_f64(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
                           int64_t ldb, double* C, int64_t ldc, int sms, cudaStream_t s);
int native_kernel_onto_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                           int64_t ldb, float* C, int64_t ldc, int sms, cudaStream_t s);
}  // namespace gb
