// Internal interface of the grouped GEMM (grouped.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbblas.h"

namespace gb {
gb_grouped_tuning_t grouped_default_tuning(int dtype_bytes);
int grouped_configs(int dtype_bytes);
int grouped_validate_tuning(int dtype_bytes, const gb_grouped_tuning_t& t);
size_t grouped_workspace_bytes(int count);
int grouped_launch(int dtype_bytes, const gb_problem_t* d_probs, int count, const gb_grouped_tuning_t& tuning,
                   long long* d_offsets, int sms, cudaStream_t s);
int grouped_autotune(int dtype_bytes, const gb_problem_t* h_probs, int count, int sms, cudaMemPool_t pool,
                     int reps, gb_grouped_tuning_t* out, float* class_ms, cudaStream_t s);
int grouped_f64_noalloc(const gb_problem_t* d_probs, int count, const gb_grouped_tuning_t* tuning, cudaStream_t s);
// Fills a device problem table for a strided batch (count entries).
int grouped_fill_strided(gb_problem_t* d_probs, int count, int64_t M, int64_t N, int64_t K, int64_t lda, int64_t ldb,
                         int64_t ldc, const void* A, const void* B, void* C, int64_t strideA_bytes,
                         int64_t strideB_bytes, int64_t strideC_bytes, double alpha, double beta, cudaStream_t s);
}  // namespace gb
