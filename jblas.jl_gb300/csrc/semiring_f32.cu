// Semiring GEMM, float elements: 128x128 CTA tiles, 8x8 per thread (semiring.cuh).
#include "semiring.cuh"

namespace gb {

int semiring_gemm_f32(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                      const float* B, int64_t ldb, int accumulate, float* C, int64_t ldc, cudaStream_t s) {
  return semiring_gemm<float, 128, 128, 8, 8, 8>(sr, ta, tb, M, N, K, A, lda, B, ldb, accumulate, C, ldc, s);
}

}  // namespace gb
