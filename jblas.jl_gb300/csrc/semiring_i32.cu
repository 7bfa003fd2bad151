// Semiring GEMM, int32_t elements: 128x128 CTA tiles, 8x8 per thread (semiring.cuh).
#include "semiring.cuh"

namespace gb {

int semiring_gemm_i32(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const int32_t* A, int64_t lda,
                      const int32_t* B, int64_t ldb, int accumulate, int32_t* C, int64_t ldc, cudaStream_t s) {
  return semiring_gemm<int32_t, 128, 128, 16, 8, 8>(sr, ta, tb, M, N, K, A, lda, B, ldb, accumulate, C, ldc, s);
}

}  // namespace gb
