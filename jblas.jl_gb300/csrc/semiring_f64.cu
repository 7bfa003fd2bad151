// Semiring GEMM, double elements: 64x64 CTA tiles, 4x4 per thread (semiring.cuh).
#include "semiring.cuh"

namespace gb {

int semiring_gemm_f64(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, int accumulate, double* C, int64_t ldc, cudaStream_t s) {
  return semiring_gemm<double, 64, 64, 16, 4, 4>(sr, ta, tb, M, N, K, A, lda, B, ldb, accumulate, C, ldc, s);
}

}  // namespace gb
