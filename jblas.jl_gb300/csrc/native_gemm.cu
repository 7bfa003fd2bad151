// Native FP64 / FP32 GEMM on the CUDA cores (GB_MODE_NATIVE), on the register-blocked
// mainloop of simt_gemm.cuh.
//
// Per element the arithmetic is exactly jmul!'s: d = a1*x1, then d = fma(ak, xk, d) for
// k = 2..K in order (src/gemm.jl:76-89, 154-168).  The accumulator starts at -0.0 so
// that the first step fma(a1, x1, -0.0) equals the rounded product a1*x1 bit for bit,
// signed zeros included; the K tail is handled with an exact trip count (no zero
// padding, which would turn -0 into +0 and Inf*0 into NaN).
#include "gb_common.cuh"
#include "native_gemm.cuh"
#include "profile.cuh"
#include "simt_gemm.cuh"

namespace gb {

// jmul!'s FMA chain with the BLAS alpha/beta epilogue (beta == 0: C is not read).
template <typename T>
struct FmaChainOp {
  static constexpr bool kInitFromC = false;
  static constexpr bool kVecStore = false;
  static constexpr bool kPairs = false;   // the chain's order is part of its result
  T alpha, beta;
  static __device__ __forceinline__ T init() { return T(-0.0); }
  static __device__ __forceinline__ T step(T acc, T a, T b) { return fma_t<T>(a, b, acc); }
  __device__ __forceinline__ void store(T* c, T acc) const {
    *c = (beta == T(0)) ? alpha * acc : fma_t<T>(alpha, acc, beta * *c);
  }
};

// jBLAS's kernel! (src/kernels.jl:212-238): the chain starts from D's value,
// d = fma(a_n, x_n, d) for n = 1..N in order, and d is stored as is.
template <typename T>
struct FmaOntoCOp {
  static constexpr bool kInitFromC = true;
  static constexpr bool kVecStore = false;
  static constexpr bool kPairs = false;
  int unused;
  static __device__ __forceinline__ T init() { return T(0); }
  static __device__ __forceinline__ T step(T acc, T a, T b) { return fma_t<T>(a, b, acc); }
  __device__ __forceinline__ void store(T* c, T acc) const { *c = acc; }
};

// C = beta * C (alpha == 0 or K == 0); beta == 0 writes zeros without reading C.
template <typename T>
__global__ void scale_c_kernel(int64_t M, int64_t N, T beta, T* __restrict__ C, int64_t ldc) {
  const int64_t total = M * N;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t m = t % M, n = t / M;
    T* c = &C[m + n * ldc];
    *c = (beta == T(0)) ? T(0) : beta * *c;
  }
}

template <typename T>
static int launch_scale(int64_t M, int64_t N, T beta, T* C, int64_t ldc, cudaStream_t s) {
  const int64_t total = M * N;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  GB_LAUNCH(GB_KERNEL_SCALE_C, s,
            scale_c_kernel<T><<<static_cast<unsigned>(blocks), 256, 0, s>>>(M, N, beta, C, ldc));
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
static int launch_simt(int ta, int tb, int64_t M, int64_t N, int64_t K, T alpha, const T* A,
                       int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc,
                       cudaStream_t s) {
  dim3 grid;
  if (!simt_grid<BM, BN>(M, N, &grid)) return GB_ERR_UNSUPPORTED;
  constexpr int NT = (BM / TM) * (BN / TN);
  const FmaChainOp<T> op{alpha, beta};
#define GB_SIMT_CASE(TA_, TB_)                                                                   \
  GB_LAUNCH(GB_KERNEL_NATIVE_GEMM, s,                                                            \
            (simt_gemm_kernel<T, FmaChainOp<T>, BM, BN, BK, TM, TN, TA_, TB_><<<grid, NT, 0, s>>>( \
                M, N, K, op, A, lda, B, ldb, C, ldc)))
  if (!ta && !tb) GB_SIMT_CASE(false, false);
  else if (!ta && tb) GB_SIMT_CASE(false, true);
  else if (ta && !tb) GB_SIMT_CASE(true, false);
  else GB_SIMT_CASE(true, true);
#undef GB_SIMT_CASE
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
static int launch_onto(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const T* B, int64_t ldb, T* C,
                       int64_t ldc, cudaStream_t s) {
  dim3 grid;
  if (!simt_grid<BM, BN>(M, N, &grid)) return GB_ERR_UNSUPPORTED;
  constexpr int NT = (BM / TM) * (BN / TN);
  const FmaOntoCOp<T> op{0};
  GB_LAUNCH(GB_KERNEL_NATIVE_GEMM, s,
            (simt_gemm_kernel<T, FmaOntoCOp<T>, BM, BN, BK, TM, TN, false, false><<<grid, NT, 0, s>>>(
                M, N, K, op, A, lda, B, ldb, C, ldc)));
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int native_kernel_onto_f64(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
                           int64_t ldb, double* C, int64_t ldc, int sms, cudaStream_t s) {
  if (M == 0 || N == 0 || K == 0) return GB_OK;   // an empty chain leaves D as it is
  if (((M + 63) / 64) * ((N + 63) / 64) < 2 * static_cast<int64_t>(sms))
    return launch_onto<double, 32, 32, 16, 4, 4>(M, N, K, A, lda, B, ldb, C, ldc, s);
  return launch_onto<double, 64, 64, 16, 4, 4>(M, N, K, A, lda, B, ldb, C, ldc, s);
}

// FP32 always on 64x64 tiles: the 128x128 tile's 64 accumulators loaded from D exceed its
// 128-register budget.
int native_kernel_onto_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                           int64_t ldb, float* C, int64_t ldc, int sms, cudaStream_t s) {
  (void)sms;
  if (M == 0 || N == 0 || K == 0) return GB_OK;
  return launch_onto<float, 64, 64, 16, 4, 4>(M, N, K, A, lda, B, ldb, C, ldc, s);
}

// Tile choice: the large tiles (fewer operand loads per FMA) unless they leave SMs idle, then
// smaller ones for more CTAs (measured at 1024^3: FP32 64x64 tiles 24 TFLOP/s against 15.5 for
// 128x128 with 64 CTAs on 152 SMs; FP64 32x32 tiles +7%).  Every tile shape runs the same
// per-element chain, so the choice never changes a result bit.
int native_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int sms,
                    cudaStream_t s) {
  if (M == 0 || N == 0) return GB_OK;
  if (alpha == 0.0 || K == 0) return launch_scale<double>(M, N, beta, C, ldc, s);
  if (((M + 63) / 64) * ((N + 63) / 64) < 2 * static_cast<int64_t>(sms))
    return launch_simt<double, 32, 32, 16, 4, 4>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
  return launch_simt<double, 64, 64, 16, 4, 4>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

int native_gemm_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                    int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int sms,
                    cudaStream_t s) {
  if (M == 0 || N == 0) return GB_OK;
  if (alpha == 0.0f || K == 0) return launch_scale<float>(M, N, beta, C, ldc, s);
  if (((M + 127) / 128) * ((N + 127) / 128) < static_cast<int64_t>(sms))
    return launch_simt<float, 64, 64, 16, 4, 4>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
  return launch_simt<float, 128, 128, 16, 8, 8>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

}  // namespace gb
