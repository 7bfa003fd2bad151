// Native FP64 / FP32 GEMM on the CUDA cores (GB_MODE_NATIVE).
//
// Restates jBLAS's register-blocked driver (src/gemm.jl:244-348) for the GPU: each
// thread owns a TM x TN register tile of C (the reference's rows x cols tile from
// pick_kernel_size, src/kernel_structure.jl:76-99), the CTA stages BM x BK / BK x BN
// operand panels in shared memory (the role of jBLAS's prefetch schedule,
// src/memory_management.jl:181-277), and the full K reduction stays in registers.
//
// Per element the arithmetic is exactly jmul!'s: d = a1*x1, then d = fma(ak, xk, d) for
// k = 2..K in order (src/gemm.jl:76-89, 154-168).  The accumulator starts at -0.0 so
// that the first step fma(a1, x1, -0.0) equals the rounded product a1*x1 bit for bit,
// signed zeros included; the K tail is handled with an exact trip count (no zero
// padding, which would turn -0 into +0 and Inf*0 into NaN).
#include "gb_common.cuh"
#include "native_gemm.cuh"
#include "profile.cuh"

namespace gb {

template <typename T, int V>
struct alignas(sizeof(T) * V) VecT {
  T v[V];
};

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <>
__device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Tile configuration: BM x BN CTA tile, BK K-panel, TM x TN per thread split in two
// halves of VM (VN) contiguous rows (columns) to allow vector shared-memory reads.
template <typename T, int BM, int BN, int BK, int TM, int TN, bool TA, bool TB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    simt_gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha, const T* __restrict__ A, int64_t lda,
                     const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int VM = TM / 2, VN = TN / 2;
  constexpr int A_PER = (BM * BK) / NT, B_PER = (BK * BN) / NT;
  static_assert((BM * BK) % NT == 0 && (BK * BN) % NT == 0, "tile/thread mismatch");

  // Rows padded by 16 bytes: transposing stores hit distinct banks, vector reads stay aligned.
  constexpr int PAD = 16 / static_cast<int>(sizeof(T));
  __shared__ __align__(16) T As[2][BK][BM + PAD];
  __shared__ __align__(16) T Bs[2][BK][BN + PAD];

  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);
  const int64_t m0 = static_cast<int64_t>(blockIdx.x) * BM;
  const int64_t n0 = static_cast<int64_t>(blockIdx.y) * BN;

  T ra[A_PER], rb[B_PER];

  auto load_tile = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      const int idx = tid + r * NT;
      int ml, kl;
      if (TA) { kl = idx % BK; ml = idx / BK; } else { ml = idx % BM; kl = idx / BM; }
      const int64_t m = m0 + ml, k = k0 + kl;
      T v = T(0);
      if (m < M && k < K) v = TA ? A[k + m * lda] : A[m + k * lda];
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      const int idx = tid + r * NT;
      int nl, kl;
      if (TB) { nl = idx % BN; kl = idx / BN; } else { kl = idx % BK; nl = idx / BK; }
      const int64_t n = n0 + nl, k = k0 + kl;
      T v = T(0);
      if (n < N && k < K) v = TB ? B[n + k * ldb] : B[k + n * ldb];
      rb[r] = v;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      const int idx = tid + r * NT;
      int ml, kl;
      if (TA) { kl = idx % BK; ml = idx / BK; } else { ml = idx % BM; kl = idx / BM; }
      As[buf][kl][ml] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      const int idx = tid + r * NT;
      int nl, kl;
      if (TB) { nl = idx % BN; kl = idx / BN; } else { kl = idx % BK; nl = idx / BK; }
      Bs[buf][kl][nl] = rb[r];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(-0.0);

  auto compute = [&](int buf, int kc) {
    auto step = [&](int kk) {
      const VecT<T, VM> a0 = *reinterpret_cast<const VecT<T, VM>*>(&As[buf][kk][ty * VM]);
      const VecT<T, VM> a1 = *reinterpret_cast<const VecT<T, VM>*>(&As[buf][kk][BM / 2 + ty * VM]);
      const VecT<T, VN> b0 = *reinterpret_cast<const VecT<T, VN>*>(&Bs[buf][kk][tx * VN]);
      const VecT<T, VN> b1 = *reinterpret_cast<const VecT<T, VN>*>(&Bs[buf][kk][BN / 2 + tx * VN]);
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < VM; ++i) { a[i] = a0.v[i]; a[VM + i] = a1.v[i]; }
#pragma unroll
      for (int j = 0; j < VN; ++j) { b[j] = b0.v[j]; b[VN + j] = b1.v[j]; }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma_t<T>(a[i], b[j], acc[i][j]);
    };
    if (kc == BK) {
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) step(kk);
    } else {
      for (int kk = 0; kk < kc; ++kk) step(kk);
    }
  };

  if (K > 0) {
    load_tile(0);
    store_tile(0);
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
      const bool has_next = k0 + BK < K;
      if (has_next) load_tile(k0 + BK);
      const int kc = static_cast<int>(K - k0 < BK ? K - k0 : BK);
      compute(buf, kc);
      if (has_next) {
        store_tile(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
  }

#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + (i < VM ? ty * VM + i : BM / 2 + ty * VM + (i - VM));
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t n = n0 + (j < VN ? tx * VN + j : BN / 2 + tx * VN + (j - VN));
      if (n >= N) continue;
      T* c = &C[m + n * ldc];
      *c = (beta == T(0)) ? alpha * acc[i][j] : fma_t<T>(alpha, acc[i][j], beta * *c);
    }
  }
}

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
  const int64_t gx = (M + BM - 1) / BM, gy = (N + BN - 1) / BN;
  if (gx > 0x7FFFFFFF || gy > 65535) return GB_ERR_UNSUPPORTED;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  constexpr int NT = (BM / TM) * (BN / TN);
#define GB_SIMT_CASE(TA_, TB_)                                                                   \
  GB_LAUNCH(GB_KERNEL_NATIVE_GEMM, s,                                                            \
            (simt_gemm_kernel<T, BM, BN, BK, TM, TN, TA_, TB_><<<grid, NT, 0, s>>>(M, N, K, alpha, A, \
                                                                                  lda, B, ldb, beta, C, ldc)))
  if (!ta && !tb) GB_SIMT_CASE(false, false);
  else if (!ta && tb) GB_SIMT_CASE(false, true);
  else if (ta && !tb) GB_SIMT_CASE(true, false);
  else GB_SIMT_CASE(true, true);
#undef GB_SIMT_CASE
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int native_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                    cudaStream_t s) {
  if (M == 0 || N == 0) return GB_OK;
  if (alpha == 0.0 || K == 0) return launch_scale<double>(M, N, beta, C, ldc, s);
  return launch_simt<double, 64, 64, 16, 4, 4>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

int native_gemm_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A,
                    int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                    cudaStream_t s) {
  if (M == 0 || N == 0) return GB_OK;
  if (alpha == 0.0f || K == 0) return launch_scale<float>(M, N, beta, C, ldc, s);
  return launch_simt<float, 128, 128, 8, 8, 8>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

}  // namespace gb
