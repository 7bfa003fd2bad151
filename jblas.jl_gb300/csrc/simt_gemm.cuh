// Register-blocked GEMM mainloop on the CUDA cores, shared by the native FP64/FP32 GEMM
// (GB_MODE_NATIVE) and the semiring GEMM.
//
// Restates jBLAS's register-blocked driver (src/gemm.jl:244-348) for the GPU: each
// thread owns a TM x TN register tile of C (the reference's rows x cols tile from
// pick_kernel_size, src/kernel_structure.jl:76-99), the CTA stages BM x BK / BK x BN
// operand panels in shared memory (the role of jBLAS's prefetch schedule,
// src/memory_management.jl:181-277), and the full K reduction stays in registers.
//
// The per-element arithmetic is a policy `Op`:
//   Op::init()            the accumulator before k = 1
//   Op::step(acc, a, b)   one contraction step, applied for k = 1..K in order
//   op.store(c, acc)      the epilogue writing one element of C
//   Op::kInitFromC        when true the accumulator starts from C's element instead of init()
//                         (jBLAS's kernel!, which folds A*X onto D's value)
//   Op::kPairs, Op::step2(acc, a0, b0, a1, b1)
//                         when kPairs, two consecutive k are folded in by one call (for
//                         associative, exact reductions such as min / max, whose result
//                         does not depend on the grouping; the FMA chain keeps kPairs false)
// The K tail is handled with an exact trip count: no padded k is ever folded in.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

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
// 4-byte elements: two CTAs per SM (at most 128 registers a thread for 256 threads);
// 8-byte elements: no residency bound (0), which leaves ptxas its own register choice.
template <typename T, typename Op, int BM, int BN, int BK, int TM, int TN, bool TA, bool TB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), sizeof(T) == 4 ? 2 : 0)
    simt_gemm_kernel(int64_t M, int64_t N, int64_t K, Op op, const T* __restrict__ A, int64_t lda,
                     const T* __restrict__ B, int64_t ldb, T* __restrict__ C, int64_t ldc) {
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
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + (i < VM ? ty * VM + i : BM / 2 + ty * VM + (i - VM));
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      if constexpr (Op::kInitFromC) {
        const int64_t n = n0 + (j < VN ? tx * VN + j : BN / 2 + tx * VN + (j - VN));
        acc[i][j] = (m < M && n < N) ? C[m + n * ldc] : T(0);
      } else {
        acc[i][j] = Op::init();
      }
    }
  }

  auto load_k = [&](int buf, int kk, T (&a)[TM], T (&b)[TN]) {
    const VecT<T, VM> a0 = *reinterpret_cast<const VecT<T, VM>*>(&As[buf][kk][ty * VM]);
    const VecT<T, VM> a1 = *reinterpret_cast<const VecT<T, VM>*>(&As[buf][kk][BM / 2 + ty * VM]);
    const VecT<T, VN> b0 = *reinterpret_cast<const VecT<T, VN>*>(&Bs[buf][kk][tx * VN]);
    const VecT<T, VN> b1 = *reinterpret_cast<const VecT<T, VN>*>(&Bs[buf][kk][BN / 2 + tx * VN]);
#pragma unroll
    for (int i = 0; i < VM; ++i) { a[i] = a0.v[i]; a[VM + i] = a1.v[i]; }
#pragma unroll
    for (int j = 0; j < VN; ++j) { b[j] = b0.v[j]; b[VN + j] = b1.v[j]; }
  };
  auto compute = [&](int buf, int kc) {
    auto step = [&](int kk) {
      T a[TM], b[TN];
      load_k(buf, kk, a, b);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = Op::step(acc[i][j], a[i], b[j]);
    };
    if constexpr (Op::kPairs) {
      static_assert(BK % 2 == 0, "paired steps need an even K panel");
      auto step2 = [&](int kk) {
        T a[TM], b[TN], a2[TM], b2[TN];
        load_k(buf, kk, a, b);
        load_k(buf, kk + 1, a2, b2);
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = Op::step2(acc[i][j], a[i], b[j], a2[i], b2[j]);
      };
      if (kc == BK) {
#pragma unroll
        for (int kk = 0; kk < BK; kk += 2) step2(kk);
      } else {
        int kk = 0;
        for (; kk + 1 < kc; kk += 2) step2(kk);
        if (kk < kc) step(kk);
      }
    } else {
      if (kc == BK) {
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) step(kk);
      } else {
        for (int kk = 0; kk < kc; ++kk) step(kk);
      }
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
      op.store(&C[m + n * ldc], acc[i][j]);
    }
  }
}

// Grid of the kernel above for an M x N output; false when it does not fit a launch.
template <int BM, int BN>
inline bool simt_grid(int64_t M, int64_t N, dim3* grid) {
  const int64_t gx = (M + BM - 1) / BM, gy = (N + BN - 1) / BN;
  if (gx > 0x7FFFFFFF || gy > 65535) return false;
  *grid = dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  return true;
}

}  // namespace gb
