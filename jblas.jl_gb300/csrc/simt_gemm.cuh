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
//   Op::kVecStore         when true (with op.value(c, acc), the value store writes, and
//                         op.reads_c(), whether it reads C's old value) C is written with vector
//                         stores or, when C is not aligned for them, through shared memory
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

// Shared memory of one tile: double-buffered BK x BM and BK x BN panels, rows padded by 16
// bytes (transposing stores hit distinct banks, vector reads stay aligned).
template <typename T, int BM, int BN, int BK>
struct SimtSmem {
  static constexpr int PAD = 16 / static_cast<int>(sizeof(T));
  static constexpr int A_ELEMS = 2 * BK * (BM + PAD);
  static constexpr int ELEMS = A_ELEMS + 2 * BK * (BN + PAD);
};

// One BM x BN tile of C at (m0, n0), computed by the NT = (BM / TM) * (BN / TN) threads of the
// CTA in `smem` (SimtSmem<T, BM, BN, BK>::ELEMS elements, 16-byte aligned).  TM x TN per thread,
// split in two halves of VM (VN) contiguous rows (columns) to allow vector shared-memory reads.
// The last shared-memory reads are not followed by a barrier: a caller that runs another tile in
// the same shared memory synchronises first.
template <typename T, typename Op, int BM, int BN, int BK, int TM, int TN, bool TA, bool TB>
__device__ __forceinline__ void simt_tile(int64_t M, int64_t N, int64_t K, const Op& op, const T* __restrict__ A,
                                          int64_t lda, const T* __restrict__ B, int64_t ldb, T* __restrict__ C,
                                          int64_t ldc, int64_t m0, int64_t n0, T* smem) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int VM = TM / 2, VN = TN / 2;
  constexpr int A_PER = (BM * BK) / NT, B_PER = (BK * BN) / NT;
  static_assert((BM * BK) % NT == 0 && (BK * BN) % NT == 0, "tile/thread mismatch");
  static_assert(TM % 2 == 0 && TN % 2 == 0, "two halves per thread tile");

  constexpr int PAD = SimtSmem<T, BM, BN, BK>::PAD;
  T (*As)[BK][BM + PAD] = reinterpret_cast<T (*)[BK][BM + PAD]>(smem);
  T (*Bs)[BK][BN + PAD] = reinterpret_cast<T (*)[BK][BN + PAD]>(smem + SimtSmem<T, BM, BN, BK>::A_ELEMS);

  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);

  // Global-load geometry, fixed for the whole K loop.  With NT a multiple of the panel's
  // leading extent, every load of a thread sits in one row (column) of the panel, or at one k,
  // and its r-th element lies a fixed stride after the first: one pointer per operand,
  // advanced by one K panel per iteration, replaces the per-element 64-bit index arithmetic.
  // A (not transposed, A[m + k*lda]): row ml fixed, k = kA + r*(NT/BM), one row check.
  // A (transposed,     A[k + m*lda]): k fixed,       m = mA + r*(NT/BK), one check per r.
  // B likewise, with rows and columns exchanged.
  static_assert(TA ? NT % BK == 0 : NT % BM == 0, "A panel: NT must tile its leading extent");
  static_assert(TB ? NT % BN == 0 : NT % BK == 0, "B panel: NT must tile its leading extent");
  constexpr int A_RSTEP = TA ? NT / BK : NT / BM;   // k (or m) between a thread's loads
  constexpr int B_RSTEP = TB ? NT / BN : NT / BK;
  const int a_lead = TA ? tid % BK : tid % BM;        // k (TA) or m within the panel
  const int a_0 = TA ? tid / BK : tid / BM;           // first m (TA) or k
  const int b_lead = TB ? tid % BN : tid % BK;        // n (TB) or k
  const int b_0 = TB ? tid / BN : tid / BK;           // first k (TB) or n
  const T* pa = TA ? A + a_lead + (m0 + a_0) * lda : A + (m0 + a_lead) + a_0 * lda;
  const T* pb = TB ? B + (n0 + b_lead) + b_0 * ldb : B + b_lead + (n0 + b_0) * ldb;
  const int64_t a_rs = static_cast<int64_t>(A_RSTEP) * lda;   // between a thread's loads
  const int64_t b_rs = static_cast<int64_t>(B_RSTEP) * ldb;
  const int64_t a_ks = TA ? BK : static_cast<int64_t>(BK) * lda;
  const int64_t b_ks = TB ? static_cast<int64_t>(BK) * ldb : BK;
  // Rows of A (columns of B) inside the matrix: one flag, or one bit per load.
  uint32_t a_ok = 0, b_ok = 0;
#pragma unroll
  for (int r = 0; r < A_PER; ++r)
    if (TA ? (m0 + a_0 + r * A_RSTEP < M) : (r == 0 && m0 + a_lead < M)) a_ok |= 1u << r;
#pragma unroll
  for (int r = 0; r < B_PER; ++r)
    if (TB ? (r == 0 && n0 + b_lead < N) : (n0 + b_0 + r * B_RSTEP < N)) b_ok |= 1u << r;
  if (!TA) a_ok = (a_ok & 1u) ? ~0u : 0u;   // one row of A for all loads
  if (TB) b_ok = (b_ok & 1u) ? ~0u : 0u;    // one column of B for all loads

  T ra[A_PER], rb[B_PER];

  // Loads the K panel at pa / pb, of which the first kc k are inside the matrix.
  auto load_tile = [&](int kc) {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      const int kl = TA ? a_lead : a_0 + r * A_RSTEP;
      T v = T(0);
      if (((a_ok >> r) & 1u) && kl < kc) v = pa[r * a_rs];
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      const int kl = TB ? b_0 + r * B_RSTEP : b_lead;
      T v = T(0);
      if (((b_ok >> r) & 1u) && kl < kc) v = pb[r * b_rs];
      rb[r] = v;
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int r = 0; r < A_PER; ++r) {
      if (TA) As[buf][a_lead][a_0 + r * A_RSTEP] = ra[r];
      else As[buf][a_0 + r * A_RSTEP][a_lead] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < B_PER; ++r) {
      if (TB) Bs[buf][b_0 + r * B_RSTEP][b_lead] = rb[r];
      else Bs[buf][b_lead][b_0 + r * B_RSTEP] = rb[r];
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
    load_tile(static_cast<int>(K < BK ? K : BK));
    store_tile(0);
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
      const bool has_next = k0 + BK < K;
      if (has_next) {
        pa += a_ks;
        pb += b_ks;
        load_tile(static_cast<int>(K - k0 - BK < BK ? K - k0 - BK : BK));
      }
      const int kc = static_cast<int>(K - k0 < BK ? K - k0 : BK);
      compute(buf, kc);
      if (has_next) {
        store_tile(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
  }

  if constexpr (Op::kVecStore) {
    // Epilogue for policies with kVecStore (and op.value / op.reads_c), where short K loops
    // make the stores of C a large part of a tile.  The per-element stores of the general path
    // write one element in each of 16 columns per warp instruction; instead:
    //  - beta = 0 and C and ldc multiples of VM elements: a thread's VM consecutive rows of a
    //    column go out as one vector store (whole 32-byte sectors);
    //  - otherwise the tile goes through shared memory, half of its rows at a time, and a warp
    //    writes 32 consecutive rows of one column per instruction.  The panels' shared memory
    //    is reused: every warp has finished reading it first.
    const bool rc = op.reads_c();
    const bool vec_ok = VM > 1 && !rc && (reinterpret_cast<uintptr_t>(C) % (VM * sizeof(T))) == 0 &&
                        (ldc % VM) == 0;   // the same for the whole CTA
    if (vec_ok) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t mb = m0 + h * (BM / 2) + ty * VM;   // first of this half's VM rows
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          const int64_t n = n0 + (j < VN ? tx * VN + j : BN / 2 + tx * VN + (j - VN));
          if (n >= N) continue;
          T* __restrict__ c = &C[mb + n * ldc];
          if (mb + VM <= M) {
            VecT<T, VM> v;
#pragma unroll
            for (int i = 0; i < VM; ++i) v.v[i] = op.value(T(0), acc[h * VM + i][j]);
            *reinterpret_cast<VecT<T, VM>*>(c) = v;
          } else {
#pragma unroll
            for (int i = 0; i < VM; ++i)
              if (mb + i < M) c[i] = op.value(T(0), acc[h * VM + i][j]);
          }
        }
      }
    } else {
      constexpr int HR = BM / 2;    // rows per half
      constexpr int LDS = HR + 1;   // column stride: consecutive rows in consecutive banks
      static_assert(BN * LDS <= SimtSmem<T, BM, BN, BK>::ELEMS, "staged epilogue does not fit");
      __syncthreads();
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          const int col = (j < VN ? tx * VN + j : BN / 2 + tx * VN + (j - VN));
#pragma unroll
          for (int i = 0; i < VM; ++i) smem[col * LDS + ty * VM + i] = acc[h * VM + i][j];
        }
        __syncthreads();
        for (int e = tid; e < HR * BN; e += NT) {
          const int r = e % HR, col = e / HR;
          const int64_t m = m0 + h * HR + r, n = n0 + col;
          if (m < M && n < N) {
            T* c = &C[m + n * ldc];
            *c = op.value(rc ? *c : T(0), smem[col * LDS + r]);
          }
        }
        __syncthreads();
      }
    }
  } else {
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
}

// The tile above as a kernel: CTA (x, y) computes the tile at (x BM, y BN).
// 4-byte elements: two CTAs per SM (at most 128 registers a thread for 256 threads);
// 8-byte elements: no residency bound (0), which leaves ptxas its own register choice.
template <typename T, typename Op, int BM, int BN, int BK, int TM, int TN, bool TA, bool TB>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), sizeof(T) == 4 ? 2 : 0)
    simt_gemm_kernel(int64_t M, int64_t N, int64_t K, Op op, const T* __restrict__ A, int64_t lda,
                     const T* __restrict__ B, int64_t ldb, T* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) T smem[SimtSmem<T, BM, BN, BK>::ELEMS];
  simt_tile<T, Op, BM, BN, BK, TM, TN, TA, TB>(M, N, K, op, A, lda, B, ldb, C, ldc,
                                               static_cast<int64_t>(blockIdx.x) * BM,
                                               static_cast<int64_t>(blockIdx.y) * BN, smem);
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
