// Semiring GEMM on the CUDA cores: C = [C (+)] (+)_k op(A)[i,k] (x) op(B)[k,j].
//
// jBLAS keeps a tuple-SIMD Vec type (src/simd.jl) out of its module with the note that it
// could serve "custom number types ... so it works with min-plus algebra" (src/jBLAS.jl:10).
// Here the custom arithmetic is a policy of the register-blocked mainloop shared with the
// native GEMM (simt_gemm.cuh): the accumulator starts at the identity of (+), each k folds
// in one (x) product, and the epilogue folds in C when accumulating.
//
// (+) is min or max.  For floating point it ignores a NaN operand (fminf / fmaxf) and a
// zero result is stored as +0.0: min and max are then associative and commutative on every
// input, including the sign of zero, so the result does not depend on the K order.  int32
// + and * wrap modulo 2^32 (computed on uint32_t).
//
// Because (+) is exact and associative, two consecutive k can be folded in by one
// three-input min / max (min.f32 / max.f32 with three sources; __vimin3_s32 / __vimax3_s32):
// 1.5 instructions per element instead of 2 where that is faster (float: every semiring;
// int32: (max, min) and (min, max)).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "gb_common.cuh"
#include "profile.cuh"
#include "simt_gemm.cuh"

namespace gb {

template <typename T>
struct SrArith;

template <>
struct SrArith<float> {
  static __device__ __forceinline__ float lo() { return __int_as_float(0xff800000); }   // -Inf
  static __device__ __forceinline__ float hi() { return __int_as_float(0x7f800000); }   // +Inf
  static __device__ __forceinline__ float min(float a, float b) { return fminf(a, b); }
  static __device__ __forceinline__ float max(float a, float b) { return fmaxf(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float canon(float v) { return v == 0.0f ? 0.0f : v; }
  static constexpr bool kHas3 = true;
  static __device__ __forceinline__ float min3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
  }
  static __device__ __forceinline__ float max3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
  }
};

template <>
struct SrArith<double> {
  static __device__ __forceinline__ double lo() { return __longlong_as_double(0xfff0000000000000ll); }
  static __device__ __forceinline__ double hi() { return __longlong_as_double(0x7ff0000000000000ll); }
  static __device__ __forceinline__ double min(double a, double b) { return fmin(a, b); }
  static __device__ __forceinline__ double max(double a, double b) { return fmax(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double canon(double v) { return v == 0.0 ? 0.0 : v; }
  static constexpr bool kHas3 = false;
  static __device__ __forceinline__ double min3(double a, double b, double c) { return fmin(fmin(a, b), c); }
  static __device__ __forceinline__ double max3(double a, double b, double c) { return fmax(fmax(a, b), c); }
};

template <>
struct SrArith<int32_t> {
  static __device__ __forceinline__ int32_t lo() { return INT32_MIN; }
  static __device__ __forceinline__ int32_t hi() { return INT32_MAX; }
  static __device__ __forceinline__ int32_t min(int32_t a, int32_t b) { return a < b ? a : b; }
  static __device__ __forceinline__ int32_t max(int32_t a, int32_t b) { return a > b ? a : b; }
  static __device__ __forceinline__ int32_t add(int32_t a, int32_t b) {
    return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b));
  }
  static __device__ __forceinline__ int32_t mul(int32_t a, int32_t b) {
    return static_cast<int32_t>(static_cast<uint32_t>(a) * static_cast<uint32_t>(b));
  }
  static __device__ __forceinline__ int32_t canon(int32_t v) { return v; }
  static constexpr bool kHas3 = true;
  static __device__ __forceinline__ int32_t min3(int32_t a, int32_t b, int32_t c) { return __vimin3_s32(a, b, c); }
  static __device__ __forceinline__ int32_t max3(int32_t a, int32_t b, int32_t c) { return __vimax3_s32(a, b, c); }
};

template <typename T, int SR>
struct SemiringOp {
  using Ar = SrArith<T>;
  static constexpr bool kMinPlus = SR == GB_SEMIRING_MIN_PLUS || SR == GB_SEMIRING_MIN_MAX;
  static constexpr bool kInitFromC = false;   // C is folded in by the epilogue instead
  static constexpr bool kVecStore = false;
  static constexpr bool kPairs =
      Ar::kHas3 && (std::is_floating_point<T>::value || SR == GB_SEMIRING_MAX_MIN || SR == GB_SEMIRING_MIN_MAX);
  int accumulate;

  static __device__ __forceinline__ T oplus(T x, T y) { return kMinPlus ? Ar::min(x, y) : Ar::max(x, y); }
  static __device__ __forceinline__ T otimes(T a, T b) {
    if (SR == GB_SEMIRING_MIN_PLUS || SR == GB_SEMIRING_MAX_PLUS) return Ar::add(a, b);
    if (SR == GB_SEMIRING_MAX_MIN) return Ar::min(a, b);
    if (SR == GB_SEMIRING_MIN_MAX) return Ar::max(a, b);
    return Ar::mul(a, b);
  }
  static __device__ __forceinline__ T init() { return kMinPlus ? Ar::hi() : Ar::lo(); }
  static __device__ __forceinline__ T step(T acc, T a, T b) { return oplus(acc, otimes(a, b)); }
  static __device__ __forceinline__ T step2(T acc, T a0, T b0, T a1, T b1) {
    const T p0 = otimes(a0, b0), p1 = otimes(a1, b1);
    return kMinPlus ? Ar::min3(acc, p0, p1) : Ar::max3(acc, p0, p1);
  }
  __device__ __forceinline__ void store(T* c, T acc) const { *c = Ar::canon(accumulate ? oplus(*c, acc) : acc); }
};

template <typename T, int SR, int BM, int BN, int BK, int TM, int TN>
static int launch_semiring(int ta, int tb, int64_t M, int64_t N, int64_t K, const T* A, int64_t lda,
                           const T* B, int64_t ldb, int accumulate, T* C, int64_t ldc, cudaStream_t s) {
  dim3 grid;
  if (!simt_grid<BM, BN>(M, N, &grid)) return GB_ERR_UNSUPPORTED;
  constexpr int NT = (BM / TM) * (BN / TN);
  const SemiringOp<T, SR> op{accumulate};
#define GB_SR_CASE(TA_, TB_)                                                                        \
  GB_LAUNCH(GB_KERNEL_SEMIRING_GEMM, s,                                                             \
            (simt_gemm_kernel<T, SemiringOp<T, SR>, BM, BN, BK, TM, TN, TA_, TB_><<<grid, NT, 0, s>>>( \
                M, N, K, op, A, lda, B, ldb, C, ldc)))
  if (!ta && !tb) GB_SR_CASE(false, false);
  else if (!ta && tb) GB_SR_CASE(false, true);
  else if (ta && !tb) GB_SR_CASE(true, false);
  else GB_SR_CASE(true, true);
#undef GB_SR_CASE
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// All semirings for one element type and tile configuration (M, N > 0; arguments checked).
template <typename T, int BM, int BN, int BK, int TM, int TN>
static int semiring_gemm(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const T* A, int64_t lda,
                         const T* B, int64_t ldb, int accumulate, T* C, int64_t ldc, cudaStream_t s) {
  switch (sr) {
#define GB_SR(SR_)                                                                                 \
  case SR_:                                                                                        \
    return launch_semiring<T, SR_, BM, BN, BK, TM, TN>(ta, tb, M, N, K, A, lda, B, ldb, accumulate, C, \
                                                       ldc, s);
    GB_SR(GB_SEMIRING_MIN_PLUS)
    GB_SR(GB_SEMIRING_MAX_PLUS)
    GB_SR(GB_SEMIRING_MAX_MIN)
    GB_SR(GB_SEMIRING_MIN_MAX)
    GB_SR(GB_SEMIRING_MAX_TIMES)
#undef GB_SR
    default:
      return GB_ERR_INVALID_VALUE;
  }
}

int semiring_gemm_f64(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, int accumulate, double* C, int64_t ldc, cudaStream_t s);
int semiring_gemm_f32(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                      const float* B, int64_t ldb, int accumulate, float* C, int64_t ldc, cudaStream_t s);
int semiring_gemm_i32(int sr, int ta, int tb, int64_t M, int64_t N, int64_t K, const int32_t* A,
                      int64_t lda, const int32_t* B, int64_t ldb, int accumulate, int32_t* C, int64_t ldc,
                      cudaStream_t s);

}  // namespace gb
