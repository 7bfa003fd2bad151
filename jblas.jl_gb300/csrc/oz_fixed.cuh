// Fixed-point view of FP64 operands shared by the Ozaki split kernels (digit planes and
// CRT residue planes): row exponents, round-half-away scaling to integers, exact BF16 of
// small integers.  Integer arithmetic only: GB300's FP64 pipe is narrow.
#pragma once
#include <stdint.h>

namespace gb {

constexpr int OZ_EXP_NONFINITE = 0x7FFFFFFF;

// Row exponent e with amax < 2^e (e = ilogb(amax) + 1), from the IEEE fields in integer
// arithmetic (GB300's FP64 pipe is narrow): biased exponent - 1022 for normal amax,
// -1010 - clz(bits) for subnormal amax.
__device__ __forceinline__ int row_exponent_of(unsigned long long amax_bits) {
  if (amax_bits >= 0x7FF0000000000000ull) return OZ_EXP_NONFINITE;  // Inf or NaN in the row
  if (amax_bits == 0) return 0;
  const int ex = static_cast<int>(amax_bits >> 52);
  return ex ? ex - 1022 : -1010 - __clzll(static_cast<long long>(amax_bits));
}

__device__ __forceinline__ int row_exponent(unsigned long long amax_bits) { return row_exponent_of(amax_bits); }

// Fixed point in integer arithmetic (GB300's FP64 pipe is ~1/64 of FP32, so the splits
// never touch it).  For a row with exponent e (amax < 2^e) and SB = slices*bits:
//   Y = round-half-away(x * 2^(SB-1-e))          an integer, |Y| <= 2^(SB-1)
//   digits d_s..d_2 = balanced base-2^b digits of Y, in [-2^(b-1), 2^(b-1));  d_1 the rest
//   so x * 2^-e = sum_p d_p 2^(1 - p*b) + delta,  |delta| <= 2^-SB,  |d_1| <= 2^(b-1).
// Y is built from the IEEE fields of x (m * 2^(ex-52)) with shifts only.  Word = uint64_t
// for SB <= 62, unsigned __int128 beyond.
template <typename Word>
__device__ __forceinline__ Word fixed_point(double x, int e, int SB) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
  const int biased = static_cast<int>((bits >> 52) & 0x7FF);
  unsigned long long m = bits & 0x000FFFFFFFFFFFFFull;
  int ex = -1022;
  if (biased) {
    m |= 0x0010000000000000ull;
    ex = biased - 1023;
  }
  Word mag = 0;
  if (m) {
    const int sh = ex - 53 + SB - e;   // v = m * 2^sh
    if (sh >= 0) {
      mag = static_cast<Word>(m) << sh;
    } else {
      const int t = -sh;
      if (t < 64) mag = static_cast<Word>((m + (1ull << (t - 1))) >> t);
    }
  }
  return (bits >> 63) ? static_cast<Word>(0) - mag : mag;
}

// Signed arithmetic shift of a two's-complement word.
template <typename Word>
__device__ __forceinline__ Word sar(Word y, int b);
template <>
__device__ __forceinline__ uint64_t sar<uint64_t>(uint64_t y, int b) {
  return static_cast<uint64_t>(static_cast<int64_t>(y) >> b);
}
template <>
__device__ __forceinline__ unsigned __int128 sar<unsigned __int128>(unsigned __int128 y, int b) {
  return static_cast<unsigned __int128>(static_cast<__int128>(y) >> b);
}

// Exact BF16 of a small integer |d| <= 2^22 without a conversion instruction:
// float(d) = bits(1.5*2^23 + d) - 1.5*2^23, then the upper half of the float is the BF16.
__device__ __forceinline__ uint32_t bf16_bits_of_int(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return __float_as_uint(f) >> 16;
}

}  // namespace gb
