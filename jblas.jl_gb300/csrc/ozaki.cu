// FP64-accurate GEMM by Ozaki-scheme splitting onto BF16 tcgen05 tensor cores.
//
// Method: Ozaki, Ogita, Oishi and Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59 (2012), with the fixed-point (per-row / per-column power-of-two
// scaled) digit splitting used by Mukunoki, Ozaki, Ogita and Imamura, "DGEMM using
// Tensor Cores, and Its Accurate and Reproducible Versions", ISC 2020.
//
//   op(A)[i,k] = 2^ea_i * sum_p dA_p[i,k] * 2^(1 - p*b),   |dA_p| <= 2^(b-1), p = 1..s
//   op(B)[k,j] = 2^eb_j * sum_q dB_q[k,j] * 2^(1 - q*b)
//   C[i,j] ~= alpha * 2^(ea_i + eb_j) * sum_{p+q <= s+1} 2^(2 - (p+q)*b) * S_pq[i,j] + beta*C
//   S_pq = dA_p * dB_q    (integer digits held exactly in BF16, products exact in FP32:
//                          the planner keeps every partial sum an integer below 2^24)
//
// The digit planes are the GPU analogue of the packing buffers jBLAS never built
// (src/memory_management.jl:78-177 plans cache blocks but nothing packs): K-major,
// BF16, one plane per digit, read by TMA with the 128-byte swizzle.
//
// Slice-product kernel (one persistent CTA per SM, warp-specialised):
//   warp 0      TMA producer: A/B digit tiles into a 4-stage shared-memory ring
//               (the role of jBLAS's prefetch schedule, src/memory_management.jl:181-277)
//   warp 1      allocates 512 TMEM columns; lane 0 issues tcgen05.mma 128x256x16 into a
//               double-buffered FP32 accumulator (jBLAS's register tile, src/gemm.jl:318-333)
//   warps 2-5   epilogue: tcgen05.ld each exact group sum, FP64 accumulation of the
//               groups in a per-CTA tile buffer, final power-of-two rescale with alpha/beta
//               (jBLAS's store_block, src/gemm.jl:3-11, here with the recombination fused)
// Every mbarrier wait is bounded (gb_common.cuh); on expiry the CTA records
// GB_ERR_PIPELINE_TIMEOUT, drains its in-flight copies and MMAs, frees TMEM and exits.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "gb_common.cuh"
#include "oz_fixed.cuh"
#include "ozaki.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

// ============================================================== planner (host)

int oz_bits_for(int64_t kc) {
  int lg = 0;
  while ((int64_t(1) << lg) < kc) ++lg;           // ceil(log2 kc)
  int b = (26 - lg) / 2;                          // kc * 2^(2b-2) <= 2^24
  if (b > 9) b = 9;                               // |digit| <= 256 is exact in BF16
  return b;
}

int oz_make_plan(int64_t M, int64_t N, int64_t K, int slices, OzPlan* plan) {
  return oz_make_plan_chunks(M, N, K, slices, 1, plan);
}

int oz_make_plan_chunks(int64_t M, int64_t N, int64_t K, int slices, int min_chunks, OzPlan* plan) {
  if (slices < 1 || slices > OZ_MAX_SLICES || min_chunks < 1) return GB_ERR_INVALID_VALUE;
  OzPlan& P = *plan;
  P.slices = slices;
  // One exact chunk covers K up to 2^16 (b >= 5); longer K, or a requested split into
  // min_chunks (shorter chunks allow wider digits), gives equal chunks of whole K panels.
  int64_t kb_total = (K + TC_BK - 1) / TC_BK;
  if (kb_total < 1) kb_total = 1;
  int64_t nchunks = (K + 65535) / 65536;
  if (nchunks < min_chunks) nchunks = min_chunks;
  if (nchunks > kb_total) nchunks = kb_total;
  if (nchunks < 1) nchunks = 1;
  int64_t kb_chunk = (kb_total + nchunks - 1) / nchunks;
  nchunks = (kb_total + kb_chunk - 1) / kb_chunk;
  int64_t kc = kb_chunk * TC_BK;
  if (kc > K) kc = K < 1 ? 1 : K;
  P.k_chunk = kc;
  P.nchunks = static_cast<int>(nchunks);
  P.bits = oz_bits_for(kc);
  // the split builds x * 2^(slices*bits - 1 - e) in at most 128-bit integers
  if (slices * P.bits > 126) return GB_ERR_UNSUPPORTED;
  // pairs that can share one exact FP32 sum
  const double per_pair = static_cast<double>(kc) * std::ldexp(1.0, 2 * P.bits - 2);
  int share = static_cast<int>(std::floor(16777216.0 / per_pair));
  if (share < 1) share = 1;
  if (share > 8) share = 8;

  SliceSchedule& S = P.sched;
  std::memset(&S, 0, sizeof(S));
  P.kb_total = static_cast<int32_t>(kb_total);
  S.kb_chunk = static_cast<int32_t>(kb_chunk);
  S.bits = P.bits;
  // Levels from the smallest contribution (slices + 1) up to the leading one (2): the FP64
  // recombination then adds small terms first, so its rounding error stays near one ulp of
  // the result instead of growing with the number of groups.
  int g = 0, np = 0;
  for (int level = slices + 1; level >= 2; --level) {
    // pairs (p, q), p + q = level, 1 <= p, q <= slices, in increasing p
    int in_group = 0;
    for (int p = 1; p <= slices; ++p) {
      const int q = level - p;
      if (q < 1 || q > slices) continue;
      if (in_group == 0) {
        if (g >= TC_MAX_GROUPS) return GB_ERR_UNSUPPORTED;
        S.level[g] = static_cast<int8_t>(level);
        S.npairs[g] = 0;
        S.pair_off[g] = static_cast<int16_t>(np);
        ++g;
      }
      if (np >= TC_MAX_PAIRS) return GB_ERR_UNSUPPORTED;
      S.pp[np] = static_cast<uint8_t>(p - 1);
      S.pq[np] = static_cast<uint8_t>(q - 1);
      ++np;
      S.npairs[g - 1]++;
      if (++in_group == share) in_group = 0;
    }
  }
  S.ngroups = g;
  P.groups = g;
  P.products = np;
  P.flops_tensor = 2.0 * static_cast<double>(M) * static_cast<double>(N) *
                   static_cast<double>(kb_total * TC_BK) * np;
  return GB_OK;
}

// ============================================================== statistics kernels

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
}

// Exponent e of |x| with |x| < 2^e (e = ilogb|x| + 1, as row_exponent_of), from the IEEE
// fields of |x| (abits); 0 for x = 0, OZ_EXP_NONFINITE for Inf / NaN.
__device__ __forceinline__ int exp_of_abits(unsigned long long a) {
  const int ex = static_cast<int>(a >> 52);
  if (ex == 0x7FF) return OZ_EXP_NONFINITE;
  if (ex) return ex - 1022;
  if (a == 0) return 0;
  return -1010 - __clzll(static_cast<long long>(a));   // subnormal: m 2^-1074, m = a
}

// v * 2^d for d <= 0 rounded toward zero (never above the true value), 0 below FP32's range.
__device__ __forceinline__ float scale_down_rz(float v, int d) {
  if (d == 0 || v == 0.0f) return v;
  if (d < -300) return 0.0f;
  while (d < -126) {
    v = __fmul_rz(v, 0x1p-126f);
    d += 126;
  }
  return __fmul_rz(v, __uint_as_float(static_cast<uint32_t>(d + 127) << 23));
}

// |x| * 2^-e as FP32 from the IEEE fields of |x| (abits), never above the true value (the
// mantissa is truncated; relative error below 2^-23 in FP32's normal range); subnormal x are
// scaled exactly (rounded toward zero), values below FP32's range give 0.
__device__ __forceinline__ float scaled_f32_trunc(unsigned long long abits, int e) {
  const int ex = static_cast<int>(abits >> 52);
  if (ex) {
    const int fe = ex - 1023 - e + 127;   // <= 126 because |x| < 2^e
    if (fe < 1) return 0.0f;
    return __uint_as_float((static_cast<uint32_t>(fe) << 23) | static_cast<uint32_t>((abits >> 29) & 0x7FFFFF));
  }
  if (abits == 0) return 0.0f;
  // subnormal: m 2^-1074 with m = abits < 2^52; m truncated to FP32, then times 2^(-1074 - e)
  const int sh = -1074 - e;
  if (sh < -300) return 0.0f;
  const float fm = __ull2float_rz(abits);
  if (sh >= 0) return fm;   // cannot happen while |x| < 2^e and the max is subnormal; kept exact-safe
  return scale_down_rz(fm, sh);
}

// Running statistics of one thread's elements: exponent e of its max, sums of |x| 2^-e and
// x^2 2^-2e in FP32.  When a larger exponent arrives the sums are rescaled by an exact power
// of two (rounded toward zero below FP32's normal range), so one read of X suffices.
struct RunStats {
  unsigned long long mx = 0;
  int e = -2000;   // no element yet
  bool nonfinite = false;
  float sa = 0.0f, sq = 0.0f;

  __device__ __forceinline__ void add(unsigned long long bits, bool sums) {
    const unsigned long long a = bits & 0x7FFFFFFFFFFFFFFFull;
    mx = a > mx ? a : mx;
    if (!sums) return;
    // Fast path: a normal element whose exponent field does not exceed the running one
    // (e > -2000 once an element has been seen; e = field - 1022 for a normal maximum).  Its
    // scaled value |x| 2^-e truncated to FP32 takes the exponent field - e - 896 and the top 23
    // fraction bits; below FP32's normal range it is 0, as in scaled_f32_trunc.
    const uint32_t hi = static_cast<uint32_t>(a >> 32);
    const int field = static_cast<int>(hi >> 20);
    if (field != 0 && field != 0x7FF && field - 1022 <= e) {
      const int fe = field - e - 896;   // (field - 1023) - e + 127
      const uint32_t frac = __funnelshift_r(static_cast<uint32_t>(a), hi, 29) & 0x7FFFFFu;
      const float f = fe >= 1 ? __uint_as_float((static_cast<uint32_t>(fe) << 23) | frac) : 0.0f;
      sa += f;
      sq = fmaf(f, f, sq);
      return;
    }
    if (a == 0) return;
    const int ea = exp_of_abits(a);
    if (ea == OZ_EXP_NONFINITE) {
      nonfinite = true;
      return;
    }
    if (ea > e) {
      sa = scale_down_rz(sa, e - ea);
      sq = scale_down_rz(sq, 2 * (e - ea));
      e = ea;
    }
    const float f = scaled_f32_trunc(a, e);
    sa += f;
    sq = fmaf(f, f, sq);
  }
  // rescales this thread's sums to exponent e2 >= e
  __device__ __forceinline__ void to(int e2) {
    if (e2 != e && e > -2000) {
      sa = scale_down_rz(sa, e - e2);
      sq = scale_down_rz(sq, 2 * (e - e2));
    }
    e = e2;
  }
};

// Row statistics without FP64 arithmetic (GB300's FP64 pipe is narrow), in one read of X:
// the exact max |x| by integer compare (atomicMax across K slices) and, when asked, the FP32
// sums of |x| 2^-e_s and x^2 2^-2e_s over truncated scaled values, e_s the exponent of the
// slice's own max (running per thread, combined by exact rescaling).  The host or the
// device planner rescales the slice sums to the row exponent and turns them into rigorous
// one-sided bounds (every FP32 rounding is one of the K - 1 additions of a K-term sum).
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// k contiguous (ks == 1): one warp per row, one K slice.
template <bool SUMS>
__global__ void __launch_bounds__(256) stats_kc_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                       int64_t rs, OzRowStats st) {
  const int lane = threadIdx.x & 31;
  const int64_t r = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (r >= R) return;
  const unsigned long long* row = reinterpret_cast<const unsigned long long*>(X + r * rs);
  RunStats rs_;
  int64_t k = lane;
  for (; k + 96 < K; k += 128) {
    const unsigned long long b0 = row[k], b1 = row[k + 32], b2 = row[k + 64], b3 = row[k + 96];
    rs_.add(b0, SUMS);
    rs_.add(b1, SUMS);
    rs_.add(b2, SUMS);
    rs_.add(b3, SUMS);
  }
  for (; k < K; k += 32) rs_.add(row[k], SUMS);
  unsigned long long mx = rs_.mx;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) st.amax_bits[r] = mx;
  if (!SUMS) return;
  const int e = row_exponent_of(mx);
  float sa = 0.0f, sq = 0.0f;
  if (e != OZ_EXP_NONFINITE) {
    rs_.to(e);
    sa = rs_.sa;
    sq = rs_.sq;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
  }
  if (lane == 0) {
    st.part_e[r] = e;
    st.part_sa[r] = sa;
    st.part_sq[r] = sq;
  }
}

// rows contiguous (rs == 1): 32 rows x one K slice per block, 8 warps stride over k.
template <bool SUMS>
__global__ void __launch_bounds__(256) stats_rc_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                       int64_t ks, int64_t kslice, OzRowStats st) {
  __shared__ unsigned long long smx[8][32];
  __shared__ float ssa[8][32], ssq[8][32];
  const int tr = threadIdx.x & 31, tk = threadIdx.x >> 5;
  const int64_t r = static_cast<int64_t>(blockIdx.x) * 32 + tr;
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * kslice;
  const int64_t k1 = (k0 + kslice < K) ? k0 + kslice : K;
  const unsigned long long* Xb = reinterpret_cast<const unsigned long long*>(X);
  RunStats rs_;
  if (r < R) {
    int64_t k = k0 + tk;
    for (; k + 24 < k1; k += 32) {
      const unsigned long long b0 = Xb[r + k * ks], b1 = Xb[r + (k + 8) * ks];
      const unsigned long long b2 = Xb[r + (k + 16) * ks], b3 = Xb[r + (k + 24) * ks];
      rs_.add(b0, SUMS);
      rs_.add(b1, SUMS);
      rs_.add(b2, SUMS);
      rs_.add(b3, SUMS);
    }
    for (; k < k1; k += 8) rs_.add(Xb[r + k * ks], SUMS);
  }
  smx[tk][tr] = rs_.mx;
  __syncthreads();
  unsigned long long mx = 0;
  for (int w = 0; w < 8; ++w) mx = umax64(mx, smx[w][tr]);
  if (tk == 0 && r < R && mx) atomicMax(st.amax_bits + r, mx);
  if (!SUMS) return;
  const int e = row_exponent_of(mx);
  if (e != OZ_EXP_NONFINITE) rs_.to(e);
  ssa[tk][tr] = (e != OZ_EXP_NONFINITE) ? rs_.sa : 0.0f;
  ssq[tk][tr] = (e != OZ_EXP_NONFINITE) ? rs_.sq : 0.0f;
  __syncthreads();
  if (tk == 0 && r < R) {
    float sa = 0.0f, sq = 0.0f;
    for (int w = 0; w < 8; ++w) {
      sa += ssa[w][tr];
      sq += ssq[w][tr];
    }
    const int64_t o = static_cast<int64_t>(blockIdx.y) * R + r;
    st.part_e[o] = e;
    st.part_sa[o] = sa;
    st.part_sq[o] = sq;
  }
}

// The same statistics with 16-byte loads (double2), for aligned operands: twice the bytes in
// flight per load instruction and half the address arithmetic of the 8-byte forms above.
// k contiguous: one warp per row, lane l reads the pairs (k, k + 1) with k = 2 (l + 32 i).
// Needs the row starts 16-byte aligned (X aligned, rs even).
template <bool SUMS>
__global__ void __launch_bounds__(256) stats_kc2_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                        int64_t rs, OzRowStats st) {
  const int lane = threadIdx.x & 31;
  const int64_t r = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (r >= R) return;
  const ulonglong2* row = reinterpret_cast<const ulonglong2*>(X + r * rs);
  const int64_t K2 = K / 2;
  RunStats rs_;
  int64_t k = lane;
  // software-pipelined: the next four 16-byte loads are in flight while the current four are
  // folded in (the data-dependent branches of the running statistics would otherwise keep the
  // compiler from hoisting them)
  if (k + 96 < K2) {
    ulonglong2 b[4] = {row[k], row[k + 32], row[k + 64], row[k + 96]};
    for (; k + 128 + 96 < K2; k += 128) {
      const ulonglong2 n[4] = {row[k + 128], row[k + 160], row[k + 192], row[k + 224]};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        rs_.add(b[q].x, SUMS);
        rs_.add(b[q].y, SUMS);
        b[q] = n[q];
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      rs_.add(b[q].x, SUMS);
      rs_.add(b[q].y, SUMS);
    }
    k += 128;
  }
  for (; k < K2; k += 32) {
    const ulonglong2 b = row[k];
    rs_.add(b.x, SUMS);
    rs_.add(b.y, SUMS);
  }
  if ((K & 1) && lane == 0)
    rs_.add(reinterpret_cast<const unsigned long long*>(X + r * rs)[K - 1], SUMS);
  unsigned long long mx = rs_.mx;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = umax64(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) st.amax_bits[r] = mx;
  if (!SUMS) return;
  const int e = row_exponent_of(mx);
  float sa = 0.0f, sq = 0.0f;
  if (e != OZ_EXP_NONFINITE) {
    rs_.to(e);
    sa = rs_.sa;
    sq = rs_.sq;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
  }
  if (lane == 0) {
    st.part_e[r] = e;
    st.part_sa[r] = sa;
    st.part_sq[r] = sq;
  }
}

// rows contiguous: 64 rows x one K slice per block, lane l holds rows 2l and 2l + 1 of the
// block (one 16-byte load per k), 8 warps stride over k.  Needs X aligned, ks even, R even.
template <bool SUMS>
__global__ void __launch_bounds__(256) stats_rc2_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                        int64_t ks, int64_t kslice, OzRowStats st) {
  __shared__ unsigned long long smx[8][64];
  __shared__ float ssa[8][64], ssq[8][64];
  __shared__ int sexp[64];
  const int lane = threadIdx.x & 31, tk = threadIdx.x >> 5;
  const int64_t rb = static_cast<int64_t>(blockIdx.x) * 64;
  const int64_t r = rb + 2 * lane;   // rows r and r + 1 (R even: both valid or both not)
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * kslice;
  const int64_t k1 = (k0 + kslice < K) ? k0 + kslice : K;
  const ulonglong2* Xb = reinterpret_cast<const ulonglong2*>(X);
  RunStats s0, s1;
  if (r < R) {
    const int64_t h = r >> 1, hs = ks >> 1;   // pair index of (r, k): (r + k ks) / 2
    int64_t k = k0 + tk;
    // software-pipelined as in stats_kc2_kernel
    if (k + 24 < k1) {
      ulonglong2 b[4] = {Xb[h + k * hs], Xb[h + (k + 8) * hs], Xb[h + (k + 16) * hs], Xb[h + (k + 24) * hs]};
      for (; k + 32 + 24 < k1; k += 32) {
        const ulonglong2 n[4] = {Xb[h + (k + 32) * hs], Xb[h + (k + 40) * hs], Xb[h + (k + 48) * hs],
                                 Xb[h + (k + 56) * hs]};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          s0.add(b[q].x, SUMS);
          s1.add(b[q].y, SUMS);
          b[q] = n[q];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        s0.add(b[q].x, SUMS);
        s1.add(b[q].y, SUMS);
      }
      k += 32;
    }
    for (; k < k1; k += 8) {
      const ulonglong2 b = Xb[h + k * hs];
      s0.add(b.x, SUMS);
      s1.add(b.y, SUMS);
    }
  }
  smx[tk][2 * lane] = s0.mx;
  smx[tk][2 * lane + 1] = s1.mx;
  __syncthreads();
  unsigned long long m0 = 0, m1 = 0;
  for (int w = 0; w < 8; ++w) {
    m0 = umax64(m0, smx[w][2 * lane]);
    m1 = umax64(m1, smx[w][2 * lane + 1]);
  }
  if (tk == 0 && r < R) {
    if (m0) atomicMax(st.amax_bits + r, m0);
    if (m1) atomicMax(st.amax_bits + r + 1, m1);
  }
  if (!SUMS) return;
  const int e0 = row_exponent_of(m0), e1 = row_exponent_of(m1);
  if (tk == 0) {
    sexp[2 * lane] = e0;
    sexp[2 * lane + 1] = e1;
  }
  if (e0 != OZ_EXP_NONFINITE) s0.to(e0);
  if (e1 != OZ_EXP_NONFINITE) s1.to(e1);
  ssa[tk][2 * lane] = (e0 != OZ_EXP_NONFINITE) ? s0.sa : 0.0f;
  ssq[tk][2 * lane] = (e0 != OZ_EXP_NONFINITE) ? s0.sq : 0.0f;
  ssa[tk][2 * lane + 1] = (e1 != OZ_EXP_NONFINITE) ? s1.sa : 0.0f;
  ssq[tk][2 * lane + 1] = (e1 != OZ_EXP_NONFINITE) ? s1.sq : 0.0f;
  __syncthreads();
  if (tk < 2) {   // warps 0 and 1 finish rows rb + lane and rb + 32 + lane
    const int rr = tk * 32 + lane;
    const int64_t row = rb + rr;
    if (row < R) {
      float sa = 0.0f, sq = 0.0f;
      for (int w = 0; w < 8; ++w) {
        sa += ssa[w][rr];
        sq += ssq[w][rr];
      }
      const int64_t o = static_cast<int64_t>(blockIdx.y) * R + row;
      st.part_e[o] = sexp[rr];
      st.part_sa[o] = sa;
      st.part_sq[o] = sq;
    }
  }
}

int oz_stats_kslices(int64_t R, int64_t K, int64_t ks, int sms) {
  if (ks == 1 || R <= 0 || K <= 0) return 1;
  const int64_t row_blocks = (R + 63) / 64;
  int64_t S = (4 * static_cast<int64_t>(sms) + row_blocks - 1) / row_blocks;
  const int64_t smax = (K + 255) / 256;
  if (S > smax) S = smax;
  if (S > 65535) S = 65535;
  if (S < 1) S = 1;
  const int64_t kslice = (K + S - 1) / S;
  return static_cast<int>((K + kslice - 1) / kslice);
}

int oz_row_stats(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, OzRowStats st, bool sums,
                 cudaStream_t s) {
  if (R <= 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(st.amax_bits, 0, R * sizeof(unsigned long long), s));
  if (K <= 0) return GB_OK;
  const bool aligned = (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  if (ks == 1 && aligned && (rs & 1) == 0) {
    const int64_t blocks = (R + 7) / 8;
    if (sums)
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s,
                stats_kc2_kernel<true><<<static_cast<unsigned>(blocks), 256, 0, s>>>(X, R, K, rs, st));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s,
                stats_kc2_kernel<false><<<static_cast<unsigned>(blocks), 256, 0, s>>>(X, R, K, rs, st));
  } else if (ks != 1 && rs == 1 && aligned && (ks & 1) == 0 && (R & 1) == 0) {
    const int64_t kslice = (K + st.kslices - 1) / st.kslices;
    dim3 grid(static_cast<unsigned>((R + 63) / 64), static_cast<unsigned>(st.kslices));
    if (sums)
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s, stats_rc2_kernel<true><<<grid, 256, 0, s>>>(X, R, K, ks, kslice, st));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s, stats_rc2_kernel<false><<<grid, 256, 0, s>>>(X, R, K, ks, kslice, st));
  } else if (ks == 1) {
    const int64_t blocks = (R + 7) / 8;
    if (sums)
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s,
                stats_kc_kernel<true><<<static_cast<unsigned>(blocks), 256, 0, s>>>(X, R, K, rs, st));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s,
                stats_kc_kernel<false><<<static_cast<unsigned>(blocks), 256, 0, s>>>(X, R, K, rs, st));
  } else {
    const int64_t kslice = (K + st.kslices - 1) / st.kslices;
    dim3 grid(static_cast<unsigned>((R + 31) / 32), static_cast<unsigned>(st.kslices));
    if (sums)
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s, stats_rc_kernel<true><<<grid, 256, 0, s>>>(X, R, K, ks, kslice, st));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s, stats_rc_kernel<false><<<grid, 256, 0, s>>>(X, R, K, ks, kslice, st));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ============================================================== split kernels

// 16 consecutive k of one row -> `slices` planes of 16 BF16 digits (two 16-byte stores each).
template <typename Word>
__device__ __forceinline__ void split_16(const double (&x)[16], int e, int slices, int bits,
                                         __nv_bfloat16* out0, int64_t plane_stride, int nvalid) {
  const int SB = slices * bits;
  const int H = 1 << (bits - 1);
  const Word MASK = (static_cast<Word>(1) << bits) - 1;
  Word y[16];
  const bool nonfinite = (e == 0x7FFFFFFF);
#pragma unroll
  for (int j = 0; j < 16; ++j) y[j] = nonfinite ? static_cast<Word>(0) : fixed_point<Word>(x[j], e, SB);
  // Balanced digits with one bias add: Z = Y + sum_{i < s-1} H 2^(i b) has plain base-2^b
  // digits d_i + H in its low s-1 positions (no carries, since d_i + H lies in [0, 2^b)),
  // and Z >> ((s-1) b) (arithmetic) is the top digit.
  Word hsum = 0;
  for (int i = 0; i + 1 < slices; ++i) hsum += static_cast<Word>(H) << (i * bits);
#pragma unroll
  for (int j = 0; j < 16; ++j) y[j] += hsum;
  for (int p = slices - 1; p >= 0; --p) {
    uint32_t packed[8];
    const int shift = (slices - 1 - p) * bits;   // plane p holds the digit at bit position shift
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      int d0, d1;
      if (p > 0) {
        d0 = static_cast<int>(static_cast<uint32_t>(y[j] >> shift) & static_cast<uint32_t>(MASK)) - H;
        d1 = static_cast<int>(static_cast<uint32_t>(y[j + 1] >> shift) & static_cast<uint32_t>(MASK)) - H;
      } else {
        d0 = static_cast<int>(static_cast<int64_t>(sar<Word>(y[j], shift)));
        d1 = static_cast<int>(static_cast<int64_t>(sar<Word>(y[j + 1], shift)));
      }
      packed[j / 2] = bf16_bits_of_int(d0) | (bf16_bits_of_int(d1) << 16);
    }
    __nv_bfloat16* dst = out0 + p * plane_stride;
    if (nvalid == 16) {
      uint4* d4 = reinterpret_cast<uint4*>(dst);
      d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
      d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    } else {
      unsigned short* d2 = reinterpret_cast<unsigned short*>(dst);
      for (int j = 0; j < nvalid; ++j) d2[j] = static_cast<unsigned short>(packed[j / 2] >> (16 * (j & 1)));
    }
  }
}

// One thread = one row r and 16 consecutive k.  RC (rows contiguous, rs == 1): threads of a
// block run along r, so every load instruction reads consecutive rows; otherwise (k
// contiguous) threads run along k.  Stores are 32 contiguous bytes per plane per thread.
template <bool RC, typename Word>
__global__ void __launch_bounds__(256) split_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                    int64_t rs, int64_t ks,
                                                    const unsigned long long* __restrict__ amax_bits,
                                                    int slices, int bits, __nv_bfloat16* __restrict__ planes,
                                                    int64_t pitch, int64_t plane_stride, int32_t* __restrict__ exps) {
  int64_t r, kc;
  if (RC) {
    r = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
    kc = blockIdx.y;
  } else {
    kc = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x;
    r = blockIdx.y;
  }
  const int64_t k0 = kc * 16;
  if (r >= R || k0 >= K) return;
  const int e = row_exponent(amax_bits[r]);
  if (k0 == 0) exps[r] = e;
  const int nvalid = static_cast<int>(K - k0 < 16 ? K - k0 : 16);
  double x[16];
  const double* src = X + r * rs + k0 * ks;
#pragma unroll
  for (int j = 0; j < 16; ++j) x[j] = (j < nvalid) ? src[j * ks] : 0.0;
  __nv_bfloat16* out0 = planes + r * pitch + k0;
  split_16<Word>(x, e, slices, bits, out0, plane_stride, nvalid);
}

// Rows [0, R) of X; plane_stride = the element distance between consecutive digit planes (the
// planes of the whole operand: its rows times the pitch, also for a band of its rows).
static int oz_split_rows(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks,
                         const unsigned long long* amax_bits, int slices, int bits, __nv_bfloat16* planes,
                         int64_t pitch, int64_t plane_stride, int32_t* exps, cudaStream_t s) {
  if (R <= 0 || K <= 0) return GB_OK;
  const int64_t kchunks = (K + 15) / 16;
  const bool wide = slices * bits > 62;
  if (rs == 1 && R > 1) {
    const int64_t gx = (R + 255) / 256;
    if (kchunks > 65535) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(kchunks));
    if (wide)
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (split_kernel<true, unsigned __int128><<<grid, 256, 0, s>>>(X, R, K, rs, ks, amax_bits, slices,
                                                                             bits, planes, pitch, plane_stride,
                                                                             exps)));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (split_kernel<true, uint64_t><<<grid, 256, 0, s>>>(X, R, K, rs, ks, amax_bits, slices, bits,
                                                                    planes, pitch, plane_stride, exps)));
  } else {
    const int64_t gx = (kchunks + 255) / 256;
    if (R > 65535) {
      // rows beyond the grid's y range: launch in row bands (same planes, same plane stride)
      for (int64_t r0 = 0; r0 < R; r0 += 65535) {
        const int64_t rb = (R - r0 < 65535) ? R - r0 : 65535;
        int rc = oz_split_rows(X + r0 * rs, rb, K, rs, ks, amax_bits + r0, slices, bits, planes + r0 * pitch,
                               pitch, plane_stride, exps + r0, s);
        if (rc) return rc;
      }
      return GB_OK;
    }
    dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(R));
    if (wide)
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (split_kernel<false, unsigned __int128><<<grid, 256, 0, s>>>(X, R, K, rs, ks, amax_bits, slices,
                                                                              bits, planes, pitch, plane_stride,
                                                                              exps)));
    else
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (split_kernel<false, uint64_t><<<grid, 256, 0, s>>>(X, R, K, rs, ks, amax_bits, slices, bits,
                                                                     planes, pitch, plane_stride, exps)));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int oz_split(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks,
             const unsigned long long* amax_bits, int slices, int bits, __nv_bfloat16* planes,
             int64_t pitch, int32_t* exps, cudaStream_t s) {
  return oz_split_rows(X, R, K, rs, ks, amax_bits, slices, bits, planes, pitch, R * pitch, exps, s);
}

// ============================================================== slice products

int oz_gemm_launch(const OzGemmArgs& a, const OzPlan& plan, cudaStream_t s) {
  CUtensorMap ta, tb;
  int rc = make_plane_tmap(&ta, a.planes_a, a.K, a.M, a.slices, a.pitch, TC_BM);
  if (rc) return rc;
  rc = make_plane_tmap(&tb, a.planes_b, a.K, a.N, a.slices, a.pitch, TC_BN);
  if (rc) return rc;
  const bool pair = a.engine == 2;
  TcParams prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.band = a.band;
  TcProblem& P = prm.prob[0];
  P.M = a.M;
  P.N = a.N;
  P.K = a.K;
  P.tiles_m = static_cast<int32_t>(pair ? (a.M + 255) / 256 : (a.M + TC_BM - 1) / TC_BM);
  P.tiles_n = static_cast<int32_t>(pair ? (a.N + 255) / 256 : (a.N + TC_BN - 1) / TC_BN);
  P.tile_begin = 0;
  P.kb_total = plan.kb_total;
  P.nchunks = plan.nchunks;
  P.C = a.C;
  P.ldc = a.ldc;
  P.alpha = a.alpha;
  P.beta = a.beta;
  P.ea = a.ea;
  P.eb = a.eb;
  prm.nprob = 1;
  prm.total_tiles = P.tiles_m * P.tiles_n;
  prm.tws = a.tws;
  prm.status = a.status;
  prm.wait_limit_ns = a.wait_limit_ns;
  if (pair) {
    CUtensorMap tb2;   // B boxes of 128 rows: each CTA of a pair loads half of a 256-row tile
    rc = make_plane_tmap(&tb2, a.planes_b, a.K, a.N, a.slices, a.pitch, 128);
    if (rc) return rc;
    return tc_gemm_pair_launch(TC_EPI_OZAKI_F64, ta, tb2, nullptr, nullptr, plan.sched, prm, a.grid,
                               GB_KERNEL_OZAKI_SLICE_MMA, s);
  }
  return tc_gemm_launch(TC_EPI_OZAKI_F64, ta, tb, nullptr, nullptr, plan.sched, prm, a.grid,
                        GB_KERNEL_OZAKI_SLICE_MMA, s);
}

int oz_grid_for(int sms, int64_t M, int64_t N, int engine) {
  if (engine == 2) {
    const int64_t ctas = 2 * static_cast<int64_t>(tc_pair_tiles(M, N));
    const int64_t cap = sms & ~1;
    return static_cast<int>(ctas < cap ? ctas : cap);
  }
  const int64_t tiles = tc_tiles(M, N);
  return static_cast<int>(tiles < sms ? tiles : sms);
}

}  // namespace gb

namespace gb {
// Relative cost of a plan for one output tile: tensor work (products x K panels) and FP64
// drains (one per group and K chunk) overlap, so the larger dominates.  DRAIN_PANELS is the
// measured cost of draining one 128 x 256 group into the FP64 tile buffer, in units of one
// 64-wide K panel of MMA work (GB300: ~29 us per drain, bound by the FP64 adds, vs ~0.35 us
// per panel).
double oz_plan_cost(const OzPlan& p) {
  constexpr double DRAIN_PANELS = 80.0;
  const double mma = static_cast<double>(p.products) * p.kb_total;
  const double drain = static_cast<double>(p.groups) * p.nchunks * DRAIN_PANELS;
  return (mma > drain ? mma : drain) + 0.1 * (mma < drain ? mma : drain);
}
}  // namespace gb
