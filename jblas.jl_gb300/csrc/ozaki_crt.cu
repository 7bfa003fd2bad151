// FP64-accurate GEMM by the Chinese-remainder method (Ozaki scheme II) on BF16 tensor cores.
//
// Method: K. Ozaki, Y. Uchino and T. Imamura, "Ozaki Scheme II: A GEMM-oriented emulation
// of floating-point matrix multiplication using an integer modular technique" (2025).
//
//   A'[i,k] = round-half-away(op(A)[i,k] * 2^(t - ea_i))    |A'| <= 2^t  (ea_i: row exponent)
//   B'[k,j] = round-half-away(op(B)[k,j] * 2^(t - eb_j))    |B'| <= 2^t
//   C' = A' B' exactly, from its residues modulo n pairwise coprime p_g <= 253:
//     R_g = (A' mod p_g)(B' mod p_g)    balanced residues, |r| <= 126 (exact in BF16); FP32
//                                       sums over K chunks of <= 1024 stay exact (1024 *
//                                       126^2 + 127 < 2^24) and are reduced mod p_g
//     C' = CRT(R_1, ..., R_n)           exact because |C'| <= M/4, M = prod p_g
//   C = alpha * fl(C' * 2^(ea_i + eb_j - 2t)) + beta * C
// Only the rounding of A and B to t-bit integers and the final conversion round; the
// product is exact.  n moduli cost n BF16 GEMMs, against s(s+1)/2 for s digit slices
// (ozaki.cu), which is why this is the faster FP64-accurate mode.
//
// Kernels: crt_split_kernel (residue planes, [modulus][row][pitch] BF16, K-major, read by TMA
// like the digit planes), the CTA-pair slice-product kernel with the TC_EPI_CRT epilogue
// (tc_gemm2.cu: one group per modulus, uint8 residue planes out), crt_combine_kernel
// (reconstruction in 128-bit integer arithmetic, FP64 rounding by integer ops, alpha/beta).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gb_common.cuh"
#include "oz_fixed.cuh"
#include "ozaki.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

// ============================================================== moduli and planner (host)

namespace {

uint32_t gcd_u32(uint32_t a, uint32_t b) {
  while (b) {
    const uint32_t r = a % b;
    a = b;
    b = r;
  }
  return a;
}

// 253 first, then descending integers coprime to every modulus taken so far.  p <= 253
// keeps one FP32 reduction of (chunk sum + running residue) within |r| <= 127.
struct ModuliTable {
  uint32_t p[TC_MAX_MODULI];
  ModuliTable() {
    int cnt = 0;
    for (uint32_t c = 253; cnt < TC_MAX_MODULI; --c) {
      bool ok = true;
      for (int i = 0; i < cnt && ok; ++i) ok = gcd_u32(c, p[i]) == 1;
      if (ok) p[cnt++] = c;
    }
  }
};

const ModuliTable& moduli_table() {
  static const ModuliTable t;
  return t;
}

// Little-endian base-2^32 unsigned integers, for exact planner comparisons.
using Big = std::vector<uint32_t>;

void big_mul_small(Big& a, uint32_t m) {
  uint64_t carry = 0;
  for (auto& w : a) {
    const uint64_t v = static_cast<uint64_t>(w) * m + carry;
    w = static_cast<uint32_t>(v);
    carry = v >> 32;
  }
  if (carry) a.push_back(static_cast<uint32_t>(carry));
}

Big big_u64_shl(uint64_t v, int sh) {
  Big a(static_cast<size_t>(sh / 32) + 3, 0u);
  const int w = sh / 32, b = sh % 32;
  const unsigned __int128 x = static_cast<unsigned __int128>(v) << b;
  a[w] = static_cast<uint32_t>(x);
  a[w + 1] = static_cast<uint32_t>(x >> 32);
  a[w + 2] = static_cast<uint32_t>(x >> 64);
  return a;
}

int big_cmp(Big a, Big b) {
  while (!a.empty() && a.back() == 0) a.pop_back();
  while (!b.empty() && b.back() == 0) b.pop_back();
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

Big moduli_product(int n) {
  Big m{1u};
  for (int g = 0; g < n; ++g) big_mul_small(m, moduli_table().p[g]);
  return m;
}

uint32_t inverse_mod(uint32_t a, uint32_t p) {   // a * x == 1 (mod p), gcd(a, p) = 1
  int64_t t = 0, nt = 1, r = p, nr = a % p;
  while (nr) {
    const int64_t q = r / nr;
    int64_t tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  if (t < 0) t += p;
  return static_cast<uint32_t>(t);
}

}  // namespace

const uint32_t* crt_moduli() { return moduli_table().p; }

double crt_log2_product(int n) {
  double s = 0.0;
  for (int g = 0; g < n; ++g) s += std::log2(static_cast<double>(moduli_table().p[g]));
  return s;
}

int crt_bits_for(int64_t K, int n) {
  if (n < 1 || n > TC_MAX_MODULI) return 0;
  const uint64_t Kb = static_cast<uint64_t>(K < 1 ? 1 : K);
  const Big m = moduli_product(n);
  const Big cap = big_u64_shl(1, 125);
  for (int t = 62; t >= 1; --t) {
    // 4 K 2^(2t) <= M  (so |C'| <= M/4)  and  K 2^(2t) <= 2^125  (C' fits 128-bit words)
    if (big_cmp(big_u64_shl(Kb, 2 * t + 2), m) <= 0 && big_cmp(big_u64_shl(Kb, 2 * t), cap) <= 0) return t;
  }
  return 0;
}

int crt_make_plan(int64_t M, int64_t N, int64_t K, int n, int t, CrtPlan* plan) {
  if (n < 1 || n > TC_MAX_MODULI || t < 0 || t > 62) return GB_ERR_INVALID_VALUE;
  if (t == 0) t = crt_bits_for(K, n);
  if (t < 1) return GB_ERR_UNSUPPORTED;   // too few moduli for this K
  CrtPlan& P = *plan;
  std::memset(&P, 0, sizeof(P));
  P.n = n;
  P.t = t;
  int64_t kb_total = (K + TC_BK - 1) / TC_BK;
  if (kb_total < 1) kb_total = 1;
  // exact FP32 chunk sums: at most 16 panels (1024 products of |r| <= 126)
  int64_t nchunks = (kb_total + 15) / 16;
  const int64_t kb_chunk = (kb_total + nchunks - 1) / nchunks;
  nchunks = (kb_total + kb_chunk - 1) / kb_chunk;
  P.kb_total = static_cast<int32_t>(kb_total);
  P.nchunks = static_cast<int>(nchunks);
  P.k_chunk = kb_chunk * TC_BK;
  P.log2_m = crt_log2_product(n);
  P.flops_tensor = 2.0 * static_cast<double>(M) * static_cast<double>(N) * static_cast<double>(kb_total * TC_BK) * n;

  SliceSchedule& S = P.sched;
  S.ngroups = n;
  S.kb_chunk = static_cast<int32_t>(kb_chunk);
  S.bits = t;
  for (int g = 0; g < n; ++g) {
    S.level[g] = 0;
    S.npairs[g] = 1;
    S.pair_off[g] = static_cast<int16_t>(g);
    S.pp[g] = static_cast<uint8_t>(g);
    S.pq[g] = static_cast<uint8_t>(g);
  }

  CrtConsts& cc = P.cc;
  cc.n = n;
  cc.t = t;
  unsigned __int128 m128 = 1;
  for (int g = 0; g < n; ++g) m128 *= moduli_table().p[g];
  for (int w = 0; w < 4; ++w) cc.m[w] = static_cast<uint32_t>(m128 >> (32 * w));
  unsigned __int128 bias128 = 0;
  double bias_k = 0.0;
  for (int g = 0; g < n; ++g) {
    const uint32_t p = moduli_table().p[g];
    const uint64_t c21 = (uint64_t(1) << 21) % p;
    const uint64_t c42 = (c21 * c21) % p;
    const uint64_t c62 = (c42 * ((uint64_t(1) << 20) % p)) % p;
    cc.p[g] = p;
    cc.c21[g] = static_cast<uint32_t>(c21);
    cc.c42[g] = static_cast<uint32_t>(c42);
    cc.bias[g] = static_cast<uint32_t>((p - c62) % p);
    cc.mg[g] = static_cast<uint32_t>((uint64_t(1) << 32) / p);
    // M / p_g modulo p_g and modulo 2^128
    uint64_t rest_mod_p = 1;
    unsigned __int128 rest128 = 1;
    for (int h = 0; h < n; ++h) {
      if (h == g) continue;
      rest_mod_p = (rest_mod_p * (moduli_table().p[h] % p)) % p;
      rest128 *= moduli_table().p[h];
    }
    const uint32_t inv = inverse_mod(static_cast<uint32_t>(rest_mod_p), p);
    cc.finv[g] = static_cast<float>(static_cast<double>(inv) / static_cast<double>(p));
    const unsigned __int128 w128 = rest128 * inv;
    for (int w = 0; w < 4; ++w) cc.w[g][w] = static_cast<uint32_t>(w128 >> (32 * w));
    bias128 += w128 * 128u;
    bias_k += 128.0 * static_cast<double>(cc.finv[g]);
  }
  for (int w = 0; w < 4; ++w) cc.bw[w] = static_cast<uint32_t>(bias128 >> (32 * w));
  cc.bias_k = static_cast<float>(bias_k);
  return GB_OK;
}

// ============================================================== residue split

// Residue of the two's-complement integer Y (|Y| <= 2^62) modulo p from 21-bit limbs of
// Y + 2^62 (bias folds the 2^62 back out), reduced with a multiply-high by floor(2^32 / p):
// the quotient estimate is low by at most one, so one conditional subtraction finishes.
__device__ __forceinline__ uint32_t residue_of(uint32_t y0, uint32_t y1, uint32_t y2, uint32_t p, uint32_t c21,
                                               uint32_t c42, uint32_t bias, uint32_t mg) {
  const uint32_t s = y0 + y1 * c21 + y2 * c42 + bias;   // < 2^30
  uint32_t r = s - __umulhi(s, mg) * p;                 // in [0, 2p)
  return r >= p ? r - p : r;
}

// One thread = one row r and 16 consecutive k, as in split_kernel; n planes of 16 BF16
// balanced residues (r > p/2 becomes r - p), two 16-byte stores per plane.
template <bool RC>
__global__ void __launch_bounds__(256) crt_split_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                        int64_t rs, int64_t ks,
                                                        const unsigned long long* __restrict__ amax_bits,
                                                        __nv_bfloat16* __restrict__ planes, int64_t pitch,
                                                        int32_t* __restrict__ exps, const __grid_constant__ CrtConsts cc) {
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
  const bool nonfinite = (e == OZ_EXP_NONFINITE);
  const int nvalid = static_cast<int>(K - k0 < 16 ? K - k0 : 16);
  const double* src = X + r * rs + k0 * ks;
  uint32_t y0[16], y1[16], y2[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const double x = (j < nvalid) ? src[j * ks] : 0.0;
    const uint64_t y = (nonfinite ? 0ull : fixed_point<uint64_t>(x, e, cc.t + 1)) + (1ull << 62);
    y0[j] = static_cast<uint32_t>(y) & 0x1FFFFFu;
    y1[j] = static_cast<uint32_t>(y >> 21) & 0x1FFFFFu;
    y2[j] = static_cast<uint32_t>(y >> 42);
  }
  __nv_bfloat16* out0 = planes + r * pitch + k0;
  const int64_t plane_stride = R * pitch;
  for (int g = 0; g < cc.n; ++g) {
    const uint32_t p = cc.p[g], c21 = cc.c21[g], c42 = cc.c42[g], bias = cc.bias[g], mg = cc.mg[g];
    const uint32_t half = p >> 1;
    uint32_t packed[8];
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      const uint32_t r0 = residue_of(y0[j], y1[j], y2[j], p, c21, c42, bias, mg);
      const uint32_t r1 = residue_of(y0[j + 1], y1[j + 1], y2[j + 1], p, c21, c42, bias, mg);
      const int d0 = static_cast<int>(r0) - (r0 > half ? static_cast<int>(p) : 0);
      const int d1 = static_cast<int>(r1) - (r1 > half ? static_cast<int>(p) : 0);
      packed[j / 2] = bf16_bits_of_int(d0) | (bf16_bits_of_int(d1) << 16);
    }
    __nv_bfloat16* dst = out0 + g * plane_stride;
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

int crt_split(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, const unsigned long long* amax_bits,
              const CrtPlan& plan, __nv_bfloat16* planes, int64_t pitch, int32_t* exps, cudaStream_t s) {
  if (R <= 0 || K <= 0) return GB_OK;
  const int64_t kchunks = (K + 15) / 16;
  if (rs == 1 && R > 1) {
    if (kchunks > 65535) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>((R + 255) / 256), static_cast<unsigned>(kchunks));
    GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
              (crt_split_kernel<true><<<grid, 256, 0, s>>>(X, R, K, rs, ks, amax_bits, planes, pitch, exps, plan.cc)));
  } else {
    for (int64_t r0 = 0; r0 < R; r0 += 65535) {   // rows beyond the grid's y range: bands
      const int64_t rb = (R - r0 < 65535) ? R - r0 : 65535;
      dim3 grid(static_cast<unsigned>((kchunks + 255) / 256), static_cast<unsigned>(rb));
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (crt_split_kernel<false><<<grid, 256, 0, s>>>(X + r0 * rs, rb, K, rs, ks, amax_bits + r0,
                                                               planes + r0 * pitch, pitch, exps + r0, plan.cc)));
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ============================================================== reconstruction

// The double nearest (ties to even) to the signed 128-bit integer hi:lo times 2^E.  Normal
// results are assembled from the rounded 53-bit significand in integer arithmetic; results
// outside the normal range round the significand to 53 bits (the 64-bit window keeps a
// sticky bit, so one conversion rounds correctly) and then take one correctly rounded
// power-of-two scaling, as ldexp(double(C'), E) does.
__device__ __forceinline__ double i128_times_pow2(uint64_t hi, uint64_t lo, int E) {
  const bool neg = static_cast<int64_t>(hi) < 0;
  if (neg) {
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
  }
  if ((hi | lo) == 0) return 0.0;
  uint64_t top;
  bool sticky;
  int lead;   // bit position of the leading one
  if (hi) {
    const int lz = __clzll(static_cast<long long>(hi));
    top = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    sticky = lz ? (lo << lz) != 0 : lo != 0;
    lead = 127 - lz;
  } else {
    const int lz = __clzll(static_cast<long long>(lo));
    top = lo << lz;
    sticky = false;
    lead = 63 - lz;
  }
  uint64_t mant = top >> 11;
  const uint64_t rest = top & 0x7FFull;
  const bool up = rest > 0x400ull || (rest == 0x400ull && (sticky || (mant & 1ull)));
  mant += up ? 1ull : 0ull;
  int ex = lead + E;
  if (mant >> 53) {
    mant >>= 1;
    ++ex;
  }
  if (ex >= -1022 && ex <= 1023) {
    const uint64_t bits = (neg ? 0x8000000000000000ull : 0ull) | (static_cast<uint64_t>(ex + 1023) << 52) |
                          (mant & 0x000FFFFFFFFFFFFFull);
    return __longlong_as_double(static_cast<long long>(bits));
  }
  const double d = scale_pow2(__ull2double_rn(top | (sticky ? 1ull : 0ull)), lead - 63 + E);
  return neg ? -d : d;
}

// One thread = 4 consecutive rows of one column (a 32-bit load per residue plane).  The
// planes hold biased bytes u_g = r_g + 128 with r_g = C' mod p_g (|r_g| <= 127), so
//   X = sum_g r_g W_g = sum_g u_g W_g - 128 sum_g W_g   (mod 2^128),
//       W_g = (M/p_g) ((M/p_g)^-1 mod p_g)
//   k = round(sum_g r_g inv_g / p_g) = round(X / M), exact in FP32 because |C'| <= M/4
//   C' = X - k M  (mod 2^128), a two's-complement 128-bit integer
__global__ void __launch_bounds__(256) crt_combine_kernel(const uint8_t* __restrict__ res, int64_t res_ld,
                                                          int64_t res_plane, int64_t M, int64_t N,
                                                          const int32_t* __restrict__ ea,
                                                          const int32_t* __restrict__ eb, double alpha, double beta,
                                                          double* __restrict__ C, int64_t ldc,
                                                          const __grid_constant__ CrtConsts cc) {
  const int64_t i0 = (static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x) * 4;
  if (i0 >= M) return;
  int eai[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) eai[q] = (i0 + q < M) ? ea[i0 + q] : 0;
  const int two_t = 2 * cc.t;
  for (int64_t j = blockIdx.y; j < N; j += gridDim.y) {
    const uint8_t* base = res + j * res_ld + i0;
    uint32_t words[TC_MAX_MODULI];   // all loads in flight before any use
#pragma unroll
    for (int g = 0; g < TC_MAX_MODULI; ++g)
      words[g] = (g < cc.n) ? __ldg(reinterpret_cast<const uint32_t*>(base + g * res_plane)) : 0u;
    uint64_t acc[4][4];
    float ks[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      ks[q] = -cc.bias_k;
#pragma unroll
      for (int w = 0; w < 4; ++w) acc[q][w] = 0ull;
    }
#pragma unroll
    for (int g = 0; g < TC_MAX_MODULI; ++g) {
      if (g >= cc.n) break;
      const uint32_t word = words[g];
      const float fi = cc.finv[g];
      const uint32_t w0 = cc.w[g][0], w1 = cc.w[g][1], w2 = cc.w[g][2], w3 = cc.w[g][3];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t u = (word >> (8 * q)) & 0xFFu;
        ks[q] = fmaf(__uint_as_float(0x4B000000u | u) - 8388608.0f, fi, ks[q]);
        acc[q][0] += static_cast<uint64_t>(u) * w0;
        acc[q][1] += static_cast<uint64_t>(u) * w1;
        acc[q][2] += static_cast<uint64_t>(u) * w2;
        acc[q][3] += static_cast<uint64_t>(u) * w3;
      }
    }
    const int ebj = eb[j];
    double* ccol = C + j * ldc;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (i0 + q >= M) continue;
      const int64_t k = __float_as_int(ks[q] + 12582912.0f) - 0x4B400000;   // round(X / M)
      int64_t c = 0;
      uint32_t word[4];
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int64_t v = static_cast<int64_t>(acc[q][w]) - static_cast<int64_t>(cc.bw[w]) -
                          k * static_cast<int64_t>(cc.m[w]) + c;
        word[w] = static_cast<uint32_t>(v);
        c = v >> 32;
      }
      double val;
      if (eai[q] == OZ_EXP_NONFINITE || ebj == OZ_EXP_NONFINITE) {
        val = __longlong_as_double(0x7FF8000000000000ll);
      } else {
        const uint64_t lo = (static_cast<uint64_t>(word[1]) << 32) | word[0];
        const uint64_t hi = (static_cast<uint64_t>(word[3]) << 32) | word[2];
        val = i128_times_pow2(hi, lo, eai[q] + ebj - two_t);
      }
      if (cc.ab == 1)
        val = alpha * val;
      else if (cc.ab == 2)
        val = fma(alpha, val, beta * ccol[i0 + q]);
      ccol[i0 + q] = val;
    }
  }
}

// ============================================================== driver

int crt_gemm_launch(const CrtGemmArgs& a, const CrtPlan& plan, cudaStream_t s) {
  CUtensorMap ta, tb;
  int rc = make_plane_tmap(&ta, a.planes_a, a.K, a.M, plan.n, a.pitch, 128);
  if (rc) return rc;
  rc = make_plane_tmap(&tb, a.planes_b, a.K, a.N, plan.n, a.pitch, 128);
  if (rc) return rc;
  TcParams prm;
  std::memset(&prm, 0, sizeof(prm));
  TcProblem& P = prm.prob[0];
  P.M = a.M;
  P.N = a.N;
  P.K = a.K;
  P.tiles_m = static_cast<int32_t>((a.M + 255) / 256);
  P.tiles_n = static_cast<int32_t>((a.N + 255) / 256);
  P.tile_begin = 0;
  P.kb_total = plan.kb_total;
  P.nchunks = plan.nchunks;
  prm.nprob = 1;
  prm.total_tiles = P.tiles_m * P.tiles_n;
  prm.status = a.status;
  prm.wait_limit_ns = a.wait_limit_ns;
  prm.res = a.res;
  prm.res_ld = a.res_ld;
  prm.res_plane = a.res_plane;
  for (int g = 0; g < plan.n; ++g) {
    prm.crt_p[g] = static_cast<float>(plan.cc.p[g]);
    prm.crt_inv[g] = 1.0f / static_cast<float>(plan.cc.p[g]);
  }
  rc = tc_gemm_pair_launch(TC_EPI_CRT, ta, tb, nullptr, nullptr, plan.sched, prm, a.grid, GB_KERNEL_OZAKI_SLICE_MMA, s);
  if (rc) return rc;
  const int64_t bx = (a.M + 1023) / 1024;
  const int64_t by = a.N < 65535 ? a.N : 65535;
  if (bx > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
  dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(by));
  CrtConsts cc = plan.cc;   // output rule decided once on the host (no FP64 compares per element)
  cc.ab = (a.beta != 0.0) ? 2 : (a.alpha != 1.0 ? 1 : 0);
  GB_LAUNCH(GB_KERNEL_OZAKI_COMBINE, s,
            (crt_combine_kernel<<<grid, 256, 0, s>>>(a.res, a.res_ld, a.res_plane, a.M, a.N, a.ea, a.eb, a.alpha, a.beta,
                                                     a.C, a.ldc, cc)));
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
