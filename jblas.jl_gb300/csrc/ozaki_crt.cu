// FP64-accurate GEMM by the Chinese-remainder method (Ozaki scheme II) on BF16 tensor cores.
//
// Method: K. Ozaki, Y. Uchino and T. Imamura, "Ozaki Scheme II: A GEMM-oriented emulation
// of floating-point matrix multiplication using an integer modular technique" (2025).
//
//   A'[i,k] = round-half-away(op(A)[i,k] * 2^(t - ea_i))    |A'| <= 2^t  (ea_i: row exponent)
//   B'[k,j] = round-half-away(op(B)[k,j] * 2^(t - eb_j))    |B'| <= 2^t
//   C' = A' B' exactly, from its residues modulo n pairwise coprime p_g <= 253:
//     R_g = (A' mod p_g)(B' mod p_g)    residues |r| <= 127 (exact in BF16); FP32 sums over
//                                       K chunks of <= 1024 stay exact (1024 * 127^2 + 127
//                                       < 2^24) and are reduced mod p_g
//     C' = CRT(R_1, ..., R_n)           exact because |C'| <= M/4, M = prod p_g
//   C = alpha * fl(C' * 2^(ea_i + eb_j - 2t)) + beta * C
// Only the rounding of A and B to t-bit integers and the final conversion round; the
// product is exact.  n moduli cost n BF16 GEMMs, against s(s+1)/2 for s digit slices
// (ozaki.cu), which is why this is the faster FP64-accurate mode.
//
// Kernels: crt_split_kc_kernel / crt_split_rc_kernel (residue planes, [modulus][row][pitch]
// BF16, K-major, read by TMA like the digit planes; k-contiguous and row-contiguous operands), the CTA-pair slice-product kernel with the TC_EPI_CRT epilogue
// (tc_gemm2.cu: one group per modulus, uint8 residue planes out), crt_combine_kernel
// (reconstruction in 128-bit integer arithmetic, FP64 rounding by integer ops, alpha/beta).
#include <cuda_bf16.h>

#include <cmath>
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
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

uint64_t inverse_mod64(uint64_t a, uint64_t m) {   // a * x == 1 (mod m), gcd(a, m) = 1, m < 2^31
  int64_t t = 0, nt = 1, r = static_cast<int64_t>(m), nr = static_cast<int64_t>(a % m);
  while (nr) {
    const int64_t q = r / nr;
    int64_t tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  if (t < 0) t += static_cast<int64_t>(m);
  return static_cast<uint64_t>(t);
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

namespace {
CrtTable build_table() {
  CrtTable tab;
  std::memset(&tab, 0, sizeof(tab));
  CrtModuli& md = tab.mod;
  for (int g = 0; g < TC_MAX_MODULI; ++g) {
    const uint32_t p = moduli_table().p[g];
    md.p[g] = p;
    md.pf[g] = static_cast<float>(p);
    md.pinv[g] = 1.0f / static_cast<float>(p);
    uint64_t pw = 1;   // 2^(14 (l + 1)) mod p, taken in (-p/2, p/2]
    for (int l = 0; l < 3; ++l) {
      pw = (pw << 14) % p;
      md.climb4[g][l] = static_cast<float>(2 * pw > p ? static_cast<int64_t>(pw) - static_cast<int64_t>(p)
                                                      : static_cast<int64_t>(pw));
    }
    pw = 1;   // 2^(13 (l + 1)) mod p
    for (int l = 0; l < 4; ++l) {
      pw = (pw << 13) % p;
      md.climb5[g][l] = static_cast<float>(pw);
    }
  }
  for (int n = 1; n <= TC_MAX_MODULI; ++n) {
    CrtRecon& rc = tab.rec[n - 1];
    const uint32_t* p = moduli_table().p;
    unsigned __int128 m128 = 1;
    for (int g = 0; g < n; ++g) m128 *= p[g];
    for (int w = 0; w < 4; ++w) rc.m[w] = static_cast<uint32_t>(m128 >> (32 * w));
    rc.ngroups = (n + 2) / 3;
    double ks0 = 0.0;
    for (int G = 0; G < rc.ngroups; ++G) {
      const int a = 3 * G, b = a + 1, c = a + 2;
      uint64_t P = p[a];
      if (b < n) P *= p[b];
      if (c < n) P *= p[c];
      // M / P_G modulo P_G and modulo 2^128
      uint64_t rest_mod = 1;
      unsigned __int128 rest128 = 1;
      for (int h = 0; h < n; ++h) {
        if (h >= a && h <= c) continue;
        rest_mod = (rest_mod * (p[h] % P)) % P;
        rest128 *= p[h];
      }
      const uint64_t psi = inverse_mod64(rest_mod, P);
      for (int g = a; g <= c && g < n; ++g) rc.psi[g] = static_cast<float>(psi % p[g]);
      rc.pa[G] = static_cast<float>(p[a]);
      rc.a1[G] = (b < n) ? static_cast<float>(inverse_mod(p[a] % p[b], p[b])) : 0.0f;
      rc.pab[G] = (b < n) ? static_cast<float>(p[a] * p[b]) : 0.0f;
      rc.a2[G] = (c < n) ? static_cast<float>(inverse_mod(static_cast<uint32_t>((uint64_t(p[a]) * p[b]) % p[c]), p[c]))
                         : 0.0f;
      rc.P[G] = static_cast<float>(P);
      rc.Pinv[G] = 1.0f / static_cast<float>(P);
      rc.voff[G] = static_cast<int32_t>(static_cast<int64_t>(P) - 8388736);
      ks0 += (static_cast<double>(P) - 8388736.0) / static_cast<double>(P);
      for (int w = 0; w < 4; ++w) rc.w[G][w] = static_cast<uint32_t>(rest128 >> (32 * w));
    }
    rc.ks0 = static_cast<float>(ks0);
  }
  return tab;
}
}  // namespace

const CrtTable& crt_table() {
  static const CrtTable tab = build_table();
  return tab;
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
  // exact FP32 chunk sums: at most 16 panels (1024 products of |r| <= 127)
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

  return GB_OK;
}

// ============================================================== device table and plans

namespace {
struct CrtDeviceState {
  CrtPlanRecord* ring = nullptr;
  std::atomic<unsigned long long> next{0};
};
std::mutex g_crt_mu;
std::vector<std::unique_ptr<CrtDeviceState>> g_crt_dev;
}  // namespace

int crt_plan_record(CrtPlanRecord** record, unsigned long long* seq) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  CrtDeviceState* st = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_crt_mu);
    if (static_cast<int>(g_crt_dev.size()) <= dev) g_crt_dev.resize(dev + 1);
    if (!g_crt_dev[dev]) {
      auto fresh = std::make_unique<CrtDeviceState>();
      GB_CUDA_TRY(cudaMalloc(&fresh->ring, sizeof(CrtPlanRecord) * CRT_PLAN_RING));
      GB_CUDA_TRY(cudaMemset(fresh->ring, 0xFF, sizeof(CrtPlanRecord) * CRT_PLAN_RING));   // no call's tag
      g_crt_dev[dev] = std::move(fresh);
    }
    st = g_crt_dev[dev].get();
  }
  const unsigned long long k = st->next.fetch_add(1);
  *record = st->ring + (k % CRT_PLAN_RING);
  *seq = k;
  return GB_OK;
}

// ---------------------------------------------------------------- planner
// Restates, on the device, the one-sided bounds of the statistics (the FP32 K-slice sums are
// rescaled to each row's exponent; |x| sums rounded up, x^2 sums rounded down), then picks
//   t(n)  largest t <= 62 with |C'| <= 2^(2t) (min(max sa, max sb) + K 2^(-t-1)) <= M_n / 4
//         and <= 2^125 (checked in log2 with a safety margin)
//   bound(t) = 1.01 (h (EA SB + EB SA) + K h^2 EA EB + 2u (na nb + trunc)) / (na nb),
//         h = 2^(-t-1): rounding A and B to the 2^(e - t) grid moves each element by at most
//         h 2^e; the integer product is exact; the FP64 conversion and alpha round once each
//   n     the fewest moduli with bound(t(n)) <= tol (or pp.n_fixed with t = pp.t_fixed).
// Many blocks reduce row ranges (sums relative to the block's largest row exponent); the
// last block to finish combines them in block order and chooses the plan.  Terms smaller
// than 2^-1022 of the largest are dropped: far inside the 1.01 slack of the bound.
constexpr int CRT_PLAN_THREADS = 256;
constexpr int CRT_PLAN_BLOCKS = 128;   // per operand at most

struct CrtPlanPartial {
  double e2, s2, n2, smax;   // sums of 4^(e - ref), (sa 2^(e - ref))^2, x^2 sums, max sa
  int32_t ref, nonfinite, any, pad;
};

size_t crt_plan_scratch_bytes() { return sizeof(CrtPlanPartial) * 2 * CRT_PLAN_BLOCKS + 256; }

__device__ __forceinline__ int exp_of_bits_dev(unsigned long long bits) {
  if (bits >= 0x7FF0000000000000ull) return 0x7FFFFFFF;
  if (bits == 0) return 0;
  return ilogb(__longlong_as_double(static_cast<long long>(bits))) + 1;
}

// 2^k for k <= 1023; 0 below the normal range.
__device__ __forceinline__ double pow2_or_zero(int k) {
  return k < -1022 ? 0.0 : __longlong_as_double(static_cast<long long>(k + 1023) << 52);
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ double crt_bound_dev(bool nonfinite, double na, double nb, double EA, double EB, double SA, double SB,
                                int64_t K, int t) {
  if (nonfinite) return INFINITY;
  if (na == 0.0 || nb == 0.0) return 0.0;
  const double h = ldexp(1.0, -t - 1);
  const double Kd = static_cast<double>(K);
  const double trunc = h * (EA * SB + EB * SA) + Kd * h * h * EA * EB;
  const double fin = 2.0 * 0x1p-53 * (na * nb + trunc);
  return 1.01 * (trunc + fin) / (na * nb);
}

__device__ int crt_bits_dev(double sa_max, double sb_max, int64_t K, double lm) {
  const double Kd = static_cast<double>(K < 1 ? 1 : K);
  // S(t) >= min(sa_max, sb_max, K): start from the t that bound allows and step down
  const double ls = log2(fmin(fmin(sa_max, sb_max), Kd));
  int t0 = 62;
  const double cap = fmin(lm - 2.0, 125.0) - ls;
  if (cap < 124.0) t0 = min(62, static_cast<int>(floor(cap * 0.5)) + 1);
  for (int t = t0; t >= 1; --t) {
    double S = fmin(sa_max, sb_max) + Kd * ldexp(1.0, -t - 1);
    S = fmin(S, Kd) * (1.0 + 1e-12);
    const double need = 2.0 * t + log2(S);
    if (need + 2.0 <= lm - 1e-9 && need <= 125.0 - 1e-9) return t;
  }
  return 0;
}

__global__ void __launch_bounds__(CRT_PLAN_THREADS) crt_plan_kernel(const OzRowStats sa, const OzRowStats sb,
                                                                    const __grid_constant__ CrtPlanParams pp,
                                                                    int blocks_a, CrtPlanPartial* __restrict__ part,
                                                                    unsigned int* __restrict__ counter,
                                                                    CrtDevicePlan* __restrict__ out,
                                                                    CrtPlanRecord* __restrict__ record,
                                                                    unsigned long long seq) {
  __shared__ int s_ref[CRT_PLAN_THREADS / 32], s_nf[CRT_PLAN_THREADS / 32];
  __shared__ double s_acc[4][CRT_PLAN_THREADS / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (!pp.with_sums) {   // fixed plan, no bound asked for
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      out->n = pp.n_fixed;
      out->t = pp.t_fixed;
      out->bound = __longlong_as_double(0x7FF8000000000000ll);
      record->plan = *out;
      record->seq = seq;
    }
    return;
  }
  const bool is_b = static_cast<int>(blockIdx.x) >= blocks_a;
  const OzRowStats& st = is_b ? sb : sa;
  const int64_t R = is_b ? pp.N : pp.M;
  const int nb = is_b ? gridDim.x - blocks_a : blocks_a;
  const int bi = is_b ? blockIdx.x - blocks_a : blockIdx.x;
  const int64_t per = (R + nb - 1) / nb;
  const int64_t r0 = bi * per, r1 = (r0 + per < R) ? r0 + per : R;
  // block's reference exponent and non-finite flag
  int ref = -1100, nf = 0;
  for (int64_t i = r0 + threadIdx.x; i < r1; i += CRT_PLAN_THREADS) {
    const unsigned long long b = st.amax_bits[i];
    const int e = exp_of_bits_dev(b);
    if (e == 0x7FFFFFFF) nf = 1;
    else if (b && e > ref) ref = e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ref = max(ref, __shfl_xor_sync(0xffffffffu, ref, o));
    nf |= __shfl_xor_sync(0xffffffffu, nf, o);
  }
  if (lane == 0) {
    s_ref[wid] = ref;
    s_nf[wid] = nf;
  }
  __syncthreads();
  ref = -1100;
  nf = 0;
  for (int w = 0; w < CRT_PLAN_THREADS / 32; ++w) {
    ref = max(ref, s_ref[w]);
    nf |= s_nf[w];
  }
  // one-sided row sums, as the host bound restates them
  const double Kd = static_cast<double>(pp.K);
  const double gk = Kd * 0x1p-24;
  const double up = (gk < 0.5 ? (1.0 + 0x1p-23) / (1.0 - gk) : 4.0) * (1.0 + 0x1p-40);
  const double down = (1.0 - 0x1p-40) / (1.0 + 2.0 * gk);
  const double tiny = Kd * 0x1p-126;
  double e2 = 0.0, s2 = 0.0, n2 = 0.0, smax = 0.0;
  if (!nf) {
    for (int64_t i = r0 + threadIdx.x; i < r1; i += CRT_PLAN_THREADS) {
      const unsigned long long b = st.amax_bits[i];
      if (!b) continue;
      const int e = exp_of_bits_dev(b);
      double sabs = 0.0, ssq = 0.0;
      for (int sl = 0; sl < st.kslices; ++sl) {
        const int64_t o = static_cast<int64_t>(sl) * R + i;
        const int pe = st.part_e[o];
        if (pe == 0x7FFFFFFF) continue;
        sabs += static_cast<double>(st.part_sa[o]) * pow2_or_zero(pe - e);
        ssq += static_cast<double>(st.part_sq[o]) * pow2_or_zero(2 * (pe - e));
      }
      const double su = sabs * up + tiny;
      const double sc = pow2_or_zero(e - ref);
      e2 += sc * sc;
      s2 += (su * sc) * (su * sc);
      n2 += ssq * down * (sc * sc);
      smax = fmax(smax, su);
    }
  }
  e2 = warp_sum(e2);
  s2 = warp_sum(s2);
  n2 = warp_sum(n2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  __syncthreads();
  if (lane == 0) {
    s_acc[0][wid] = e2;
    s_acc[1][wid] = s2;
    s_acc[2][wid] = n2;
    s_acc[3][wid] = smax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    CrtPlanPartial pt;
    pt.e2 = pt.s2 = pt.n2 = pt.smax = 0.0;
    for (int w = 0; w < CRT_PLAN_THREADS / 32; ++w) {
      pt.e2 += s_acc[0][w];
      pt.s2 += s_acc[1][w];
      pt.n2 += s_acc[2][w];
      pt.smax = fmax(pt.smax, s_acc[3][w]);
    }
    pt.ref = ref;
    pt.nonfinite = nf;
    pt.any = (ref > -1100) ? 1 : 0;
    pt.pad = 0;
    part[blockIdx.x] = pt;
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last || threadIdx.x >= 32) return;
  __threadfence();
  // last block, warp 0: combine the partials of each operand (lane l takes blocks l, l + 32, ...;
  // butterfly reductions leave the same sums in every lane), then lane c - 1 evaluates c moduli
  // and a ballot picks the fewest that pass
  double nrm[2], E[2], S[2], smx[2];
  int nonfinite = 0;
#pragma unroll
  for (int op = 0; op < 2; ++op) {
    const int b0 = op ? blocks_a : 0, b1 = op ? static_cast<int>(gridDim.x) : blocks_a;
    int gref = -1100, nfl = 0;
    for (int b = b0 + lane; b < b1; b += 32) {
      const CrtPlanPartial& q = part[b];
      nfl |= q.nonfinite;
      if (q.any && q.ref > gref) gref = q.ref;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      gref = max(gref, __shfl_xor_sync(0xffffffffu, gref, o));
      nfl |= __shfl_xor_sync(0xffffffffu, nfl, o);
    }
    nonfinite |= nfl;
    double ae2 = 0.0, as2 = 0.0, an2 = 0.0, amx = 0.0;
    for (int b = b0 + lane; b < b1; b += 32) {
      const CrtPlanPartial& q = part[b];
      if (!q.any) continue;
      const double f = pow2_or_zero(2 * (q.ref - gref));
      ae2 += q.e2 * f;
      as2 += q.s2 * f;
      an2 += q.n2 * f;
      amx = fmax(amx, q.smax);
    }
    ae2 = warp_sum(ae2);
    as2 = warp_sum(as2);
    an2 = warp_sum(an2);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amx = fmax(amx, __shfl_xor_sync(0xffffffffu, amx, o));
    nrm[op] = sqrt(an2);
    E[op] = sqrt(ae2);
    S[op] = sqrt(as2);
    smx[op] = amx;
  }
  int n = pp.n_fixed, t = pp.t_fixed;
  if (n == 0) {
    const int c = lane + 1;
    int tc = 0;
    bool ok = false;
    if (c <= TC_MAX_MODULI) {
      tc = nonfinite ? pp.tk[c] : crt_bits_dev(smx[0], smx[1], pp.K, pp.log2m[c]);
      ok = tc >= 1 && (nonfinite || crt_bound_dev(false, nrm[0], nrm[1], E[0], E[1], S[0], S[1], pp.K, tc) <= pp.tol);
    }
    const unsigned pass = __ballot_sync(0xffffffffu, ok);
    const int tmax = __shfl_sync(0xffffffffu, tc, TC_MAX_MODULI - 1);
    if (pass) {
      const int first = __ffs(pass) - 1;
      n = first + 1;
      t = __shfl_sync(0xffffffffu, tc, first);
    } else {   // tolerance out of reach: the most moduli
      n = TC_MAX_MODULI;
      t = tmax >= 1 ? tmax : pp.tk[n];
    }
  }
  if (lane == 0) {
    out->n = n;
    out->t = t;
    out->bound = crt_bound_dev(nonfinite, nrm[0], nrm[1], E[0], E[1], S[0], S[1], pp.K, t);
    record->plan = *out;
    record->seq = seq;
    *counter = 0u;
  }
}

int crt_plan_device(const OzRowStats& sa, const OzRowStats& sb, const CrtPlanParams& pp, CrtDevicePlan* plan,
                    CrtPlanRecord* record, unsigned long long seq, void* scratch, cudaStream_t s) {
  auto blocks_for = [](int64_t R) {
    int64_t b = (R + CRT_PLAN_THREADS - 1) / CRT_PLAN_THREADS;
    if (b > CRT_PLAN_BLOCKS) b = CRT_PLAN_BLOCKS;
    return static_cast<int>(b < 1 ? 1 : b);
  };
  const int ba = blocks_for(pp.M), bb = blocks_for(pp.N);
  CrtPlanPartial* part = static_cast<CrtPlanPartial*>(scratch);
  unsigned int* counter = reinterpret_cast<unsigned int*>(static_cast<char*>(scratch) +
                                                          sizeof(CrtPlanPartial) * 2 * CRT_PLAN_BLOCKS);
  GB_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  GB_LAUNCH(GB_KERNEL_OZAKI_STATS, s,
            (crt_plan_kernel<<<ba + bb, CRT_PLAN_THREADS, 0, s>>>(sa, sb, pp, ba, part, counter, plan, record,
                                                                   seq)));
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ============================================================== residue split

// round-half-away(x 2^(SB - 53 + ex - e)) as a two's-complement word, for the CRT split
// (SB = t + 1 <= 63, every |x| < 2^e).  A subnormal significand is first normalised (its
// leading bit moved to bit 52, the exponent lowered to match), so 2^ex <= |x| < 2^e and the
// shift sh = ex - 53 + SB - e is at most 9: the significand is placed at bit 9 once and only
// ever shifted right (by 9 - sh, with rounding).  Equal to fixed_point<uint64_t> for these
// arguments, without its branches.
__device__ __forceinline__ uint64_t crt_fixed_point(double x, int e, int SB) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
  const int biased = static_cast<int>((bits >> 52) & 0x7FF);
  const unsigned long long frac = bits & 0x000FFFFFFFFFFFFFull;
  const int lz = biased ? 0 : __clzll(static_cast<long long>(frac)) - 11;   // <= 53 (frac == 0: 53)
  const unsigned long long m = biased ? (frac | 0x0010000000000000ull) : (frac << lz);
  const int ex = biased ? biased - 1023 : -1022 - lz;
  const int s = 9 - (ex - 53 + SB - e);   // >= 0 whenever m != 0
  const unsigned long long m9 = m << 9;   // < 2^62
  unsigned long long mag = 0;
  if (s < 64) mag = s <= 0 ? m9 : (m9 + (1ull << (s - 1))) >> s;
  return (bits >> 63) ? 0ull - mag : mag;
}

// Balanced digits of Y = round-half-away(x 2^(t - e)) (|Y| <= 2^t), as exact FP32 values.
//   ND = 4 (t <= 52): Y = d_0 + d_1 2^14 + d_2 2^28 + d_3 2^42, d_0..d_2 in [-8192, 8191],
//        |d_3| <= 1024: the fields of Y + 8192 (1 + 2^14 + 2^28) and its signed top bits
//   ND = 5 (t <= 62): Y = sum_{l<4} d_l 2^(13 l) + d_4 2^52, d_0..d_3 in [-4096, 4095],
//        |d_4| <= 1024: the fields of Y + 4096 (1 + 2^13 + 2^26 + 2^39) and its top bits
template <int ND>
__device__ __forceinline__ void crt_digits(double x, int e, int tbits, bool nonfinite, float (&d)[ND]) {
  constexpr int W = (ND == 4) ? 14 : 13;
  constexpr uint32_t MASK = (1u << W) - 1u, H = 1u << (W - 1);
  constexpr float DBIAS = 8388608.0f + static_cast<float>(H);
  constexpr unsigned long long BAL = (ND == 4) ? 8192ull * (1ull + (1ull << 14) + (1ull << 28))
                                               : 4096ull * (1ull + (1ull << 13) + (1ull << 26) + (1ull << 39));
  const uint64_t u = (nonfinite ? 0ull : crt_fixed_point(x, e, tbits + 1)) + BAL;
  const uint32_t lo = static_cast<uint32_t>(u), hi = static_cast<uint32_t>(u >> 32);
#pragma unroll
  for (int l = 0; l < ND - 1; ++l) {
    const int sh = W * l;
    const uint32_t field = (sh < 32 ? __funnelshift_r(lo, hi, sh) : hi >> (sh - 32)) & MASK;
    d[l] = __uint_as_float(0x4B000000u | field) - DBIAS;
  }
  const uint32_t top = static_cast<uint32_t>(static_cast<int32_t>(hi) >> (W * (ND - 1) - 32)) + H;
  d[ND - 1] = __uint_as_float(0x4B000000u | (top & MASK)) - DBIAS;
}

// Residues of 8 elements (digits d[.][j]) modulo p, packed as BF16 pairs.  Per element
//   s = d_0 + sum_{l>=1} d_l c_l     ND = 4: c_l = 2^(14 l) mod p in (-p/2, p/2],
//                                      |s| <= 8192 (1 + 2 * 126) + 1024 * 126 < 2^22;
//                                    ND = 5: c_l = 2^(13 l) mod p in [0, p),
//                                      |s| <= 4096 (1 + 3 * 252) + 1024 * 252 < 2^22;
//                                    exact in FP32 (ND - 1 FMAs)
//   r = s - p rint(s / p)            |r| <= p/2 + 1/2, so |r| <= 127
// all on the FMA pipe; r has at most 7 significant bits, so its BF16 is the upper half of its
// FP32 bits.
template <int ND>
__device__ __forceinline__ uint4 crt_residues8(const float (&d)[ND][8], const CrtModuli& mod, int g) {
  constexpr float MAGIC = 12582912.0f;   // 1.5 * 2^23: x + MAGIC - MAGIC = rint(x), |x| < 2^22
  float c[ND - 1];
#pragma unroll
  for (int l = 0; l < ND - 1; ++l) c[l] = (ND == 4) ? mod.climb4[g][l] : mod.climb5[g][l];
  const float pf = mod.pf[g], inv = mod.pinv[g];
  uint32_t packed[4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    float rr[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float sj = d[0][j + h];
#pragma unroll
      for (int l = 1; l < ND; ++l) sj = fmaf(d[l][j + h], c[l - 1], sj);
      const float q = fmaf(sj, inv, MAGIC) - MAGIC;
      rr[h] = fmaf(-pf, q, sj);
    }
    packed[j / 2] = __byte_perm(__float_as_uint(rr[0]), __float_as_uint(rr[1]), 0x7632u);
  }
  return make_uint4(packed[0], packed[1], packed[2], packed[3]);
}

__device__ __forceinline__ void store_residues(__nv_bfloat16* dst, uint4 v, int nvalid) {
  if (nvalid == 8) {
    *reinterpret_cast<uint4*>(dst) = v;
  } else {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    unsigned short* d2 = reinterpret_cast<unsigned short*>(dst);
    for (int j = 0; j < nvalid; ++j) d2[j] = static_cast<unsigned short>(w[j / 2] >> (16 * (j & 1)));
  }
}

// Digits and residue planes of 8 consecutive k of one row: plane g at out0 + g * plane_stride.
template <int ND>
__device__ __forceinline__ void crt_split8(const double (&x)[8], int e, int tbits, bool nonfinite, int nmod,
                                           const CrtModuli& mod, __nv_bfloat16* out0, int64_t plane_stride,
                                           int nvalid) {
  float d[ND][8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float dj[ND];
    crt_digits<ND>(x[j], e, tbits, nonfinite, dj);
#pragma unroll
    for (int l = 0; l < ND; ++l) d[l][j] = dj[l];
  }
  // The moduli counts automatic plans pick for FP64 data (t = 52) run a straight loop whose
  // table constants are immediate operands; other counts loop over the planes.
  if (ND == 4) {
    switch (nmod) {
#define GB_CRT_SPLIT_CASE(n)                                                                          \
  case n: {                                                                                           \
    _Pragma("unroll") for (int g = 0; g < n; ++g)                                                     \
        store_residues(out0 + g * plane_stride, crt_residues8<ND>(d, mod, g), nvalid);                \
    return;                                                                                           \
  }
      GB_CRT_SPLIT_CASE(14) GB_CRT_SPLIT_CASE(15) GB_CRT_SPLIT_CASE(16)
#undef GB_CRT_SPLIT_CASE
      default: break;
    }
  }
  for (int g = 0; g < nmod; ++g) store_residues(out0 + g * plane_stride, crt_residues8<ND>(d, mod, g), nvalid);
}

// k contiguous: one thread = one row and 8 consecutive k, neighbouring threads neighbouring k
// (a warp reads 2 KB and writes 512 B of one row per plane).  One 16-byte store per plane.
__global__ void __launch_bounds__(256) crt_split_kc_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                           int64_t rs, int64_t ks,
                                                           const unsigned long long* __restrict__ amax_bits,
                                                           __nv_bfloat16* __restrict__ planes, int64_t pitch,
                                                           int64_t plane_stride, int32_t* __restrict__ exps,
                                                           const __grid_constant__ CrtModuli mod,
                                                           const CrtDevicePlan* __restrict__ plan) {
  const int64_t kc = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x, r = blockIdx.y;
  const int64_t k0 = kc * 8;
  if (r >= R || k0 >= K) return;
  const int nmod = plan->n, tbits = plan->t;
  const int e = row_exponent(amax_bits[r]);
  if (k0 == 0) exps[r] = e;
  const bool nonfinite = (e == OZ_EXP_NONFINITE);
  const int nvalid = static_cast<int>(K - k0 < 8 ? K - k0 : 8);
  const double* src = X + r * rs + k0 * ks;
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = (j < nvalid) ? src[j * ks] : 0.0;
  __nv_bfloat16* out0 = planes + r * pitch + k0;
  if (tbits <= 52) crt_split8<4>(x, e, tbits, nonfinite, nmod, mod, out0, plane_stride, nvalid);
  else crt_split8<5>(x, e, tbits, nonfinite, nmod, mod, out0, plane_stride, nvalid);
}

// Rows contiguous (element (r, k) at X[r + k ks]): warp w of a CTA owns rows 4w..4w+3 of a
// 32-row x 64-k tile; lane l takes row 4w + l / 8 and the 8 consecutive k of chunk l % 8.  Each
// of its 8 loads is one 8-byte element, and a warp's load instruction reads 8 whole 32-byte
// sectors (4 rows of one column, 8 columns); per modulus a warp stores 4 rows x 128 bytes of
// the plane, whole lines.  No shared memory and no barriers: the residue work of one modulus
// overlaps the stores of the previous one.
__global__ void __launch_bounds__(256) crt_split_rc_kernel(const double* __restrict__ X, int64_t R, int64_t K,
                                                           int64_t ks, const unsigned long long* __restrict__ amax_bits,
                                                           __nv_bfloat16* __restrict__ planes, int64_t pitch,
                                                           int64_t plane_stride, int32_t* __restrict__ exps,
                                                           const __grid_constant__ CrtModuli mod,
                                                           const CrtDevicePlan* __restrict__ plan) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t r = static_cast<int64_t>(blockIdx.x) * 32 + 4 * w + (lane >> 3);
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * 64 + 8 * (lane & 7);
  if (r >= R || k0 >= K) return;
  const int nmod = plan->n, tbits = plan->t;
  const int e = row_exponent(amax_bits[r]);
  if (k0 == 0) exps[r] = e;
  const bool nonfinite = (e == OZ_EXP_NONFINITE);
  const int nvalid = static_cast<int>(K - k0 < 8 ? K - k0 : 8);
  const double* src = X + r + k0 * ks;
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = (j < nvalid) ? src[j * ks] : 0.0;
  __nv_bfloat16* out0 = planes + r * pitch + k0;
  if (tbits <= 52) crt_split8<4>(x, e, tbits, nonfinite, nmod, mod, out0, plane_stride, nvalid);
  else crt_split8<5>(x, e, tbits, nonfinite, nmod, mod, out0, plane_stride, nvalid);
}

int crt_split(const double* X, int64_t R, int64_t K, int64_t rs, int64_t ks, const unsigned long long* amax_bits,
              const CrtDevicePlan* plan, __nv_bfloat16* planes, int64_t pitch, int64_t plane_rows, int32_t* exps,
              cudaStream_t s) {
  const CrtModuli& mod = crt_table().mod;
  if (R <= 0 || K <= 0) return GB_OK;
  if (plane_rows < R) return GB_ERR_INVALID_VALUE;
  const int64_t plane_stride = plane_rows * pitch;   // modulus planes of the whole operand
  if (rs == 1 && R > 1) {
    const int64_t gy = (K + 63) / 64;
    if (gy > 65535 || (R + 31) / 32 > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
    dim3 grid(static_cast<unsigned>((R + 31) / 32), static_cast<unsigned>(gy));
    GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
              (crt_split_rc_kernel<<<grid, 256, 0, s>>>(X, R, K, ks, amax_bits, planes, pitch, plane_stride, exps,
                                                        mod, plan)));
  } else {
    const int64_t kchunks = (K + 7) / 8;
    for (int64_t r0 = 0; r0 < R; r0 += 65535) {   // rows beyond the grid's y range: bands
      const int64_t rb = (R - r0 < 65535) ? R - r0 : 65535;
      dim3 grid(static_cast<unsigned>((kchunks + 255) / 256), static_cast<unsigned>(rb));
      GB_LAUNCH(GB_KERNEL_OZAKI_SPLIT, s,
                (crt_split_kc_kernel<<<grid, 256, 0, s>>>(X + r0 * rs, rb, K, rs, ks, amax_bits + r0,
                                                          planes + r0 * pitch, pitch, plane_stride, exps + r0, mod,
                                                          plan)));
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ============================================================== reconstruction

// The double nearest (ties to even) to the signed 128-bit integer hi:lo times 2^E.  The top 64
// bits from the leading one, with a sticky bit for everything below, round to 53 bits (ties to
// even, in integer arithmetic); a normal result then only needs its exponent moved
// (an integer add on the bits), and results outside the normal range take one correctly
// rounded power-of-two scaling of that double, as ldexp(double(C'), E) does.
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
  // round the 64-bit window (sticky bit folded into its last place) to 53 bits, ties to even, by
  // integer operations (GB300's FP64 pipe, which a u64 -> f64 conversion would use, is narrow):
  // the bits of a double in [2^63, 2^64] are (1085 << 52) + the rounded 53-bit significand,
  // whose carry out of bit 52 (a window rounded up to 2^64) lands in the exponent field.
  const uint64_t win = top | (sticky ? 1ull : 0ull);
  const uint64_t mant = win >> 11;
  const uint32_t below = static_cast<uint32_t>(win) & 0x7FFu;
  const long long db = (1085ll << 52) + static_cast<long long>(mant + ((below + (mant & 1u)) > 0x400u ? 1u : 0u));
  const int shift = lead - 63 + E;
  const int exf = static_cast<int>(db >> 52) + shift;   // biased exponent of the result
  if (exf >= 1 && exf <= 2046)
    return __longlong_as_double((db + (static_cast<long long>(shift) << 52)) |
                                (neg ? static_cast<long long>(0x8000000000000000ull) : 0ll));
  const double d = scale_pow2(__longlong_as_double(db), shift);
  return neg ? -d : d;
}

// One thread = 4 consecutive rows of one column (a 32-bit load per residue plane).  The
// planes hold biased bytes x_g + 128, x_g = psi_G C' mod p_g (|x_g| <= 127), read as the exact
// floats F + x_g (F = 2^23 + 128).  Per group of up to three moduli (a, b, c), in exact FP32
// on biased values (the bias cancels in every difference; every value stays in (0, 2^24)):
//   vb = F + x_a
//   vb += p_a ((x_b - x_a) a1 mod p_b)                 vb = F + (psi_G C' mod p_a p_b)
//   vb += p_a p_b ((x_c - (vb - F)) a2 mod p_c)        vb = F + v, v = psi_G C' mod P_G,
//                                                      |v| < P_G / 2 + 2^15
// then v' = int(vb) + (P_G - F) = v + P_G in (0, 2 P_G) (same class mod P_G),
// X = sum_G v'_G (M / P_G) (mod 2^128), k = round(sum_G v'_G / P_G) = round(X / M) (the FP32
// sum starts from the constant sum_G (P_G - F) / P_G and adds vb_G / P_G: error below 0.05,
// within the 1/4 margin of |C'| <= M/4), C' = X - k M as a two's-complement 128-bit integer,
// rounded to FP64 by integer arithmetic.
__device__ __forceinline__ float mods_f32(float x, float p, float pinv) {   // x - p rint(x / p)
  const float q = fmaf(x, pinv, 12582912.0f) - 12582912.0f;
  return fmaf(-p, q, x);
}

// The element loop for NMOD moduli: every table index is a compile-time constant, so the
// constants are direct operands (no per-use constant loads) and the group loop is straight.
template <int NMOD>
__device__ __forceinline__ void crt_combine_column(const uint8_t* __restrict__ base, int64_t res_plane, int64_t i0,
                                                   int64_t M, const int (&eai)[4], int ebj, int two_t, double alpha,
                                                   double beta, double* __restrict__ ccol, int ab,
                                                   const CrtTable& tab) {
  constexpr int NG = (NMOD + 2) / 3;
  const CrtRecon& rc = tab.rec[NMOD - 1];
  const CrtModuli& md = tab.mod;
  uint32_t words[NMOD];   // all loads in flight before any use
#pragma unroll
  for (int g = 0; g < NMOD; ++g) words[g] = __ldg(reinterpret_cast<const uint32_t*>(base + g * res_plane));
  double out[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {   // one element at a time: only its accumulators are live
    if (i0 + q >= M) continue;
    const uint32_t sel = 0x7540u + q;   // byte q of a word over 0x4B0000..: 2^23 + byte
    uint64_t acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
    float ks = rc.ks0;
#pragma unroll
    for (int G = 0; G < NG; ++G) {
      const int a = 3 * G;
      float vb = __uint_as_float(__byte_perm(words[a], 0x4B000000u, sel));
      if (a + 1 < NMOD) {
        const float xb = __uint_as_float(__byte_perm(words[(a + 1) % NMOD], 0x4B000000u, sel));
        vb = fmaf(rc.pa[G], mods_f32((xb - vb) * rc.a1[G], md.pf[a + 1], md.pinv[a + 1]), vb);
        if (a + 2 < NMOD) {
          const float xc = __uint_as_float(__byte_perm(words[(a + 2) % NMOD], 0x4B000000u, sel));
          vb = fmaf(rc.pab[G], mods_f32((xc - vb) * rc.a2[G], md.pf[a + 2], md.pinv[a + 2]), vb);
        }
      }
      ks = fmaf(vb, rc.Pinv[G], ks);
      const uint32_t vi = static_cast<uint32_t>(static_cast<int32_t>(vb) + rc.voff[G]);
      acc0 += static_cast<uint64_t>(vi) * rc.w[G][0];
      acc1 += static_cast<uint64_t>(vi) * rc.w[G][1];
      acc2 += static_cast<uint64_t>(vi) * rc.w[G][2];
      acc3 += static_cast<uint64_t>(vi) * rc.w[G][3];
    }
    const int64_t k = __float_as_int(ks + 12582912.0f) - 0x4B400000;   // round(X / M)
    const uint64_t accw[4] = {acc0, acc1, acc2, acc3};
    int64_t c = 0;
    uint32_t word[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int64_t v = static_cast<int64_t>(accw[w]) - k * static_cast<int64_t>(rc.m[w]) + c;
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
    if (ab == 1)
      val = alpha * val;
    else if (ab == 2)
      val = fma(alpha, val, beta * ccol[i0 + q]);
    out[q] = val;
  }
  double* dst = ccol + i0;
  if (i0 + 3 < M && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {   // two 16-byte stores
    reinterpret_cast<double2*>(dst)[0] = make_double2(out[0], out[1]);
    reinterpret_cast<double2*>(dst)[1] = make_double2(out[2], out[3]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (i0 + q < M) dst[q] = out[q];
  }
}

__global__ void __launch_bounds__(256) crt_combine_kernel(const uint8_t* __restrict__ res, int64_t res_ld,
                                                          int64_t res_plane, int64_t M, int64_t N,
                                                          const int32_t* __restrict__ ea,
                                                          const int32_t* __restrict__ eb, double alpha, double beta,
                                                          double* __restrict__ C, int64_t ldc, int ab,
                                                          const __grid_constant__ CrtTable tab,
                                                          const CrtDevicePlan* __restrict__ plan) {
  const int64_t i0 = (static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x) * 4;
  if (i0 >= M) return;
  const int nmod = plan->n;
  int eai[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) eai[q] = (i0 + q < M) ? ea[i0 + q] : 0;
  const int two_t = 2 * plan->t;
  for (int64_t j = blockIdx.y; j < N; j += gridDim.y) {
    const uint8_t* base = res + j * res_ld + i0;
    const int ebj = eb[j];
    double* ccol = C + j * ldc;
#define GB_CRT_CASE(n) \
  case n: crt_combine_column<n>(base, res_plane, i0, M, eai, ebj, two_t, alpha, beta, ccol, ab, tab); break;
    switch (nmod) {
      GB_CRT_CASE(1) GB_CRT_CASE(2) GB_CRT_CASE(3) GB_CRT_CASE(4) GB_CRT_CASE(5) GB_CRT_CASE(6) GB_CRT_CASE(7)
      GB_CRT_CASE(8) GB_CRT_CASE(9) GB_CRT_CASE(10) GB_CRT_CASE(11) GB_CRT_CASE(12) GB_CRT_CASE(13)
      GB_CRT_CASE(14) GB_CRT_CASE(15) GB_CRT_CASE(16) GB_CRT_CASE(17) GB_CRT_CASE(18) GB_CRT_CASE(19)
      GB_CRT_CASE(20)
      default: break;
    }
#undef GB_CRT_CASE
  }
}

// ============================================================== driver

int crt_mma_launch(const CrtGemmArgs& a, const CrtPlan& plan, cudaStream_t s) {
  CUtensorMap ta, tb;
  // maps and schedule cover plan.n planes; the kernels run the device plan's n of them
  int rc = make_plane_tmap(&ta, a.planes_a, a.K, a.M, plan.n, a.pitch, 128, a.a_plane_rows ? a.a_plane_rows : a.M);
  if (rc) return rc;
  rc = make_plane_tmap(&tb, a.planes_b, a.K, a.N, plan.n, a.pitch, 128, a.b_plane_rows ? a.b_plane_rows : a.N);
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
  prm.dev_ngroups = &a.plan->n;
  prm.band = a.band;
  for (int g = 0; g < plan.n; ++g) {
    prm.crt_p[g] = crt_table().mod.pf[g];
    prm.crt_inv[g] = crt_table().mod.pinv[g];
  }
  for (int n = 1; n <= plan.n; ++n)
    for (int g = 0; g < n; ++g) prm.crt_psi[n - 1][g] = crt_table().rec[n - 1].psi[g];
  return tc_gemm_pair_launch(TC_EPI_CRT, ta, tb, nullptr, nullptr, plan.sched, prm, a.grid, GB_KERNEL_OZAKI_SLICE_MMA,
                             s);
}

int crt_combine_launch(const CrtGemmArgs& a, cudaStream_t s) {
  const int64_t bx = (a.M + 1023) / 1024;
  const int64_t by = a.N < 65535 ? a.N : 65535;
  if (bx > 0x7FFFFFFF) return GB_ERR_UNSUPPORTED;
  dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(by));
  const int ab = (a.beta != 0.0) ? 2 : (a.alpha != 1.0 ? 1 : 0);   // output rule, decided on the host
  GB_LAUNCH(GB_KERNEL_OZAKI_COMBINE, s,
            (crt_combine_kernel<<<grid, 256, 0, s>>>(a.res, a.res_ld, a.res_plane, a.M, a.N, a.ea, a.eb, a.alpha, a.beta,
                                                     a.C, a.ldc, ab, crt_table(), a.plan)));
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
