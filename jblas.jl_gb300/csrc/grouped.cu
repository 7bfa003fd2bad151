// Grouped GEMM: thousands of independent, uneven C_i = alpha_i A_i B_i + beta_i C_i in one
// persistent launch (FP64 or FP32, CUDA cores, jmul!'s per-element FMA order).
//
// jBLAS multiplies small static matrices one call at a time (fastmul!/kernel!,
// src/kernels.jl:202-208, 239) with a tile size fixed at code-generation time
// (pick_kernel_size, src/kernel_structure.jl:76-99; BLASOptions, src/blas_options.jl:2-7).
// Here one launch walks every tile of every problem:
//   1. a prologue kernel classifies each problem by max(m, n) into a size class, takes
//      that class's tile configuration from the tuning table (chosen by the autotuner,
//      gb_autotune_grouped), counts its tiles and writes the exclusive prefix sum;
//   2. the persistent kernel (grid = SMs x resident CTAs) strides over the global tile
//      index, finds its problem by binary search in the prefix sums and runs that
//      configuration's tile routine.
// Both kernels read only device memory, so a call can be captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "grouped.cuh"
#include "profile.cuh"
#include "simt_gemm.cuh"

namespace gb {

struct TileCfg {
  int bm, bn, bk, tm, tn;
};
// Every configuration runs on 256 threads: (bm / tm) * (bn / tn) == 256.  0-3 serve both
// element types; 4-9 (FP32 only) are the larger and rectangular tiles of the FP32 tile loop.
__host__ __device__ constexpr TileCfg tile_cfg(int c) {
  return c == 0 ? TileCfg{16, 16, 16, 1, 1}
       : c == 1 ? TileCfg{32, 32, 16, 2, 2}
       : c == 2 ? TileCfg{64, 32, 16, 4, 2}
       : c == 3 ? TileCfg{64, 64, 16, 4, 4}
       : c == 4 ? TileCfg{128, 64, 16, 8, 4}
       : c == 5 ? TileCfg{128, 128, 16, 8, 8}
       : c == 6 ? TileCfg{32, 64, 16, 2, 4}
       : c == 7 ? TileCfg{64, 128, 16, 4, 8}
       : c == 8 ? TileCfg{128, 32, 16, 8, 2}
                : TileCfg{32, 128, 16, 2, 8};
}
constexpr int GROUPED_CONFIGS_F64 = 4;
constexpr int GROUPED_CONFIGS_F32 = 10;

__host__ __device__ inline int size_class(int64_t m, int64_t n) {
  const int64_t d = m > n ? m : n;
  return d <= 16 ? 0 : d <= 32 ? 1 : d <= 64 ? 2 : d <= 128 ? 3 : d <= 256 ? 4 : 5;
}

// Per-problem choice (GB_GROUPED_AUTO): the configuration with the least modelled time
//   tiles x (bm bn max(k, 1) / eff(tm tn) + overhead)
// where eff is the measured FMA efficiency of a register tile of tm x tn elements per thread
// relative to the 8 x 8 tile, and overhead the fixed cost of one tile (its first panel's load
// latency, index set-up and epilogue) in the same units.  Padding rows and columns of a tile
// cost as much as real ones, so tall and wide problems take rectangular tiles.
__host__ __device__ inline int auto_config(int64_t m, int64_t n, int64_t k, int nconfigs) {
  float best = 3.4e38f;
  int arg = 0;
  for (int c = 0; c < nconfigs; ++c) {
    const TileCfg t = tile_cfg(c);
    const int e = t.tm * t.tn;
    const float eff = e >= 64 ? 1.0f : e >= 32 ? 0.9f : e >= 16 ? 0.75f : e >= 8 ? 0.55f : e >= 4 ? 0.35f : 0.1f;
    const float tiles = static_cast<float>((m + t.bm - 1) / t.bm) * static_cast<float>((n + t.bn - 1) / t.bn);
    const float cost = tiles * (static_cast<float>(t.bm * t.bn) * static_cast<float>(k > 1 ? k : 1) / eff + 32768.0f);
    if (cost < best) {
      best = cost;
      arg = c;
    }
  }
  return arg;
}

// tuning.config[cls] without a dynamically indexed (local-memory) array
__device__ __forceinline__ int config_of(const gb_grouped_tuning_t& t, int cls) {
  int v = t.config[0];
#pragma unroll
  for (int c = 1; c < GB_GROUPED_CLASSES; ++c) v = (cls == c) ? t.config[c] : v;
  return v;
}

// The configuration one problem runs under (the table's, or the per-problem choice).
template <int NCFG>
__host__ __device__ inline int problem_config(int table_cfg, int64_t m, int64_t n, int64_t k) {
  return table_cfg == GB_GROUPED_AUTO ? auto_config(m, n, k, NCFG) : table_cfg;
}

template <typename T>
__device__ __forceinline__ T fmad(T a, T b, T c);
template <>
__device__ __forceinline__ double fmad<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmad<float>(float a, float b, float c) { return fmaf(a, b, c); }

constexpr int GROUPED_THREADS = 256;
// largest shared memory of any tile routine (bytes): the double-buffered 128 x 128 x 16 FP32
// panels of the SIMT mainloop (the FP64 16 x 64 + 16 x 65 panels take 16.5 KB)
constexpr int GROUPED_SMEM = SimtSmem<float, 128, 128, 16>::ELEMS * 4;
static_assert(GROUPED_SMEM >= (16 * 64 + 16 * 65) * 8, "FP64 tile panels");

// jmul!'s FMA chain with the alpha/beta epilogue of the grouped call (alpha != 0 here).
template <typename T>
struct GroupedChainOp {
  static constexpr bool kInitFromC = false;
  static constexpr bool kPairs = false;
  static constexpr bool kVecStore = true;   // short K loops: the epilogue's stores matter
  T alpha, beta;
  static __device__ __forceinline__ T init() { return T(-0.0); }
  static __device__ __forceinline__ T step(T acc, T a, T b) { return fma_t<T>(a, b, acc); }
  __device__ __forceinline__ void store(T* c, T acc) const {
    *c = (beta == T(0)) ? alpha * acc : fma_t<T>(alpha, acc, beta * *c);
  }
  __device__ __forceinline__ T value(T c, T acc) const {
    return (beta == T(0)) ? alpha * acc : fma_t<T>(alpha, acc, beta * c);
  }
  __device__ __forceinline__ bool reads_c() const { return beta != T(0); }
};

// One BM x BN tile of problem `p` (column-major, no transposes).  Per element the FMA chain
// runs k = 0..K-1 in order from -0.0 (equal to jmul!'s a1*x1 first step, bit for bit).
// The next K slab is loaded into registers while the current one is multiplied from shared
// memory; B's slab is stored [k][n] with rows padded by one word, so the k-fastest global
// reads land in distinct banks.
template <typename T, int BM, int BN, int BK, int TM, int TN>
__device__ __forceinline__ void grouped_tile(const gb_problem_t& p, int tm, int tn, unsigned char* smem) {
  static_assert((BM / TM) * (BN / TN) == GROUPED_THREADS, "configuration must use 256 threads");
  constexpr int LA = (BM * BK + GROUPED_THREADS - 1) / GROUPED_THREADS;   // A elements per thread
  constexpr int LB = (BK * BN + GROUPED_THREADS - 1) / GROUPED_THREADS;   // B elements per thread
  constexpr int BNP = BN + 1;
  T* As = reinterpret_cast<T*>(smem);   // [BK][BM]
  T* Bs = As + BK * BM;                 // [BK][BN + 1]
  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);
  const int64_t M = p.m, N = p.n, K = p.k;
  const int64_t m0 = static_cast<int64_t>(tm) * BM, n0 = static_cast<int64_t>(tn) * BN;
  const T* __restrict__ A = static_cast<const T*>(p.A);
  const T* __restrict__ B = static_cast<const T*>(p.B);
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(-0.0);

  // alpha and beta decoded once per warp (FP64 compares and conversions run on the narrow
  // FP64 pipe) and broadcast
  T alpha, beta;
  bool alpha_zero, unit;   // alpha == 0; alpha == 1 and beta == 0 (C = the chain itself)
  {
    const int lane = threadIdx.x & 31;
    float2 ab = make_float2(0.0f, 0.0f);
    double ad = 0.0, bd = 0.0;
    if (sizeof(T) == 8) {
      ad = p.alpha;
      bd = p.beta;
    } else if (lane == 0) {
      ab = make_float2(static_cast<float>(p.alpha), static_cast<float>(p.beta));
    }
    if (sizeof(T) == 4) {
      ab.x = __shfl_sync(0xffffffffu, ab.x, 0);
      ab.y = __shfl_sync(0xffffffffu, ab.y, 0);
    }
    alpha = (sizeof(T) == 8) ? static_cast<T>(ad) : static_cast<T>(ab.x);
    beta = (sizeof(T) == 8) ? static_cast<T>(bd) : static_cast<T>(ab.y);
    alpha_zero = ((__double_as_longlong(p.alpha) & 0x7FFFFFFFFFFFFFFFll) == 0);
    unit = __double_as_longlong(p.alpha) == 0x3FF0000000000000ll && __double_as_longlong(p.beta) == 0ll;
  }
  const int64_t Kc = alpha_zero ? 0 : K;   // alpha == 0: A and B are not read
  T ra[LA], rb[LB];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int l = 0; l < LA; ++l) {
      const int e = tid + l * GROUPED_THREADS;
      const int ml = e % BM, kl = e / BM;
      const int64_t m = m0 + ml, k = k0 + kl;
      ra[l] = (e < BM * BK && m < M && k < K) ? A[m + k * p.lda] : T(0);
    }
#pragma unroll
    for (int l = 0; l < LB; ++l) {
      const int e = tid + l * GROUPED_THREADS;
      const int kl = e % BK, nl = e / BK;
      const int64_t n = n0 + nl, k = k0 + kl;
      rb[l] = (e < BK * BN && n < N && k < K) ? B[k + n * p.ldb] : T(0);
    }
  };
  if (Kc > 0) load(0);
  for (int64_t k0 = 0; k0 < Kc; k0 += BK) {
    const int kc = static_cast<int>(K - k0 < BK ? K - k0 : BK);
#pragma unroll
    for (int l = 0; l < LA; ++l) {
      const int e = tid + l * GROUPED_THREADS;
      if (e < BM * BK) As[(e / BM) * BM + e % BM] = ra[l];
    }
#pragma unroll
    for (int l = 0; l < LB; ++l) {
      const int e = tid + l * GROUPED_THREADS;
      if (e < BK * BN) Bs[(e % BK) * BNP + e / BK] = rb[l];
    }
    __syncthreads();
    if (k0 + BK < Kc) load(k0 + BK);   // in flight while this slab is multiplied
    for (int kk = 0; kk < kc; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk * BM + ty + i * (BM / TM)];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk * BNP + tx + j * (BN / TN)];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmad<T>(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  T* __restrict__ C = static_cast<T*>(p.C);
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + ty + i * (BM / TM);
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t n = n0 + tx + j * (BN / TN);
      if (n >= N) continue;
      T* c = &C[m + n * p.ldc];
      if (alpha == T(0)) *c = (beta == T(0)) ? T(0) : beta * *c;   // A, B not read
      else if (unit) *c = acc[i][j];   // jmul!'s result, without a multiply on the FP64 pipe
      else *c = (beta == T(0)) ? alpha * acc[i][j] : fmad<T>(alpha, acc[i][j], beta * *c);
    }
  }
}

// alpha = 0: C = beta C on one bm x bn tile (beta = 0 writes zeros without reading C; A and B
// are not read), as jBLAS's alpha/beta extension of gb_gemm_* defines it.
template <typename T>
__device__ __forceinline__ void scale_tile(const gb_problem_t& p, int64_t m0, int64_t n0, int bm, int bn) {
  T* __restrict__ C = static_cast<T*>(p.C);
  const T beta = static_cast<T>(p.beta);
  for (int e = threadIdx.x; e < bm * bn; e += GROUPED_THREADS) {
    const int64_t m = m0 + e % bm, n = n0 + e / bm;
    if (m < p.m && n < p.n) {
      T* c = &C[m + n * p.ldc];
      *c = (beta == T(0)) ? T(0) : beta * *c;
    }
  }
}

__device__ __forceinline__ int prologue_config(const gb_grouped_tuning_t& tuning, const gb_problem_t& p, bool f32) {
  const int c = config_of(tuning, size_class(p.m, p.n));
  return f32 ? problem_config<GROUPED_CONFIGS_F32>(c, p.m, p.n, p.k) : problem_config<GROUPED_CONFIGS_F64>(c, p.m, p.n, p.k);
}

// Workspace of a call over `count` problems (int64 words): the tile prefix sums in schedule
// order offsets[0..count], then the schedule order (count int32 entries: the problem index,
// and for count <= 2^24 its tile configuration in bits 24-30, so the tile loop need not
// evaluate the per-problem choice again for every tile).
__host__ __device__ inline long long* grouped_order_words(long long* ws, int count) { return ws + count + 1; }
constexpr int GROUPED_PACK_LIMIT = 1 << 24;
__host__ __device__ inline int grouped_order_entry(int i, int cfg, int count) {
  return count <= GROUPED_PACK_LIMIT ? (i | (cfg << 24)) : i;
}

// Prologue (one block): the schedule orders the problems by the work of one of their tiles
// (tile rows x tile columns x k, in 32 power-of-two buckets, heaviest first), so that the CTAs,
// striding over the schedule, take tiles of similar length side by side and the short ones
// fill the tail; it writes the order and the exclusive prefix sums of the tiles in that order.
// The order inside a bucket depends on timing, which changes no result (each tile is
// independent).
__global__ void __launch_bounds__(1024, 1) grouped_prefix_kernel(const gb_problem_t* __restrict__ probs, int count,
                                                              gb_grouped_tuning_t tuning, bool f32,
                                                              long long* __restrict__ ws) {
  __shared__ long long part[1024];
  __shared__ int hist[32], start[32];
  long long* offsets = ws;
  int* order = reinterpret_cast<int*>(grouped_order_words(ws, count));
  const int t = threadIdx.x;
  if (t < 32) hist[t] = 0;
  __syncthreads();
  auto bucket_of = [&](const gb_problem_t& p, const TileCfg& c) {
    const long long w = static_cast<long long>(c.bm) * c.bn * (p.k > 1 ? p.k : 1);
    const int lg = 63 - __clzll(w);                 // w >= 1
    return 31 - (lg > 31 ? 31 : lg);                 // heavy first
  };
  for (int i = t; i < count; i += 1024) {
    const gb_problem_t& p = probs[i];
    atomicAdd(&hist[bucket_of(p, tile_cfg(prologue_config(tuning, p, f32)))], 1);
  }
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int b = 0; b < 32; ++b) {
      start[b] = run;
      run += hist[b];
    }
  }
  __syncthreads();
  for (int i = t; i < count; i += 1024) {
    const gb_problem_t& p = probs[i];
    const int cfg = prologue_config(tuning, p, f32);
    order[atomicAdd(&start[bucket_of(p, tile_cfg(cfg))], 1)] = grouped_order_entry(i, cfg, count);
  }
  __syncthreads();
  const int per = (count + 1023) / 1024;
  const int b = t * per, e = min(count, b + per);
  const bool packed = count <= GROUPED_PACK_LIMIT;
  auto tiles_of = [&](int pos) -> long long {
    const int e = order[pos];
    const gb_problem_t& p = probs[packed ? (e & 0xFFFFFF) : e];
    const TileCfg c = tile_cfg(packed ? (e >> 24) : prologue_config(tuning, p, f32));
    return (p.m <= 0 || p.n <= 0) ? 0 : ((p.m + c.bm - 1) / c.bm) * ((p.n + c.bn - 1) / c.bn);
  };
  long long sum = 0;
  for (int i = b; i < e; ++i) sum += tiles_of(i);
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {   // inclusive Hillis-Steele scan of the parts
    const long long v = (t >= off) ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = (t == 0) ? 0 : part[t - 1];
  for (int i = b; i < e; ++i) {
    offsets[i] = run;
    run += tiles_of(i);
  }
  if (t == 1023) offsets[count] = part[1023];
}

// The schedule position of tile w: the last pos with offsets[pos] <= w (problems without
// tiles share their successor's offset), searched from `from` (a position with
// offsets[from] <= w: a CTA's tiles come in increasing order, so its previous tile's position).
// Each warp searches on its own: its 32 lanes probe 32 points of the remaining interval at
// once, so 4096 problems take at most 3 rounds of loads instead of the 12 dependent loads of a
// binary search.  Every warp reaches the same position.
__device__ __forceinline__ int schedule_pos(const long long* __restrict__ offsets, int count, long long w, int from) {
  const int lane = threadIdx.x & 31;
  int lo = from, hi = count - 1;   // offsets[lo] <= w holds throughout
  while (lo < hi) {
    const long long span = hi - lo;
    const int p = lo + static_cast<int>((span * (lane + 1) + 31) / 32);   // in (lo, hi]; lane 31: hi
    const unsigned ok = __ballot_sync(0xffffffffu, offsets[p] <= w);   // monotone in the lane
    if (ok == 0u) {
      hi = __shfl_sync(0xffffffffu, p, 0) - 1;
    } else {
      const int L = 31 - __clz(ok);
      const int pl = __shfl_sync(0xffffffffu, p, L);
      const int pn = __shfl_sync(0xffffffffu, p, L < 31 ? L + 1 : 31);
      hi = (L == 31) ? hi : pn - 1;
      lo = pl;
    }
  }
  return lo;
}

// Persistent tile loop: CTA b takes tiles b, b + grid, ... of the schedule.
template <typename T>
__global__ void __launch_bounds__(GROUPED_THREADS, 2) grouped_gemm_kernel(const gb_problem_t* __restrict__ probs,
                                                                       int count, gb_grouped_tuning_t tuning,
                                                                       long long* __restrict__ ws) {
  __shared__ __align__(16) unsigned char smem[GROUPED_SMEM];
  const long long* offsets = ws;
  const int* order = reinterpret_cast<const int*>(grouped_order_words(ws, count));
  const long long total = offsets[count];
  int lo = 0;   // offsets[0] = 0 <= w
  for (long long w = blockIdx.x; w < total; w += gridDim.x) {
    lo = schedule_pos(offsets, count, w, lo);
    const int e = order[lo];
    const bool packed = count <= GROUPED_PACK_LIMIT;
    const gb_problem_t p = probs[packed ? (e & 0xFFFFFF) : e];
    const int cfg = packed ? (e >> 24) : prologue_config(tuning, p, sizeof(T) == 4);
    const TileCfg c = tile_cfg(cfg);
    // tile rows of the problem and the tile's place in it, in 32-bit arithmetic (a problem's
    // tile count is below 2^31)
    const int local = static_cast<int>(w - offsets[lo]);
    const int tiles_m = static_cast<int>((p.m + c.bm - 1) / c.bm);
    const int tn = local / tiles_m, tm = local - tn * tiles_m;
    if constexpr (sizeof(T) == 8) {
      // FP64 runs at the DFMA rate whatever the tile: the small configurations keep the
      // register count (and so the resident CTAs per SM) low.
      switch (cfg) {
        case 0: grouped_tile<T, 16, 16, 16, 1, 1>(p, tm, tn, smem); break;
        case 1: grouped_tile<T, 32, 32, 16, 2, 2>(p, tm, tn, smem); break;
        case 2: grouped_tile<T, 64, 32, 16, 4, 2>(p, tm, tn, smem); break;
        default: grouped_tile<T, 64, 64, 16, 4, 4>(p, tm, tn, smem); break;
      }
    } else if (cfg == 0) {
      grouped_tile<T, 16, 16, 16, 1, 1>(p, tm, tn, smem);   // one element a thread
    } else if ((__double_as_longlong(p.alpha) & 0x7FFFFFFFFFFFFFFFll) == 0) {
      scale_tile<T>(p, static_cast<int64_t>(tm) * c.bm, static_cast<int64_t>(tn) * c.bn, c.bm, c.bn);
    } else {
      // FP32 register tiles of two or more rows and columns: the double-buffered SIMT mainloop
      // of the native GEMM (simt_gemm.cuh) on this problem's tile
      const GroupedChainOp<T> op{static_cast<T>(p.alpha), static_cast<T>(p.beta)};
      const T* A = static_cast<const T*>(p.A);
      const T* B = static_cast<const T*>(p.B);
      T* C = static_cast<T*>(p.C);
      T* sm = reinterpret_cast<T*>(smem);
      const int64_t m0 = static_cast<int64_t>(tm) * c.bm, n0 = static_cast<int64_t>(tn) * c.bn;
#define GB_GTILE(BM_, BN_, BK_, TM_, TN_)                                                                    \
  simt_tile<T, GroupedChainOp<T>, BM_, BN_, BK_, TM_, TN_, false, false>(p.m, p.n, p.k, op, A, p.lda, B, p.ldb, C, \
                                                                        p.ldc, m0, n0, sm)
      switch (cfg) {
        case 1: GB_GTILE(32, 32, 16, 2, 2); break;
        case 2: GB_GTILE(64, 32, 16, 4, 2); break;
        case 3: GB_GTILE(64, 64, 16, 4, 4); break;
        case 4: GB_GTILE(128, 64, 16, 8, 4); break;
        case 5: GB_GTILE(128, 128, 16, 8, 8); break;
        case 6: GB_GTILE(32, 64, 16, 2, 4); break;
        case 7: GB_GTILE(64, 128, 16, 4, 8); break;
        case 8: GB_GTILE(128, 32, 16, 8, 2); break;
        default: GB_GTILE(32, 128, 16, 2, 8); break;
      }
#undef GB_GTILE
      __syncthreads();   // the next tile reuses the shared panels
    }
  }
}

gb_grouped_tuning_t grouped_default_tuning(int dtype_bytes) {
  gb_grouped_tuning_t t;
  std::memset(&t, 0, sizeof(t));
  // classes: <=16, <=32, <=64, <=128, <=256, >256
  // FP32: the per-problem choice in every class (rectangular tiles for tall and wide problems).
  // FP64: 16 x 16 tiles everywhere: the DFMA pipe, not the register tile, bounds FP64, and the
  // smallest tiles pad least (the autotuner picks them in every class; 1.0 TFLOP/s against 0.71
  // for larger tiles in the larger classes, 4096 log-uniform problems).
  for (int c = 0; c < GB_GROUPED_CLASSES; ++c) t.config[c] = dtype_bytes == 8 ? 0 : GB_GROUPED_AUTO;
  return t;
}

int grouped_configs(int dtype_bytes) { return dtype_bytes == 8 ? GROUPED_CONFIGS_F64 : GROUPED_CONFIGS_F32; }

int grouped_validate_tuning(int dtype_bytes, const gb_grouped_tuning_t& t) {
  for (int c = 0; c < GB_GROUPED_CLASSES; ++c)
    if (t.config[c] != GB_GROUPED_AUTO && (t.config[c] < 0 || t.config[c] >= grouped_configs(dtype_bytes)))
      return GB_ERR_INVALID_VALUE;
  return GB_OK;
}

// Resident CTAs per SM of grouped_gemm_kernel<T>, looked up once per device (the occupancy
// query runs against the current device's context); concurrent first calls may both query,
// and both store the same value.
constexpr int GROUPED_MAX_DEVICES = 64;

template <typename T>
static int grid_for(int sms) {
  static std::atomic<int> per_sm_of[GROUPED_MAX_DEVICES];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GROUPED_MAX_DEVICES) {
    cudaGetLastError();
    dev = -1;
  }
  int per_sm = dev >= 0 ? per_sm_of[dev].load(std::memory_order_relaxed) : 0;
  if (per_sm < 1) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_gemm_kernel<T>, GROUPED_THREADS, 0) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    } else if (dev >= 0) {
      per_sm_of[dev].store(per_sm, std::memory_order_relaxed);
    }
  }
  return sms * per_sm;
}

int grouped_launch(int dtype_bytes, const gb_problem_t* d_probs, int count, const gb_grouped_tuning_t& tuning,
                   long long* d_offsets, int sms, cudaStream_t s) {
  if (count <= 0) return GB_OK;
  GB_LAUNCH(GB_KERNEL_GROUPED_GEMM, s,
            (grouped_prefix_kernel<<<1, 1024, 0, s>>>(d_probs, count, tuning, dtype_bytes == 4, d_offsets)));
  if (dtype_bytes == 8) {
    const int grid = grid_for<double>(sms);
    GB_LAUNCH(GB_KERNEL_GROUPED_GEMM, s,
              (grouped_gemm_kernel<double><<<grid, GROUPED_THREADS, 0, s>>>(d_probs, count, tuning, d_offsets)));
  } else {
    const int grid = grid_for<float>(sms);
    GB_LAUNCH(GB_KERNEL_GROUPED_GEMM, s,
              (grouped_gemm_kernel<float><<<grid, GROUPED_THREADS, 0, s>>>(d_probs, count, tuning, d_offsets)));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

size_t grouped_workspace_bytes(int count) {
  // prefix sums (count + 1), the order (count int32 in (count + 1) / 2 words)
  return (static_cast<size_t>(count) + 1 + (static_cast<size_t>(count) + 1) / 2) * sizeof(long long);
}

// Autotuner: for every size class present, time each configuration on that class's
// problems alone (C redirected to scratch, beta = 0, so the caller's C is untouched) and
// keep the fastest.  Replaces BLASOptions' fixed block sizes (src/blas_options.jl:2-7).
int grouped_autotune(int dtype_bytes, const gb_problem_t* h_probs, int count, int sms, cudaMemPool_t pool,
                     int reps, gb_grouped_tuning_t* out, float* class_ms, cudaStream_t s) {
  gb_grouped_tuning_t best = grouped_default_tuning(dtype_bytes);
  std::vector<std::vector<gb_problem_t>> by_class(GB_GROUPED_CLASSES);
  size_t max_c = 1;
  for (int i = 0; i < count; ++i) {
    const gb_problem_t& p = h_probs[i];
    if (p.m <= 0 || p.n <= 0) continue;
    by_class[size_class(p.m, p.n)].push_back(p);
    max_c = std::max(max_c, static_cast<size_t>(p.m * p.n));
  }
  void* scratch = nullptr;
  gb_problem_t* d_sub = nullptr;
  long long* d_off = nullptr;
  GB_CUDA_TRY(cudaMallocFromPoolAsync(&scratch, max_c * dtype_bytes, pool, s));
  GB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&d_sub), sizeof(gb_problem_t) * (count + 1), pool, s));
  GB_CUDA_TRY(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&d_off), grouped_workspace_bytes(count), pool, s));
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  int rc = GB_OK;
  for (int c = 0; c < GB_GROUPED_CLASSES && rc == GB_OK; ++c) {
    if (class_ms) class_ms[c] = 0.f;
    auto& v = by_class[c];
    if (v.empty()) continue;
    for (auto& p : v) {
      p.C = scratch;
      p.ldc = p.m;
      p.beta = 0.0;
    }
    if (cudaMemcpyAsync(d_sub, v.data(), v.size() * sizeof(gb_problem_t), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      rc = GB_ERR_CUDA;
      break;
    }
    float best_ms = 1e30f;
    for (int ci = 0; ci <= grouped_configs(dtype_bytes); ++ci) {
      const int cfg = (ci == grouped_configs(dtype_bytes)) ? GB_GROUPED_AUTO : ci;
      gb_grouped_tuning_t t = best;
      t.config[c] = cfg;
      rc = grouped_launch(dtype_bytes, d_sub, static_cast<int>(v.size()), t, d_off, sms, s);   // warm-up
      if (rc) break;
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps; ++r) grouped_launch(dtype_bytes, d_sub, static_cast<int>(v.size()), t, d_off, sms, s);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = GB_ERR_CUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (ms < best_ms) {
        best_ms = ms;
        best.config[c] = cfg;
      }
    }
    if (class_ms) class_ms[c] = best_ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(scratch, s);
  cudaFreeAsync(d_sub, s);
  cudaFreeAsync(d_off, s);
  if (rc == GB_OK) *out = best;
  return rc;
}

}  // namespace gb

// ============================================================ allocation-free variant
//
// For callers that cannot allocate device memory at call time (see gbblas.h): the tile
// prefix sums live in a fixed file-scope device array instead of pool or caller memory.
// Every GPU that loads the library holds this array until the process exits.
namespace gb {

constexpr int GROUPED_NOALLOC_MAX = GB_GROUPED_NOALLOC_MAX;
constexpr int NOALLOC_MAX_DEVICES = 64;

// int64 words of grouped_workspace_bytes(GROUPED_NOALLOC_MAX): 98,305 (768 KiB)
constexpr int GROUPED_NOALLOC_WORDS = GROUPED_NOALLOC_MAX + 1 + (GROUPED_NOALLOC_MAX + 1) / 2;
static __device__ __align__(256) long long g_noalloc_offsets[GROUPED_NOALLOC_WORDS];

// Device address of g_noalloc_offsets per device.  In host code the symbol names a host
// stand-in, so the address is looked up once per device (with that device current) and
// reused; the lookup neither allocates nor launches.
static std::mutex g_noalloc_mu;
static long long* g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static int g_noalloc_sms[NOALLOC_MAX_DEVICES];

static int noalloc_setup(long long** ptr, int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gb_set_cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GB_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    int major = 0, minor = 0, n = 0;
    e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return gb_set_cuda_error(e, "device attributes");
    if (major != 10 || minor != 3) return GB_ERR_NO_DEVICE;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_offsets);
    if (e != cudaSuccess) return gb_set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_offsets)");
    g_noalloc_sms[dev] = n;
    g_noalloc_ptr[dev] = static_cast<long long*>(p);
  }
  *ptr = g_noalloc_ptr[dev];
  *sms = g_noalloc_sms[dev];
  return GB_OK;
}

int grouped_f64_noalloc(const gb_problem_t* d_probs, int count, const gb_grouped_tuning_t* tuning, cudaStream_t s) {
  if (count < 0 || count > GROUPED_NOALLOC_MAX) return GB_ERR_INVALID_VALUE;
  long long* offsets = nullptr;
  int sms = 0;
  int rc = noalloc_setup(&offsets, &sms);
  if (rc) return rc;
  if (count == 0) return GB_OK;
  const gb_grouped_tuning_t t = tuning ? *tuning : grouped_default_tuning(8);
  rc = grouped_validate_tuning(8, t);
  if (rc) return rc;
  // The prologue rewrites the prefix sums and the order on every call, so nothing needs
  // clearing.
  // Launched directly, not through the timing hooks (which create CUDA events while profiling
  // is on); gb_launch_counts still counts both launches.
  grouped_prefix_kernel<<<1, 1024, 0, s>>>(d_probs, count, t, false, offsets);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gb_set_cuda_error(e, "grouped prologue launch");
  prof_count(GB_KERNEL_GROUPED_GEMM);
  grouped_gemm_kernel<double><<<grid_for<double>(sms), GROUPED_THREADS, 0, s>>>(d_probs, count, t, offsets);
  e = cudaGetLastError();
  if (e != cudaSuccess) return gb_set_cuda_error(e, "grouped launch");
  prof_count(GB_KERNEL_GROUPED_GEMM);
  return GB_OK;
}


// ------------------------------------------------------------------ strided batches
__global__ void grouped_fill_strided_kernel(gb_problem_t* __restrict__ probs, int count, int64_t M, int64_t N,
                                            int64_t K, int64_t lda, int64_t ldb, int64_t ldc, const char* A,
                                            const char* B, char* C, int64_t sa, int64_t sb, int64_t sc, double alpha,
                                            double beta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  gb_problem_t p;
  p.m = M;
  p.n = N;
  p.k = K;
  p.lda = lda;
  p.ldb = ldb;
  p.ldc = ldc;
  p.A = A + static_cast<int64_t>(i) * sa;
  p.B = B + static_cast<int64_t>(i) * sb;
  p.C = C + static_cast<int64_t>(i) * sc;
  p.alpha = alpha;
  p.beta = beta;
  probs[i] = p;
}

int grouped_fill_strided(gb_problem_t* d_probs, int count, int64_t M, int64_t N, int64_t K, int64_t lda, int64_t ldb,
                         int64_t ldc, const void* A, const void* B, void* C, int64_t strideA_bytes,
                         int64_t strideB_bytes, int64_t strideC_bytes, double alpha, double beta, cudaStream_t s) {
  if (count <= 0) return GB_OK;
  const int blocks = (count + 255) / 256;
  grouped_fill_strided_kernel<<<blocks, 256, 0, s>>>(d_probs, count, M, N, K, lda, ldb, ldc,
                                                      static_cast<const char*>(A), static_cast<const char*>(B),
                                                      static_cast<char*>(C), strideA_bytes, strideB_bytes,
                                                      strideC_bytes, alpha, beta);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
}  // namespace gb
