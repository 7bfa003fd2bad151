// Slice-product GEMM engine: persistent, warp-specialised tcgen05 kernel (see tc_gemm.cuh).
//
//   warp 0      TMA producer: A/B plane tiles into a 4-stage shared-memory ring (the role
//               of jBLAS's prefetch schedule, src/memory_management.jl:181-277)
//   warp 1      allocates 512 TMEM columns; lane 0 issues tcgen05.mma 128x256x16 into a
//               double-buffered FP32 accumulator (jBLAS's register tile, src/gemm.jl:318-333)
//   warps 2-9   epilogue: tcgen05.ld of each finished group sum, then the fused store; two
//               warps per TMEM lane quadrant, each draining half of the 256 columns
//               (jBLAS's store_block, src/gemm.jl:3-11, with recombination / alpha / beta)
// Every mbarrier wait is bounded; on expiry the CTA records GB_ERR_PIPELINE_TIMEOUT, waits
// (bounded) for its in-flight copies and MMAs, frees TMEM and exits.
#include <cuda_bf16.h>

#include <atomic>

#include "gb_common.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace gb {

constexpr int TC_THREADS = 320;                 // 10 warps
constexpr int TC_EPI_THREADS = 256;             // warps 2..9
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;   // 16 KB
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;   // 32 KB
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr int TC_TMEM_COLS = 512;               // two 128 x 256 FP32 accumulators
constexpr int TC_SMEM_BYTES = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int EXP_NONFINITE = 0x7FFFFFFF;
// Cleanup waits after an abort (copies and MMAs already in flight) use their own limit,
// independent of the caller's, so that TMEM and shared memory are never released early.
constexpr uint64_t TC_CLEANUP_WAIT_NS = 2000000000ull;

// Tile raster: bands of GM row tiles (16 by default), column tiles inside a band (keeps the concurrently
// active A and B panels of one plane pair inside L2).
__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int GM, int& tm, int& tn) {
  const int band = t / (GM * tiles_n);
  const int in_band = t - band * GM * tiles_n;
  const int band_rows = min(GM, tiles_m - band * GM);
  tm = band * GM + in_band % band_rows;
  tn = in_band / band_rows;
}

// S * 2^wexp as a double, for an FP32 value S holding an integer (|S| <= 2^24) and
// wbias = (896 + wexp) << 23: the FP32 exponent is rebased to FP64 (bias 127 -> 1023) and
// shifted by wexp in integer arithmetic, so no FP32->FP64 conversion runs on the FP64 pipe.
// Exact for every such S; +-0 keeps its sign.
__device__ __forceinline__ double exact_int_f32_times_pow2(uint32_t u, unsigned long long wbias) {
  const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
  const uint32_t mag = u & 0x7FFFFFFFu;
  const unsigned long long body = mag ? ((static_cast<unsigned long long>(mag) + wbias) << 29) : 0ull;
  return __longlong_as_double(static_cast<long long>(sign | body));
}

__device__ __forceinline__ int problem_of(const TcParams& prm, int t) {
  return (prm.nprob == 2 && t >= prm.prob[1].tile_begin) ? 1 : 0;
}

template <int EPI>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmap_a0, const __grid_constant__ CUtensorMap tmap_b0,
                   const __grid_constant__ CUtensorMap tmap_a1, const __grid_constant__ CUtensorMap tmap_b1,
                   const __grid_constant__ SliceSchedule sched, const __grid_constant__ TcParams prm) {
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte alignment for the 128-byte swizzle atoms
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* empty = full + TC_STAGES;
  uint64_t* tfull = empty + TC_STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = prm.total_tiles;
  const int G = sched.ngroups;

  if (threadIdx.x == 0) {
    for (int i = 0; i < TC_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], TC_EPI_THREADS);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
    tma_prefetch_desc(&tmap_a0);
    tma_prefetch_desc(&tmap_b0);
    if (prm.nprob == 2) {
      tma_prefetch_desc(&tmap_a1);
      tma_prefetch_desc(&tmap_b1);
    }
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, TC_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued_parity[TC_STAGES];
      for (int i = 0; i < TC_STAGES; ++i) issued_parity[i] = -1;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int pr = problem_of(prm, t);
        const TcProblem& P = prm.prob[pr];
        const CUtensorMap* ta = pr ? &tmap_a1 : &tmap_a0;
        const CUtensorMap* tb = pr ? &tmap_b1 : &tmap_b0;
        int tm, tn;
        tile_coords(t - P.tile_begin, P.tiles_m, P.tiles_n, prm.band, tm, tn);
        const int m0 = tm * TC_BM, n0 = tn * TC_BN;
        for (int g = 0; g < G && ok; ++g) {
          for (int c = 0; c < P.nchunks && ok; ++c) {
            const int kb0 = c * sched.kb_chunk;
            const int kb1 = min(kb0 + sched.kb_chunk, P.kb_total);
            for (int i = 0; i < sched.npairs[g] && ok; ++i) {
              const int pa = sched.pp[sched.pair_off[g] + i];
              const int pb = sched.pq[sched.pair_off[g] + i];
              for (int kb = kb0; kb < kb1; ++kb) {
                if (!mbar_wait_bounded(&empty[stage], phase ^ 1, prm.wait_limit_ns, abort_flag,
                                       prm.status, 1)) {
                  ok = false;
                  break;
                }
                uint8_t* sa = smem + stage * TC_STAGE_BYTES;
                uint8_t* sb = sa + TC_A_BYTES;
                mbar_arrive_expect_tx(&full[stage], TC_STAGE_BYTES);
                tma_load_3d(sa, ta, &full[stage], kb * TC_BK, m0, pa);
                tma_load_3d(sb, tb, &full[stage], kb * TC_BK, n0, pb);
                issued_parity[stage] = static_cast<int>(phase);
                if (++stage == TC_STAGES) { stage = 0; phase ^= 1; }
              }
            }
          }
        }
      }
      if (!ok) {
        // let every copy this thread issued land before the CTA's shared memory goes away
        for (int i = 0; i < TC_STAGES; ++i)
          if (issued_parity[i] >= 0) {
            volatile int no_abort = 0;
            mbar_wait_bounded(&full[i], static_cast<uint32_t>(issued_parity[i]), TC_CLEANUP_WAIT_NS,
                              &no_abort, nullptr, 0);
          }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16_f32(TC_BM, TC_BN);
      int stage = 0;
      uint32_t phase = 0;
      int buf = 0;
      uint32_t acc_phase = 0;
      bool ok = true;
      bool issued_any = false;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcProblem& P = prm.prob[problem_of(prm, t)];
        for (int g = 0; g < G && ok; ++g) {
          for (int c = 0; c < P.nchunks && ok; ++c) {
            const int kb0 = c * sched.kb_chunk;
            const int kb1 = min(kb0 + sched.kb_chunk, P.kb_total);
            if (!mbar_wait_bounded(&tempty[buf], acc_phase ^ 1, prm.wait_limit_ns, abort_flag,
                                   prm.status, 2)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t d_tmem = tmem_base + static_cast<uint32_t>(buf * TC_BN);
            uint32_t accumulate = 0;
            for (int i = 0; i < sched.npairs[g] && ok; ++i) {
              for (int kb = kb0; kb < kb1; ++kb) {
                if (!mbar_wait_bounded(&full[stage], phase, prm.wait_limit_ns, abort_flag,
                                       prm.status, 3)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + stage * TC_STAGE_BYTES);
                const uint32_t sb = sa + TC_A_BYTES;
                const uint64_t adesc = smem_desc_sw128(sa);
                const uint64_t bdesc = smem_desc_sw128(sb);
#pragma unroll
                for (int kk = 0; kk < TC_BK / 16; ++kk) {
                  // advance 16 BF16 = 32 bytes along K inside the swizzle atom
                  tc_mma_f16(d_tmem, adesc + static_cast<uint64_t>(kk * 2),
                             bdesc + static_cast<uint64_t>(kk * 2), IDESC, accumulate);
                  accumulate = 1;
                }
                issued_any = true;
                tc_commit(&empty[stage]);
                if (++stage == TC_STAGES) { stage = 0; phase ^= 1; }
              }
            }
            if (!ok) break;
            tc_commit(&tfull[buf]);
            if (++buf == 2) { buf = 0; acc_phase ^= 1; }
          }
        }
      }
      if (!ok && issued_any) {
        // wait for every MMA issued so far before TMEM is released
        tc_commit(drain);
        volatile int no_abort = 0;
        mbar_wait_bounded(drain, 0, TC_CLEANUP_WAIT_NS, &no_abort, nullptr, 0);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2..5)
    const int q = warp & 3;                 // TMEM lane quadrant of this warp
    const int row_l = q * 32 + lane;        // tile row owned by this thread
    const int col0 = ((warp - 2) >> 2) * (TC_BN / 2);   // this warp's half of the columns
    // the per-CTA FP64 tile buffer is re-read at every drain while digit planes stream
    // through L2: keep it resident
    const uint64_t keep = l2_policy_evict_last();
    int buf = 0;
    uint32_t acc_phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int pr = problem_of(prm, t);
      const TcProblem& P = prm.prob[pr];
      int tm, tn;
      tile_coords(t - P.tile_begin, P.tiles_m, P.tiles_n, prm.band, tm, tn);
      const int64_t row = static_cast<int64_t>(tm) * TC_BM + row_l;
      const int64_t n0 = static_cast<int64_t>(tn) * TC_BN;
      const bool row_ok = row < P.M;
      const double alpha = P.alpha, beta = P.beta;
      int ea = 0;
      if (EPI == TC_EPI_OZAKI_F64) ea = row_ok ? P.ea[row] : 0;
      double* __restrict__ tws = prm.tws + static_cast<int64_t>(blockIdx.x) * (TC_BM * TC_BN);
      int step = 0;
      const int nsteps = G * P.nchunks;
      for (int g = 0; g < G && ok; ++g) {
        // group weight 2^wexp folded into the exponent of each exact integer group sum
        const int wexp = 2 - sched.level[g] * sched.bits;
        const unsigned long long wbias = static_cast<unsigned long long>(896 + wexp) << 23;
        for (int c = 0; c < P.nchunks; ++c, ++step) {
          // the whole warp agrees before the warp-collective tcgen05.ld
          ok = __all_sync(0xffffffffu, mbar_wait_bounded(&tfull[buf], acc_phase, prm.wait_limit_ns,
                                                         abort_flag, prm.status, 4));
          if (!ok) break;
          tc_fence_after();
          const bool first = (step == 0), last = (step == nsteps - 1);
          const uint32_t taddr = tmem_base + (static_cast<uint32_t>(q * 32) << 16) +
                                 static_cast<uint32_t>(buf * TC_BN);
#pragma unroll 1
          for (int cb = col0; cb < col0 + TC_BN / 2; cb += 32) {
            uint32_t v[32];
            tmem_ld_32x32b_x32(taddr + cb, v);
            tc_wait_ld();
            const int64_t colb = n0 + cb;
            if (EPI == TC_EPI_F32) {
              if (row_ok) {
                float* __restrict__ crow = static_cast<float*>(P.C) + row + colb * P.ldc;
                const float fa = static_cast<float>(alpha), fb = static_cast<float>(beta);
                float c0[32];
                if (fb != 0.0f) {
#pragma unroll
                  for (int j = 0; j < 32; ++j) c0[j] = (colb + j < P.N) ? crow[j * P.ldc] : 0.0f;
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                  if (colb + j >= P.N) continue;
                  const float sj = __uint_as_float(v[j]);
                  crow[j * P.ldc] = (fb == 0.0f) ? fa * sj : fmaf(fa, sj, fb * c0[j]);
                }
              }
              continue;
            }
            double* __restrict__ tcol = tws + static_cast<int64_t>(cb) * TC_BM + row_l;
            // all loads of the chunk are issued before any store (no aliasing chain)
            double tv[32];
            if (!first) {
#pragma unroll
              for (int j = 0; j < 32; ++j) tv[j] = ld_f64_hint(tcol + j * TC_BM, keep);
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const double sw = exact_int_f32_times_pow2(v[j], wbias);
              tv[j] = first ? sw : tv[j] + sw;   // == fma(S, 2^wexp, T): S * 2^wexp is exact
            }
            if (!last) {
#pragma unroll
              for (int j = 0; j < 32; ++j) st_f64_hint(tcol + j * TC_BM, tv[j], keep);
            } else if (row_ok) {
              double* __restrict__ crow = static_cast<double*>(P.C) + row + colb * P.ldc;
#pragma unroll
              for (int j8 = 0; j8 < 32; j8 += 8) {
                // 8 columns at a time: exponents and C loads issued together, then stored
                int ebj[8];
                double c0[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                  const bool in = colb + j8 + j < P.N;
                  ebj[j] = in ? __ldg(P.eb + colb + j8 + j) : 0;
                  c0[j] = (in && beta != 0.0) ? crow[(j8 + j) * P.ldc] : 0.0;
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                  if (colb + j8 + j >= P.N) continue;
                  double val;
                  if (ea == EXP_NONFINITE || ebj[j] == EXP_NONFINITE)
                    val = __longlong_as_double(0x7FF8000000000000ll);
                  else
                    val = scale_pow2(tv[j8 + j], ea + ebj[j]);
                  crow[(j8 + j) * P.ldc] = (beta == 0.0) ? alpha * val : fma(alpha, val, beta * c0[j]);
                }
              }
            }
          }
          tc_fence_before();
          mbar_arrive(&tempty[buf]);
          if (++buf == 2) { buf = 0; acc_phase ^= 1; }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem_base, TC_TMEM_COLS);
  }
}

static std::atomic<int> g_tc_engine{0};
int tc_engine_setting() { return g_tc_engine.load(std::memory_order_relaxed); }
void tc_set_engine(int e) { g_tc_engine.store(e); }

int tc_gemm_launch(int epi, const CUtensorMap& ta0, const CUtensorMap& tb0, const CUtensorMap* ta1,
                   const CUtensorMap* tb1, const SliceSchedule& sched, const TcParams& prm, int grid,
                   int kernel_kind, cudaStream_t s) {
  static std::atomic<unsigned long long> smem_opt_in[2];   // per kernel, one bit per device
  const CUtensorMap& a1 = ta1 ? *ta1 : ta0;
  const CUtensorMap& b1 = tb1 ? *tb1 : tb0;
  if (grid < 1) return GB_OK;
  if (epi == TC_EPI_OZAKI_F64) {
    const int rc = opt_in_dynamic_smem(tc_gemm_kernel<TC_EPI_OZAKI_F64>, TC_SMEM_BYTES, smem_opt_in[0]);
    if (rc) return rc;
    GB_LAUNCH(kernel_kind, s,
              (tc_gemm_kernel<TC_EPI_OZAKI_F64><<<grid, TC_THREADS, TC_SMEM_BYTES, s>>>(ta0, tb0, a1, b1, sched, prm)));
  } else {
    const int rc = opt_in_dynamic_smem(tc_gemm_kernel<TC_EPI_F32>, TC_SMEM_BYTES, smem_opt_in[1]);
    if (rc) return rc;
    GB_LAUNCH(kernel_kind, s,
              (tc_gemm_kernel<TC_EPI_F32><<<grid, TC_THREADS, TC_SMEM_BYTES, s>>>(ta0, tb0, a1, b1, sched, prm)));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
